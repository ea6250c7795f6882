// serve.cpp -- continuous-batching request server (no reference counterpart).
//
// Requests (one graph each, as host pairs) are queued on submit.  Each
// worker thread owns a context (its own CUDA stream) and loops: take pending
// requests, oldest first, that fit the server's HBM budget (at most
// max_batch of them and about kBatchPairs pairs, so that a batch stays short
// and a request arriving meanwhile soon gets its turn), decompose them
// together -- one device CSR for the whole set, one pass of the persistent
// kernels, per-graph sums (pgd_dev_decompose_pairs_batch) -- publish the
// results, release the memory.  A request that does not fit the memory left
// is skipped for now and later, smaller requests are admitted ahead of it,
// until it has waited max_wait_ms: then nothing is admitted past it until it
// fits.  Requests arriving while a batch is on the GPU are admitted by the
// next free worker as soon as memory allows, so with two or more workers
// batches from different workers run on the device at the same time.  A
// request whose own estimate exceeds the whole budget fails with
// PGD_ENOMEM; the others are unaffected.  Latencies are kept in fixed
// log-spaced histograms (2 % resolution), split into queueing (submit to
// admission) and service (admission to result).
#include <string.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>
#include <algorithm>
#include <cmath>

#include "pgd_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    std::vector<int32_t> src, dst;
    int64_t n_min = 0;
    uint64_t est_bytes = 0;
    Clock::time_point t_submit, t_admit, t_done;
    pgd_counts result{};
    pgd_status status = PGD_OK;
    bool done = false;
};

// Device bytes one request needs while it is decomposed: pairs and their
// sort buffers, the CSR with its per-slot arrays, per-edge and per-vertex
// work arrays, and for graphs of at most 2048 vertices their adjacency
// bit rows, 16-bit common-neighbour matrix and the tensor-core path's
// per-edge arrays (run flags and positions, k4, E per slot).  Deliberately
// generous; only used for admission.
uint64_t estimate_bytes(int64_t pairs, int64_t n) {
    const uint64_t p = (uint64_t)std::max<int64_t>(pairs, 1), v = (uint64_t)std::max<int64_t>(n, 1);
    uint64_t bytes = 160 * p + 64 * v + (64u << 10);
    if (v <= 2048) bytes += 2 * v * (v + 64) + 8 * v * ((v + 63) / 64) + 24 * p;
    return bytes;
}

// A batch is closed once it holds this many pairs (it always takes at least
// one request): long batches make every request that arrives meanwhile wait.
constexpr int64_t kBatchPairs = 1 << 21;
constexpr int kDefaultMaxWaitMs = 20;

// Latency histogram with log-spaced buckets: bucket b holds values in
// [kLo * kStep^b, kLo * kStep^(b+1)) ms, from 1 microsecond to about 10^6 s.
struct LatencyHist {
    static constexpr double kLo = 1e-3, kStep = 1.02;
    static constexpr int kBuckets = 1400;
    std::vector<uint64_t> count = std::vector<uint64_t>(kBuckets, 0);
    uint64_t total = 0;
    double sum = 0;
    void add(double ms) {
        int b = ms <= kLo ? 0 : (int)(std::log(ms / kLo) / std::log(kStep));
        b = std::min(std::max(b, 0), kBuckets - 1);
        count[(size_t)b]++;
        total++;
        sum += ms;
    }
    // upper edge of the bucket holding the f-quantile
    double quantile(double f) const {
        if (!total) return 0;
        const uint64_t want = std::min<uint64_t>(total, (uint64_t)(f * (double)total) + 1);
        uint64_t seen = 0;
        for (int b = 0; b < kBuckets; b++) {
            seen += count[(size_t)b];
            if (seen >= want) return kLo * std::pow(kStep, b + 1);
        }
        return kLo * std::pow(kStep, kBuckets);
    }
};

}  // namespace

struct pgd_server {
    pgd_server_opts opts{};
    std::vector<pgd_ctx *> ctxs;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending;
    std::unordered_map<uint64_t, Request *> requests;
    uint64_t next_ticket = 1, inflight = 0, peak = 0;
    uint64_t submitted = 0, completed = 0, rejected = 0, batches = 0, skipped_ahead = 0;
    LatencyHist lat, lat_queue, lat_service;
    Clock::time_point t_first{}, t_last{};
    bool have_first = false;
    bool stop = false;

    void run(int wi) {
        pgd_ctx *ctx = ctxs[(size_t)wi];
        std::vector<Request *> batch;
        std::vector<int64_t> off, nmin;
        std::vector<int32_t> src, dst;
        std::vector<pgd_counts> out;
        while (true) {
            batch.clear();
            uint64_t bytes = 0;
            {
                std::unique_lock<std::mutex> lock(mu);
                cv_work.wait(lock, [&] { return stop || !pending.empty(); });
                if (pending.empty() && stop) return;
                // admit pending requests that fit, oldest first; skip one that
                // does not fit yet unless it has waited max_wait_ms; refuse what
                // can never fit
                const Clock::time_point now = Clock::now();
                const auto max_wait = std::chrono::milliseconds(opts.max_wait_ms);
                int64_t pairs = 0;
                bool skipped = false;
                for (auto it = pending.begin();
                     it != pending.end() && (int)batch.size() < opts.max_batch && pairs < kBatchPairs;) {
                    Request *r = *it;
                    if (r->est_bytes > opts.hbm_budget) {
                        it = pending.erase(it);
                        r->status = PGD_ENOMEM;
                        r->done = true;
                        r->t_done = now;
                        rejected++;
                        cv_done.notify_all();
                        continue;
                    }
                    if (inflight + bytes + r->est_bytes > opts.hbm_budget) {
                        if (now - r->t_submit >= max_wait) break;   // it goes next, nothing passes it
                        skipped = true;
                        ++it;
                        continue;
                    }
                    if (skipped) skipped_ahead++;
                    it = pending.erase(it);
                    bytes += r->est_bytes;
                    pairs += (int64_t)r->src.size();
                    r->t_admit = now;
                    batch.push_back(r);
                }
                if (batch.empty()) {
                    // everything left waits for memory held by other workers
                    cv_work.wait_for(lock, std::chrono::milliseconds(1));
                    continue;
                }
                inflight += bytes;
                peak = std::max(peak, inflight);
                batches++;
            }
            off.assign(1, 0);
            nmin.clear();
            src.clear();
            dst.clear();
            for (Request *r : batch) {
                src.insert(src.end(), r->src.begin(), r->src.end());
                dst.insert(dst.end(), r->dst.begin(), r->dst.end());
                off.push_back((int64_t)src.size());
                nmin.push_back(r->n_min);
            }
            out.assign(batch.size(), pgd_counts{});
            pgd_status st = pgd_dev_decompose_pairs_batch(ctx, (int)batch.size(), off.data(), src.data(), dst.data(),
                                                          nmin.data(), out.data());
            const Clock::time_point now = Clock::now();
            {
                std::lock_guard<std::mutex> lock(mu);
                for (size_t i = 0; i < batch.size(); i++) {
                    Request *r = batch[i];
                    r->status = st;
                    if (st == PGD_OK) r->result = out[i];
                    r->done = true;
                    r->t_done = now;
                    r->src.clear();
                    r->src.shrink_to_fit();
                    r->dst.clear();
                    r->dst.shrink_to_fit();
                    completed++;
                    lat.add(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
                    lat_queue.add(std::chrono::duration<double, std::milli>(r->t_admit - r->t_submit).count());
                    lat_service.add(std::chrono::duration<double, std::milli>(now - r->t_admit).count());
                }
                t_last = now;
                inflight -= bytes;
            }
            cv_done.notify_all();
            cv_work.notify_all();
        }
    }
};

extern "C" pgd_status pgd_server_create(const pgd_server_opts *opts, pgd_server **out) {
    if (!out) return PGD_EINVAL;
    *out = nullptr;
    pgd_server *sv = new pgd_server();
    if (opts) sv->opts = *opts;
    if (sv->opts.workers <= 0) sv->opts.workers = 2;
    if (sv->opts.max_batch <= 0) sv->opts.max_batch = 4096;
    if (sv->opts.max_wait_ms <= 0) sv->opts.max_wait_ms = kDefaultMaxWaitMs;
    for (int i = 0; i < sv->opts.workers; i++) {
        pgd_opts o{};
        o.device = sv->opts.device;
        pgd_ctx *c = nullptr;
        pgd_status st = pgd_context_create(&o, &c);
        if (st) {
            for (pgd_ctx *x : sv->ctxs) pgd_context_destroy(x);
            delete sv;
            return st;
        }
        sv->ctxs.push_back(c);
    }
    if (!sv->opts.hbm_budget) sv->opts.hbm_budget = sv->ctxs[0]->budget / 2;
    for (pgd_ctx *c : sv->ctxs) c->budget = UINT64_MAX;  // admission is the server's job
    for (int i = 0; i < sv->opts.workers; i++) sv->workers.emplace_back([sv, i] { sv->run(i); });
    *out = sv;
    return PGD_OK;
}

extern "C" pgd_status pgd_server_submit(pgd_server *sv, const int32_t *src, const int32_t *dst, int64_t k,
                                        int64_t n_min, uint64_t *ticket) {
    if (!sv || !ticket || k < 0 || (k > 0 && (!src || !dst)) || n_min < 0) return PGD_EINVAL;
    Request *r = new Request();
    r->src.assign(src, src + k);
    r->dst.assign(dst, dst + k);
    r->n_min = n_min;
    int64_t n = n_min;
    for (int64_t i = 0; i < k; i++) n = std::max<int64_t>(n, (int64_t)std::max(src[i], dst[i]) + 1);
    r->est_bytes = estimate_bytes(k, n);
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        if (sv->stop) {
            delete r;
            return PGD_EINVAL;
        }
        r->ticket = sv->next_ticket++;
        sv->requests[r->ticket] = r;
        sv->pending.push_back(r);
        sv->submitted++;
        if (!sv->have_first) {
            sv->t_first = r->t_submit;
            sv->have_first = true;
        }
    }
    sv->cv_work.notify_one();
    *ticket = r->ticket;
    return PGD_OK;
}

static pgd_status take_result(pgd_server *sv, std::unordered_map<uint64_t, Request *>::iterator it, pgd_counts *out) {
    Request *r = it->second;
    pgd_status st = r->status;
    if (out) *out = r->result;
    sv->requests.erase(it);
    delete r;
    return st;
}

extern "C" pgd_status pgd_server_poll(pgd_server *sv, uint64_t ticket, pgd_counts *out, int *done) {
    if (!sv || !done) return PGD_EINVAL;
    std::lock_guard<std::mutex> lock(sv->mu);
    auto it = sv->requests.find(ticket);
    if (it == sv->requests.end()) return PGD_EINVAL;
    *done = it->second->done ? 1 : 0;
    if (!*done) return PGD_OK;
    return take_result(sv, it, out);
}

extern "C" pgd_status pgd_server_wait(pgd_server *sv, uint64_t ticket, int timeout_ms, pgd_counts *out) {
    if (!sv) return PGD_EINVAL;
    std::unique_lock<std::mutex> lock(sv->mu);
    auto it = sv->requests.find(ticket);
    if (it == sv->requests.end()) return PGD_EINVAL;
    Request *r = it->second;
    if (!sv->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                              [&] { return r->done; }))
        return PGD_ETIMEOUT;
    return take_result(sv, sv->requests.find(ticket), out);
}

extern "C" pgd_status pgd_server_stats(pgd_server *sv, pgd_server_stat *st) {
    if (!sv || !st) return PGD_EINVAL;
    std::lock_guard<std::mutex> lock(sv->mu);
    memset(st, 0, sizeof(*st));
    st->submitted = sv->submitted;
    st->completed = sv->completed;
    st->rejected = sv->rejected;
    st->batches = sv->batches;
    st->inflight_bytes = sv->inflight;
    st->peak_bytes = sv->peak;
    st->skipped_ahead = sv->skipped_ahead;
    if (sv->lat.total) {
        st->p50_ms = sv->lat.quantile(0.50);
        st->p99_ms = sv->lat.quantile(0.99);
        st->mean_ms = sv->lat.sum / (double)sv->lat.total;
        st->queue_p50_ms = sv->lat_queue.quantile(0.50);
        st->queue_p99_ms = sv->lat_queue.quantile(0.99);
        st->service_p50_ms = sv->lat_service.quantile(0.50);
        st->service_p99_ms = sv->lat_service.quantile(0.99);
        const double span = std::chrono::duration<double>(sv->t_last - sv->t_first).count();
        st->graphs_per_s = span > 0 ? (double)sv->completed / span : 0;
    }
    return PGD_OK;
}

extern "C" pgd_status pgd_server_destroy(pgd_server *sv) {
    if (!sv) return PGD_EINVAL;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    for (std::thread &t : sv->workers) t.join();
    for (auto &kv : sv->requests) delete kv.second;
    for (pgd_ctx *c : sv->ctxs) pgd_context_destroy(c);
    delete sv;
    return PGD_OK;
}

extern "C" pgd_status pgd_decompose_pairs_batch(pgd_ctx *ctx, int k, const int64_t *pair_off, const int32_t *src,
                                                const int32_t *dst, const int64_t *n_min, pgd_counts *out) {
    if (!ctx || k < 0 || (k > 0 && (!pair_off || !out)) || (k > 0 && pair_off[k] > 0 && (!src || !dst)))
        return pgd_fail(ctx, PGD_EINVAL, "bad arguments");
    if (k == 0) return PGD_OK;
    cudaSetDevice(ctx->device);
    return pgd_dev_decompose_pairs_batch(ctx, k, pair_off, src, dst, n_min, out);
}
