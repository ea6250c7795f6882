// decompose.cu -- the per-edge graphlet decomposition kernel.
//
// Replaces the OpenMP edge loop of graphlet_decomposition[_micro]
// (graphlet_core.cpp:1408-1424 and :1549-1577) and its helpers
// mark_neighbors / triangles_and_wedges / cycle / clique (:1069-1240),
// solve_graphlet_equations (:1326-1364) and the serial thread-sum reduction
// (:1431-1448).
//
// Per edge e = (v, u) the reference marks N(v), splits N(u)\{v} into the
// triangle set T = N(u) n N(v) and the star set S_u, then counts
//   c4(e) = #edges between S_u and S_v   (induced 4-cycles through e)
//   k4(e) = #edges inside T              (4-cliques through e)
// by scanning N(w) for every w in S_u u T.  Both counts are symmetric in
// (u, v), so this kernel scans the endpoint q whose 2-hop volume
// sum_{w in N(q)} d_w is smaller and tests membership in the other
// endpoint p.  Rows of the compute CSR are sorted, so membership is a
// binary search; N(p) with its labels (S_p / T / q) is staged in shared
// memory when it fits.  The 2-hop scan is flattened over the warp (one
// item per lane, owner found by a 5-step search over the warp's prefix sums)
// so short and long lists keep all 32 lanes busy; a neighbour w whose list
// is much longer than N(p) is handled the other way round (binary search of
// N(p)'s entries in N(w)).
//
// All per-edge arithmetic is integer; the reference's "/ 2.0" round trips
// are reproduced with explicitly rounded double intrinsics.  Partial sums
// are uint64 and wrap exactly like the reference's (addition mod 2^64 is
// order independent, so the block reduction order does not matter).
#include "pgd_internal.h"
#include "pgd_kernels.cuh"

namespace {

constexpr int kWarps = 8;          // warps per block
constexpr int kStage = 1024;       // N(p) entries staged per warp

struct DecompArgs {
    const int64_t *off;
    const int32_t *adj;
    const int32_t *deg;
    const uint64_t *vol2;
    const int32_t *ev;
    const int32_t *eu;
    const int32_t *order;
    int64_t m_edges;
    long long n, m;
    uint64_t *micro;
    unsigned long long *sums;
    unsigned long long *next;
};

__global__ void __launch_bounds__(kWarps * 32)
k_decompose(DecompArgs a) {
    __shared__ int32_t s_np[kWarps][kStage];
    __shared__ uint8_t s_lab[kWarps][kStage];
    __shared__ unsigned long long s_red[kWarps][PGD_NSUMS];

    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    int32_t *np_s = s_np[wid];
    uint8_t *lab_s = s_lab[wid];

    unsigned long long acc[PGD_NSUMS];
#pragma unroll
    for (int i = 0; i < PGD_NSUMS; i++) acc[i] = 0;

    while (true) {
        unsigned long long e = 0;
        if (lane == 0) e = atomicAdd(a.next, 1ull);
        e = __shfl_sync(0xffffffffu, e, 0);
        if (e >= (unsigned long long)a.m_edges) break;

        const int32_t id = a.order[e];
        const int32_t v = a.ev[id], u = a.eu[id];
        const long long dv = a.deg[v], du = a.deg[u];
        // scan side q: the smaller 2-hop volume; marked side p
        int32_t p = v, q = u;
        if (a.vol2[v] < a.vol2[u]) { p = u; q = v; }
        const int dp = a.deg[p], dq = a.deg[q];
        const int32_t *Np = a.adj + a.off[p];
        const int32_t *Nq = a.adj + a.off[q];
        const bool staged = dp <= kStage;

        // ---- T and labels of N(p) -------------------------------------
        unsigned long long t = 0;
        if (staged) {
            for (int i = lane; i < dp; i += 32) {
                int32_t y = __ldg(Np + i);
                np_s[i] = y;
                uint8_t lab;
                if (y == q) lab = 0;
                else lab = pgd_contains(Nq, dq, y) ? 3 : 1;
                lab_s[i] = lab;
                t += (lab == 3);
            }
            __syncwarp();
        } else {
            for (int i = lane; i < dq; i += 32) {
                int32_t x = __ldg(Nq + i);
                t += (x != p && pgd_contains(Np, dp, x)) ? 1 : 0;
            }
        }
        t = pgd_warp_sum(t);

        // label of a vertex x relative to this edge: 0 none, 1 in S_p, 3 in T
        auto label_of = [&](int32_t x) -> int {
            if (staged) {
                int pos = pgd_lower_bound(np_s, dp, x);
                return (pos < dp && np_s[pos] == x) ? lab_s[pos] : 0;
            }
            if (x == q || !pgd_contains(Np, dp, x)) return 0;
            return pgd_contains(Nq, dq, x) ? 3 : 1;
        };
        const int32_t *Nlist = staged ? np_s : Np;
        const int logp = 32 - __clz(dp | 1);

        // ---- 2-hop scan over w in N(q)\{p} -------------------------------
        unsigned long long c4 = 0, k4x2 = 0;
        for (int base = 0; base < dq; base += 32) {
            const int j = base + lane;
            int32_t w = -1;
            int cls = 0;       // 1: w in S_q, 3: w in T
            int64_t offw = 0;
            int dw = 0;
            bool rev = false;
            if (j < dq) {
                w = __ldg(Nq + j);
                if (w != p) {
                    cls = pgd_contains(Nlist, dp, w) ? 3 : 1;
                    offw = a.off[w];
                    dw = a.deg[w];
                    const int logw = 32 - __clz(dw | 1);
                    // forward cost dw*log(dp) vs reverse dp*log(dw)
                    rev = (long long)dw * logp > 4LL * dp * logw && dw > 64;
                }
            }
            int len = (cls && !rev) ? dw : 0;
            int incl = pgd_warp_incl_scan(len);
            int total = __shfl_sync(0xffffffffu, incl, 31);
            int excl = incl - len;
            for (int b2 = 0; b2 < total; b2 += 32) {
                const int it = b2 + lane;
                // owner: first lane whose inclusive prefix exceeds it
                int lo = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    int cand = lo + step - 1;
                    int pre = __shfl_sync(0xffffffffu, incl, cand);
                    if (pre <= it) lo += step;
                }
                const int owner = lo;
                const int64_t o_off = __shfl_sync(0xffffffffu, offw, owner);
                const int o_cls = __shfl_sync(0xffffffffu, cls, owner);
                const int o_excl = __shfl_sync(0xffffffffu, excl, owner);
                if (it < total) {
                    int32_t x = __ldg(a.adj + o_off + (it - o_excl));
                    int lab = label_of(x);
                    c4 += (o_cls == 1 && lab == 1);
                    k4x2 += (o_cls == 3 && lab == 3);
                }
            }
            // hub neighbours: search N(p)'s labelled entries in N(w)
            unsigned revmask = __ballot_sync(0xffffffffu, rev);
            while (revmask) {
                const int src = __ffs(revmask) - 1;
                revmask &= revmask - 1;
                const int64_t w_off = __shfl_sync(0xffffffffu, offw, src);
                const int w_deg = __shfl_sync(0xffffffffu, dw, src);
                const int w_cls = __shfl_sync(0xffffffffu, cls, src);
                const int32_t *Nw = a.adj + w_off;
                for (int i = lane; i < dp; i += 32) {
                    int32_t y = staged ? np_s[i] : __ldg(Np + i);
                    int lab = staged ? lab_s[i] : label_of(y);
                    if (lab == w_cls && pgd_contains(Nw, w_deg, y)) {
                        if (w_cls == 1) c4++;
                        else k4x2++;
                    }
                }
            }
        }
        c4 = pgd_warp_sum(c4);
        k4x2 = pgd_warp_sum(k4x2);
        const unsigned long long k4 = k4x2 >> 1;

        if (lane == 0) {
            pgd_edge_sums(acc, dv, du, t, a.m, a.n);
            acc[3] += k4;
            acc[4] += c4;
        }
        if (a.micro && lane < PGD_NMICRO) {
            a.micro[e * PGD_NMICRO + lane] = pgd_micro_col(lane, dv, du, t, k4, c4);
        }
        __syncwarp();
    }

    // block reduction of the partial sums, then one atomic per sum
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < PGD_NSUMS; i++) s_red[wid][i] = acc[i];
    }
    __syncthreads();
    if (threadIdx.x < PGD_NSUMS) {
        unsigned long long s = 0;
        for (int w = 0; w < kWarps; w++) s += s_red[w][threadIdx.x];
        atomicAdd(a.sums + threadIdx.x, s);
    }
}

}  // namespace

pgd_status pgd_dev_decompose(pgd_graph *g, bool micro, pgd_counts *out) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    if (micro && !g->micro) {
        if ((st = pgd_graph_alloc(g, (void **)&g->micro, (g->m + 1) * PGD_NMICRO * sizeof(uint64_t)))) return st;
    }
    PGD_CUDA(ctx, cudaMemsetAsync(ctx->d_sums, 0, PGD_NSUMS * sizeof(unsigned long long), s));
    PGD_CUDA(ctx, cudaMemsetAsync(ctx->d_ctr, 0, sizeof(unsigned long long), s));
    DecompArgs a;
    a.off = g->off;
    a.adj = g->adj;
    a.deg = g->deg;
    a.vol2 = g->vol2;
    a.ev = g->ev;
    a.eu = g->eu;
    a.order = g->order;
    a.m_edges = g->m;
    a.n = g->n;
    a.m = g->m;
    a.micro = micro ? g->micro : nullptr;
    a.sums = ctx->d_sums;
    a.next = ctx->d_ctr;
    int blocks = ctx->num_sms * 6;
    PGD_CUDA(ctx, cudaEventRecord(ctx->ev0, s));
    if (g->m > 0) PGD_LAUNCH(ctx, k_decompose, blocks, kWarps * 32, 0, a);
    PGD_CUDA(ctx, cudaEventRecord(ctx->ev1, s));
    PGD_CUDA(ctx, cudaGetLastError());
    unsigned long long h[PGD_NSUMS];
    PGD_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_sums, sizeof(h), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    float ms = 0;
    PGD_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    for (int i = 0; i < PGD_NSUMS; i++) out->sums[i] = h[i];
    out->n = g->n;
    out->m = g->m;
    out->kernel_ms = ms;
    pgd_close_counts(out->sums, g->n, g->m, out->totals);
    g->has_micro = micro;
    return PGD_OK;
}
