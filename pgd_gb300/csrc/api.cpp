// api.cpp -- the C ABI entry points (include/pgd_gb300.h): context and graph
// lifetime, option parsing, host<->device copies of results.  Compute is in
// graph_build.cu and decompose.cu; nothing here computes counts on the CPU.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "pgd_internal.h"

// ---------------------------------------------------------------------------
// errors and memory

pgd_status pgd_fail(pgd_ctx *ctx, pgd_status s, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return s;
}

pgd_status pgd_cuda_fail(pgd_ctx *ctx, cudaError_t e, const char *what) {
    std::string msg = std::string("CUDA error ") + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ") in " + what;
    if (e == cudaErrorMemoryAllocation) return pgd_fail(ctx, PGD_ENOMEM, msg);
    return pgd_fail(ctx, PGD_ECUDA, msg);
}

pgd_status pgd_graph_alloc(pgd_graph *g, void **p, size_t bytes) {
    pgd_ctx *ctx = g->ctx;
    if (ctx->resident + bytes > ctx->budget)
        return pgd_fail(ctx, PGD_ENOMEM, "HBM budget of the context exceeded (" + std::to_string(ctx->resident + bytes) +
                                             " > " + std::to_string(ctx->budget) + " bytes)");
    cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 16, ctx->stream);
    if (e != cudaSuccess) { cudaGetLastError(); return pgd_cuda_fail(ctx, e, "cudaMallocAsync"); }
    ctx->resident += bytes;
    g->bytes += bytes;
    return PGD_OK;
}

void pgd_graph_free(pgd_graph *g, void *p, size_t bytes) {
    if (!p) return;
    cudaFreeAsync(p, g->ctx->stream);
    g->ctx->resident -= bytes;
    g->bytes -= bytes;
}

pgd_status pgd_tmp_alloc(pgd_ctx *ctx, void **p, size_t bytes) {
    cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 16, ctx->stream);
    if (e != cudaSuccess) { cudaGetLastError(); return pgd_cuda_fail(ctx, e, "cudaMallocAsync (temporary)"); }
    return PGD_OK;
}

void pgd_tmp_free(pgd_ctx *ctx, void *p) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

// Copies on the context's stream and waits for it: the stream is created
// non-blocking, so a legacy-stream cudaMemcpy would not wait for its kernels.
static cudaError_t pgd_copy_sync(pgd_ctx *ctx, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(ctx->stream);
}

// ---------------------------------------------------------------------------
// context

extern "C" const char *pgd_status_string(pgd_status s) {
    switch (s) {
    case PGD_OK: return "ok";
    case PGD_EINVAL: return "invalid argument or input";
    case PGD_ENOMEM: return "out of memory or over budget";
    case PGD_ETIMEOUT: return "bounded device wait timed out";
    case PGD_ECUDA: return "CUDA error";
    case PGD_EIO: return "I/O error";
    case PGD_EUNSUPPORTED: return "unsupported option";
    }
    return "unknown status";
}

extern "C" pgd_status pgd_context_create(const pgd_opts *opts, pgd_ctx **out) {
    if (!out) return PGD_EINVAL;
    *out = nullptr;
    pgd_opts o;
    memset(&o, 0, sizeof(o));
    if (opts) o = *opts;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) { cudaGetLastError(); return PGD_ECUDA; }
    if (o.device < 0 || o.device >= count) return PGD_EINVAL;
    if (cudaSetDevice(o.device) != cudaSuccess) return PGD_ECUDA;
    pgd_ctx *ctx = new pgd_ctx();
    ctx->device = o.device;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, o.device) != cudaSuccess) { delete ctx; return PGD_ECUDA; }
    ctx->num_sms = prop.multiProcessorCount;
    if (o.stream) {
        ctx->stream = (cudaStream_t)o.stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return PGD_ECUDA; }
        ctx->own_stream = true;
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    ctx->budget = o.hbm_budget ? o.hbm_budget : (uint64_t)(0.9 * (double)free_b);
    // keep freed pool memory cached: graph builds reuse it
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, o.device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if (cudaMalloc((void **)&ctx->d_sums, 64 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc((void **)&ctx->d_ctr, 64 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
        cudaEventCreate(&ctx->evt0) != cudaSuccess || cudaEventCreate(&ctx->evt1) != cudaSuccess ||
        cudaEventCreate(&ctx->evh0) != cudaSuccess || cudaEventCreate(&ctx->evh1) != cudaSuccess) {
        cudaGetLastError();
        pgd_context_destroy(ctx);
        return PGD_ECUDA;
    }
    *out = ctx;
    return PGD_OK;
}

extern "C" pgd_status pgd_context_destroy(pgd_ctx *ctx) {
    if (!ctx) return PGD_EINVAL;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->d_sums) cudaFree(ctx->d_sums);
    if (ctx->d_ctr) cudaFree(ctx->d_ctr);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (cudaEvent_t e : {ctx->evt0, ctx->evt1, ctx->evh0, ctx->evh1})
        if (e) cudaEventDestroy(e);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PGD_OK;
}

extern "C" const char *pgd_last_error(const pgd_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

extern "C" uint64_t pgd_context_resident_bytes(const pgd_ctx *ctx) { return ctx ? ctx->resident : 0; }

extern "C" uint64_t pgd_context_kernel_launches(const pgd_ctx *ctx) { return ctx ? ctx->launches : 0; }

// ---------------------------------------------------------------------------
// graphs

static pgd_graph *new_graph(pgd_ctx *ctx) {
    pgd_graph *g = new pgd_graph();
    g->ctx = ctx;
    return g;
}

extern "C" pgd_status pgd_graph_destroy(pgd_graph *g) {
    if (!g) return PGD_EINVAL;
    cudaSetDevice(g->ctx->device);
    pgd_graph_free(g, g->off, (g->n + 1) * sizeof(int64_t));
    pgd_graph_free(g, g->adj, (2 * g->m + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->rank, (2 * g->m + 1) * sizeof(int64_t));
    pgd_graph_free(g, g->deg, (g->n + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->vol2, (g->n + 1) * sizeof(uint64_t));
    pgd_graph_free(g, g->ev, (g->m + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->eu, (g->m + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->core, (g->n + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->order, (g->m + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->micro, (g->m + 1) * PGD_NMICRO * sizeof(uint64_t));
    pgd_graph_free(g, g->offp, (g->n + 1) * sizeof(int64_t));
    pgd_graph_free(g, g->adjp, (g->m + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->hubid, (g->n + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->vrank, (g->n + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->adjp_rank, (g->m + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->slot, (2 * g->m + 1) * 16);
    pgd_graph_free(g, g->offh, (g->n + 1) * sizeof(int64_t));
    pgd_graph_free(g, g->adjh, (g->nadjh + 1) * sizeof(int32_t));
    pgd_graph_free(g, g->toprows, (g->top_words + 1) * sizeof(uint32_t));
    pgd_graph_free(g, g->vrec, (g->n + 1) * 32);
    pgd_graph_free(g, g->adj_rank, (2 * g->m + 1) * sizeof(int32_t));
    // whatever is left (partial builds) is returned to the budget as well
    g->ctx->resident -= g->bytes;
    cudaStreamSynchronize(g->ctx->stream);
    delete g;
    return PGD_OK;
}

static pgd_status finish_new(pgd_graph *g, pgd_status st, pgd_graph **out) {
    if (st != PGD_OK) {
        pgd_graph_destroy(g);
        return st;
    }
    *out = g;
    return PGD_OK;
}

extern "C" pgd_status pgd_graph_from_edges(pgd_ctx *ctx, const int32_t *src, const int32_t *dst, int64_t k,
                                           int64_t n_min, uint32_t flags, pgd_graph **out) {
    if (!ctx || !out || k < 0 || (k > 0 && (!src || !dst)) || n_min < 0) return pgd_fail(ctx, PGD_EINVAL, "bad arguments");
    cudaSetDevice(ctx->device);
    pgd_graph *g = new_graph(ctx);
    return finish_new(g, pgd_build_from_pairs(g, src, dst, k, n_min, (flags & PGD_EDGES_DEDUP) != 0), out);
}

extern "C" pgd_status pgd_graph_from_csr(pgd_ctx *ctx, const int64_t *off, const int32_t *adj, int64_t n,
                                         pgd_graph **out) {
    if (!ctx || !out || !off || n < 0 || (off[n] > 0 && !adj)) return pgd_fail(ctx, PGD_EINVAL, "bad arguments");
    cudaSetDevice(ctx->device);
    pgd_graph *g = new_graph(ctx);
    return finish_new(g, pgd_build_from_csr(g, off, adj, n), out);
}

extern "C" pgd_status pgd_graph_from_file(pgd_ctx *ctx, const char *path, pgd_graph **out) {
    if (!ctx || !out || !path) return pgd_fail(ctx, PGD_EINVAL, "bad arguments");
    cudaSetDevice(ctx->device);
    pgd_graph *g = new_graph(ctx);
    bool mtx = false;
    pgd_status st = pgd_build_from_file(g, path, &mtx);
    if (st == PGD_EINVAL && mtx && ctx->err.find("repeated pair") != std::string::npos)
        ctx->err = "mtx file lists an edge twice; the reference does not deduplicate mtx input and its counts "
                   "are undefined for multigraphs";
    return finish_new(g, st, out);
}

extern "C" pgd_status pgd_graph_info(const pgd_graph *g, pgd_info *info) {
    if (!g || !info) return PGD_EINVAL;
    info->n = g->n;
    info->m = g->m;
    info->max_degree = g->max_degree;
    info->avg_degree = g->n ? (int32_t)((double)(2 * g->m) / (double)g->n) : 0;
    info->self_loops = g->self_loops;
    info->duplicates = g->duplicates;
    return PGD_OK;
}

extern "C" uint64_t pgd_graph_resident_bytes(const pgd_graph *g) { return g ? g->bytes : 0; }

// ---------------------------------------------------------------------------
// ordering

static int parse_neigh(const char *s) {
    std::string o = s ? s : "";
    if (o == "degree" || o == "deg") return PGD_NEIGH_DEG;
    if (o == "kcore") return PGD_NEIGH_KCORE;
    static const char *unsupported[] = {"rand", "degree_kcore", "deg_kcore", "degree_vol", "deg_vol",
                                        "kcore_vol", "degree_kcore_vol", "deg_kcore_vol"};
    for (const char *u : unsupported)
        if (o == u) return -1;
    return PGD_NEIGH_ASREAD;
}

static int parse_order(const char *s) {
    std::string o = s ? s : "";
    if (o == "natural") return PGD_ORD_NATURAL;
    if (o == "deg" || o == "degree") return PGD_ORD_DEG;
    if (o == "kcore" || o == "kcores") return PGD_ORD_KCORE;
    if (o == "kcore_deg" || o == "kcore_degree") return PGD_ORD_KCORE_DEG;
    if (o == "deg_vol" || o == "degree_vol") return PGD_ORD_DEG_VOL;
    if (o == "kcore_vol" || o == "kcore_volume") return PGD_ORD_KCORE_VOL;
    if (o == "kcore_deg_vol" || o == "kcore_degree_vol") return PGD_ORD_KCORE_DEG_VOL;
    if (o == "rand" || o == "random" || o == "var") return -1;
    // names the reference maps to enum values past VAR use the default
    // branch of get_ordering_value (graphlet_core.cpp:829-832)
    static const char *deg_u[] = {
        "triangles", "tri", "triangle", "wedges", "tcores", "triangle_cores", "triangle_core", "tcore", "coloring",
        "greedy_coloring", "tri_vol", "triangle_vol", "tcore_vol", "tcore_volume", "triangle_core_vol",
        "triangles_only", "triangle_only", "dynamic_largest_first", "lfo", "LFO", "triangle_core_max", "tcore_max",
        "tcores_max", "degree_triangles", "degree_tri", "deg_tri", "deg_triangles", "kcore_tri", "kcore_triangles",
        "kcore_triangle", "kcore_deg_tri", "kcore_degree_triangle", "kcore_degree_tri", "kcore_tri_vol",
        "kcore_triangle_vol", "kcore_deg_tri_vol", "kcore_degree_tri_vol", "dist_two_lfo", "dist_two_largest_first",
        "dist_two_dlfo", "dist_two_dynamic_lfo", "dist_two_slo", "dist_two_smallest_last", "ido", "incidence",
        "incidence_deg", "dist_two_ido", "dist_two_incidence", "dist_two_tcore", "dist_two_triangle_core",
        "tcore_min", "triangle_core_min", "tri_core_min", "common", "common_neighbors"};
    for (const char *d : deg_u)
        if (o == d) return PGD_ORD_DEG_U;
    return PGD_ORD_NATURAL;
}

extern "C" pgd_status pgd_compute_cores(pgd_graph *g, int32_t *max_core) {
    if (!g) return PGD_EINVAL;
    cudaSetDevice(g->ctx->device);
    if (!g->has_cores) {
        pgd_status st = pgd_dev_cores(g);
        if (st) return st;
    }
    if (max_core) *max_core = g->max_core;
    return PGD_OK;
}

extern "C" pgd_status pgd_get_kcore(pgd_graph *g, int32_t *kcore) {
    if (!g || !kcore) return PGD_EINVAL;
    pgd_status st = pgd_compute_cores(g, nullptr);
    if (st) return st;
    kcore[0] = 0;
    if (g->n) PGD_CUDA(g->ctx, pgd_copy_sync(g->ctx, kcore + 1, g->core, g->n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    return PGD_OK;
}

extern "C" pgd_status pgd_preprocess(pgd_graph *g, const char *neigh_order, int small_to_large) {
    if (!g) return PGD_EINVAL;
    cudaSetDevice(g->ctx->device);
    int kind = parse_neigh(neigh_order);
    if (kind < 0)
        return pgd_fail(g->ctx, PGD_EUNSUPPORTED,
                        std::string("neighbour ordering '") + (neigh_order ? neigh_order : "") +
                            "' is not deterministic or not well defined in the reference");
    if (kind == PGD_NEIGH_KCORE && !g->has_cores) {
        pgd_status st = pgd_dev_cores(g);
        if (st) return st;
    }
    return pgd_dev_preprocess(g, kind, small_to_large);
}

extern "C" pgd_status pgd_assortativity(pgd_graph *g, double *r) {
    if (!g || !r) return PGD_EINVAL;
    cudaSetDevice(g->ctx->device);
    if (!g->preprocessed) {
        pgd_status st = pgd_preprocess(g, "deg", 0);
        if (st) return st;
    }
    return pgd_dev_assortativity(g, r);
}

extern "C" pgd_status pgd_sort_edges(pgd_graph *g, const char *order, int small_to_large) {
    if (!g) return PGD_EINVAL;
    cudaSetDevice(g->ctx->device);
    int kind = parse_order(order);
    if (kind < 0)
        return pgd_fail(g->ctx, PGD_EUNSUPPORTED,
                        std::string("edge ordering '") + (order ? order : "") +
                            "' is wall-clock seeded or divides by zero in the reference");
    pgd_status st;
    if (!g->preprocessed && (st = pgd_preprocess(g, "deg", 0))) return st;
    bool need_cores = kind == PGD_ORD_KCORE || kind == PGD_ORD_KCORE_DEG || kind == PGD_ORD_KCORE_VOL ||
                      kind == PGD_ORD_KCORE_DEG_VOL;
    if (need_cores && !g->has_cores && (st = pgd_dev_cores(g))) return st;
    return pgd_dev_sort_edges(g, kind, small_to_large);
}

extern "C" pgd_status pgd_sort_edges_sample(pgd_graph *g, const char *order, int small_to_large,
                                            const int64_t *edge_ids, int64_t k) {
    if (!g || k < 0 || (k > 0 && !edge_ids)) return g ? pgd_fail(g->ctx, PGD_EINVAL, "bad arguments") : PGD_EINVAL;
    cudaSetDevice(g->ctx->device);
    int kind = parse_order(order);
    if (kind < 0)
        return pgd_fail(g->ctx, PGD_EUNSUPPORTED,
                        std::string("edge ordering '") + (order ? order : "") +
                            "' is wall-clock seeded or divides by zero in the reference");
    pgd_status st;
    if (!g->preprocessed && (st = pgd_preprocess(g, "deg", 0))) return st;
    bool need_cores = kind == PGD_ORD_KCORE || kind == PGD_ORD_KCORE_DEG || kind == PGD_ORD_KCORE_VOL ||
                      kind == PGD_ORD_KCORE_DEG_VOL;
    if (need_cores && !g->has_cores && (st = pgd_dev_cores(g))) return st;
    return pgd_dev_sort_edges_sample(g, kind, small_to_large, edge_ids, k);
}

extern "C" int64_t pgd_graph_order_length(const pgd_graph *g) { return g && g->sorted ? g->norder : 0; }

// ---------------------------------------------------------------------------
// decomposition and results

extern "C" pgd_status pgd_decompose(pgd_graph *g, uint32_t flags, pgd_counts *out) {
    if (!g || !out) return PGD_EINVAL;
    cudaSetDevice(g->ctx->device);
    pgd_status st;
    memset(out, 0, sizeof(*out));
    if (!g->preprocessed && (st = pgd_preprocess(g, "deg", 0))) return st;
    if (!g->sorted && (st = pgd_sort_edges(g, "deg", 0))) return st;
    // Default thresholds by graph size (counts never depend on them): while the
    // caller has set none (directly or through pgd_autotune), graphs of more
    // than kLargeGraph vertices take hub anchors from degree 128 and cached W
    // from degree 40.  Measured on RMAT scales 21 to 24 (2.1 M to 16.8 M
    // vertices): 0.3 %, 1.2 %, 1.0 % and 5.7 % faster than the 64 / 32
    // defaults, which stay the fastest on RMAT scale 20 (1.05 M vertices).
    pgd_ctx *ctx = g->ctx;
    constexpr int64_t kLargeGraph = 3ll << 19;   // 1.5 * 2^20
    if (!ctx->thresholds_set && g->n > kLargeGraph) {
        const int a = ctx->anchor_hub, c = ctx->cache_hub;
        ctx->anchor_hub = 128;
        ctx->cache_hub = 40;
        st = pgd_dev_decompose(g, (flags & PGD_MICRO) != 0, out);
        ctx->anchor_hub = a;
        ctx->cache_hub = c;
        return st;
    }
    return pgd_dev_decompose(g, (flags & PGD_MICRO) != 0, out);
}

extern "C" pgd_status pgd_get_edges(pgd_graph *g, int64_t *ev, int64_t *eu, int32_t *order) {
    if (!g) return PGD_EINVAL;
    if (!g->preprocessed) return pgd_fail(g->ctx, PGD_EINVAL, "graph is not preprocessed");
    cudaSetDevice(g->ctx->device);
    std::vector<int32_t> tmp((size_t)g->m + 1);
    if (ev) {
        PGD_CUDA(g->ctx, pgd_copy_sync(g->ctx, tmp.data(), g->ev, g->m * sizeof(int32_t), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < g->m; i++) ev[i] = tmp[i];
    }
    if (eu) {
        PGD_CUDA(g->ctx, pgd_copy_sync(g->ctx, tmp.data(), g->eu, g->m * sizeof(int32_t), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < g->m; i++) eu[i] = tmp[i];
    }
    if (order) {
        if (!g->sorted) return pgd_fail(g->ctx, PGD_EINVAL, "edges are not sorted");
        if (g->norder)
            PGD_CUDA(g->ctx, pgd_copy_sync(g->ctx, order, g->order, g->norder * sizeof(int32_t), cudaMemcpyDeviceToHost));
    }
    return PGD_OK;
}

// The device's address of host memory it can access directly (page-locked
// and mapped, e.g. from cudaHostAlloc or cudaHostRegister), else null.
void *pgd_device_view(const void *host) {
    if (!host) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

extern "C" pgd_status pgd_get_micro(pgd_graph *g, int64_t *src1, int64_t *dst1, uint64_t *cols) {
    if (!g) return PGD_EINVAL;
    if (!g->has_micro) return pgd_fail(g->ctx, PGD_EINVAL, "no per-edge results: decompose with PGD_MICRO first");
    cudaSetDevice(g->ctx->device);
    // page-locked destinations: one kernel writes rows and ids through the
    // mapping (every SM's bandwidth over the host link; one copy engine here
    // moves about 20 GB/s)
    void *vc = pgd_device_view(cols), *vs = pgd_device_view(src1), *vd = pgd_device_view(dst1);
    const bool aligned = ((uintptr_t)vc & 15) == 0 && ((uintptr_t)vs & 7) == 0 && ((uintptr_t)vd & 7) == 0;
    if (aligned && (!cols || vc) && (!src1 || vs) && (!dst1 || vd)) {
        pgd_status st = pgd_dev_micro_out(g, (uint64_t *)vc, (int64_t *)vs, (int64_t *)vd);
        if (st) return st;
        PGD_CUDA(g->ctx, cudaStreamSynchronize(g->ctx->stream));
        return PGD_OK;
    }
    if (cols && g->norder)
        PGD_CUDA(g->ctx, pgd_copy_sync(g->ctx, cols, g->micro, g->norder * PGD_NMICRO * sizeof(uint64_t),
                                       cudaMemcpyDeviceToHost));
    if ((src1 || dst1) && g->norder) {
        // ids gathered on the device, then copied straight into the caller's arrays
        int64_t *d_ids = nullptr;
        const int64_t k = g->norder;
        pgd_status st = pgd_tmp_alloc(g->ctx, (void **)&d_ids, 2 * k * sizeof(int64_t));
        if (st) return st;
        st = pgd_dev_micro_ids(g, src1 ? d_ids : nullptr, dst1 ? d_ids + k : nullptr);
        cudaError_t e = cudaSuccess;
        if (!st && src1) e = pgd_copy_sync(g->ctx, src1, d_ids, k * sizeof(int64_t), cudaMemcpyDeviceToHost);
        if (!st && e == cudaSuccess && dst1)
            e = pgd_copy_sync(g->ctx, dst1, d_ids + k, k * sizeof(int64_t), cudaMemcpyDeviceToHost);
        pgd_tmp_free(g->ctx, d_ids);
        if (st) return st;
        if (e != cudaSuccess) return pgd_cuda_fail(g->ctx, e, "copy of the per-edge ids");
    }
    return PGD_OK;
}

extern "C" pgd_status pgd_decompose_batch(pgd_ctx *ctx, pgd_graph *const *graphs, int k, uint32_t flags,
                                          pgd_counts *out) {
    if (!ctx || k < 0 || (k > 0 && (!graphs || !out))) return pgd_fail(ctx, PGD_EINVAL, "bad arguments");
    if (k == 0) return PGD_OK;
    cudaSetDevice(ctx->device);
    pgd_status st;
    for (int i = 0; i < k; i++) {
        pgd_graph *g = graphs[i];
        if (!g || g->ctx != ctx) return pgd_fail(ctx, PGD_EINVAL, "batch graph is null or from another context");
        if (!g->preprocessed && (st = pgd_preprocess(g, "deg", 0))) return st;
        if (!g->sorted && (st = pgd_sort_edges(g, "deg", 0))) return st;
    }
    return pgd_dev_decompose_batch(ctx, graphs, k, (flags & PGD_MICRO) != 0, out);
}

extern "C" pgd_status pgd_set_thresholds(pgd_ctx *ctx, int anchor_hub, int cache_hub, int dense_max) {
    if (!ctx) return PGD_EINVAL;
    if (anchor_hub < 2 || anchor_hub > 256 || cache_hub < 2 || dense_max < 0 || dense_max > 2048)
        return pgd_fail(ctx, PGD_EINVAL,
                        "thresholds out of range (2 <= anchor_hub <= 256, cache_hub >= 2, 0 <= dense_max <= 2048)");
    ctx->anchor_hub = anchor_hub;
    ctx->cache_hub = cache_hub;
    ctx->dense_max = dense_max;
    ctx->thresholds_set = true;
    return PGD_OK;
}

extern "C" pgd_status pgd_get_thresholds(const pgd_ctx *ctx, int *anchor_hub, int *cache_hub, int *dense_max) {
    if (!ctx) return PGD_EINVAL;
    if (anchor_hub) *anchor_hub = ctx->anchor_hub;
    if (cache_hub) *cache_hub = ctx->cache_hub;
    if (dense_max) *dense_max = ctx->dense_max;
    return PGD_OK;
}

extern "C" pgd_status pgd_set_tensor_min_degree(pgd_ctx *ctx, int tensor_min_degree) {
    if (!ctx) return PGD_EINVAL;
    if (tensor_min_degree != 0 && (tensor_min_degree < 2 || tensor_min_degree > 1088))
        return pgd_fail(ctx, PGD_EINVAL, "tensor_min_degree out of range (0, or 2..1088)");
    ctx->tc_min_deg = tensor_min_degree;
    return PGD_OK;
}

extern "C" pgd_status pgd_get_tensor_min_degree(const pgd_ctx *ctx, int *tensor_min_degree) {
    if (!ctx) return PGD_EINVAL;
    if (tensor_min_degree) *tensor_min_degree = ctx->tc_min_deg;
    return PGD_OK;
}

extern "C" pgd_status pgd_autotune(pgd_ctx *ctx, pgd_graph *const *graphs, int k, int reps, int *anchor_hub,
                                   int *cache_hub, int *dense_max, float *best_ms) {
    if (!ctx || k <= 0 || !graphs) return pgd_fail(ctx, PGD_EINVAL, "bad arguments");
    if (reps < 1) reps = 1;
    std::vector<pgd_counts> out((size_t)k);
    std::vector<uint64_t> first;
    // times one candidate; every candidate must give the same counts
    auto trial = [&](float *ms) -> pgd_status {
        float total = 0;
        for (int r = 0; r < reps; r++) {
            pgd_status st = pgd_decompose_batch(ctx, graphs, k, 0, out.data());
            if (st) return st;
            total += out[0].kernel_ms;
        }
        std::vector<uint64_t> now;
        for (int i = 0; i < k; i++) now.insert(now.end(), out[(size_t)i].totals, out[(size_t)i].totals + PGD_NTOTALS);
        if (first.empty()) first = now;
        else if (first != now) return pgd_fail(ctx, PGD_EINVAL, "thresholds changed a count (internal error)");
        *ms = total / reps;
        return PGD_OK;
    };
    // 1. the bitset/list crossover for small graphs
    float best = -1, ms = 0;
    int bd = ctx->dense_max;
    for (int d : {0, 256, 1024, 2048}) {
        ctx->dense_max = d;
        pgd_status st = trial(&ms);
        if (st) return st;
        if (best < 0 || ms < best) { best = ms; bd = d; }
    }
    ctx->dense_max = bd;
    // 2. which runs of the dense graphs go to the tensor cores
    best = -1;
    int bt = ctx->tc_min_deg;
    for (int t : {0, 64, 128, 256}) {
        ctx->tc_min_deg = t;
        pgd_status st = trial(&ms);
        if (st) return st;
        if (best < 0 || ms < best) { best = ms; bt = t; }
    }
    ctx->tc_min_deg = bt;
    // 3. the two hub thresholds
    best = -1;
    int ba = ctx->anchor_hub, bc = ctx->cache_hub;
    for (int a : {32, 64, 128, 256}) {
        for (int c : {32, 64, 128, 512}) {
            ctx->anchor_hub = a;
            ctx->cache_hub = c;
            pgd_status st = trial(&ms);
            if (st) return st;
            if (best < 0 || ms < best) { best = ms; ba = a; bc = c; }
        }
    }
    ctx->anchor_hub = ba;
    ctx->cache_hub = bc;
    ctx->thresholds_set = true;
    if (anchor_hub) *anchor_hub = ba;
    if (cache_hub) *cache_hub = bc;
    if (dense_max) *dense_max = bd;
    if (best_ms) *best_ms = best;
    return PGD_OK;
}
