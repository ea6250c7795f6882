// pgd_internal.h -- state behind the C ABI (include/pgd_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "pgd_gb300.h"

struct pgd_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint64_t budget = 0;     // bytes graphs of this context may hold
    uint64_t resident = 0;   // bytes currently held
    std::string err;
    // decomposition scratch: per-launch counters and sums
    unsigned long long *d_sums = nullptr;   // PGD_NSUMS
    unsigned long long *d_ctr = nullptr;    // work counters
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // stage events of a decomposition: triangle pass [evt0, evt1), k_hub [evh0, evh1)
    cudaEvent_t evt0 = nullptr, evt1 = nullptr, evh0 = nullptr, evh1 = nullptr;
    unsigned long long launches = 0;        // kernels of this library launched
    // decomposition thresholds (results never depend on them; pgd_autotune sets them)
    int anchor_hub = 64;     // anchors of degree >= this take the bitmap (block) path
    int cache_hub = 32;      // W(w,p) taken from the per-anchor histogram for neighbours of degree >= this
    int dense_max = 2048;    // batched graphs with at most this many vertices use row bitsets
    int tc_min_deg = 64;     // batched CN-graph runs with d_q >= this count k4 on the tensor cores (0: never)
    bool thresholds_set = false;   // anchor_hub / cache_hub chosen by the caller or pgd_autotune
};

struct pgd_graph {
    pgd_ctx *ctx = nullptr;
    int64_t n = 0, m = 0;
    int32_t max_degree = 0;
    int64_t self_loops = 0, duplicates = 0;
    uint64_t bytes = 0;               // device bytes held

    // compute CSR: rows sorted by neighbour id
    int64_t *off = nullptr;           // n+1
    int32_t *adj = nullptr;           // 2m
    int32_t *deg = nullptr;           // n
    int64_t *rank = nullptr;          // 2m insertion rank of each entry
    uint64_t *vol2 = nullptr;         // n: sum of neighbour degrees

    // preprocess: edge arrays by edge id (graphlet_core.cpp:929-949)
    bool preprocessed = false;
    int32_t *ev = nullptr, *eu = nullptr;   // m

    // cores (0-based core numbers)
    bool has_cores = false;
    int32_t *core = nullptr;          // n
    int32_t max_core = 0;

    // E_ordered edge ids
    bool sorted = false;
    int32_t *order = nullptr;         // m entries allocated
    int64_t norder = 0;               // E_ordered length: m, or the sample size

    // per-edge results in E_ordered order
    bool has_micro = false;
    uint64_t *micro = nullptr;        // m * 8

    // decomposition structures, built on first use (decompose.cu)
    bool has_aux = false;
    int64_t *offp = nullptr;          // n+1: degree-oriented lists N+(x)
    int32_t *adjp = nullptr;          // m: neighbours of higher (degree, id)
    int32_t *hubid = nullptr;         // n: slot in the W histogram, -1 if none
    int32_t nhubs = 0;
    int32_t nhubs_wide = 0;           // hub ids below this have wide (16/32-bit) counters, the rest 8-bit
    int32_t aux_cache_hub = 0;        // threshold the hub ids were built with
    int64_t *offh = nullptr;          // n+1: hub-neighbour lists
    int32_t *adjh = nullptr;          // nadjh: hub ids of each vertex's hub neighbours
    int64_t nadjh = 0;
    uint32_t *toprows = nullptr;      // rank-bitmap rows of N+(x) for the top_r highest-ranked x
    int32_t *adj_rank = nullptr;      // 2m: vrank of each adjacency entry
    void *vrec = nullptr;             // n * 32 B: per-vertex record for the scans (decompose.cu)
    int32_t top_r = 0;
    int64_t top_words = 0;
    int32_t *vrank = nullptr;         // n: rank by (degree desc, id)
    int32_t *adjp_rank = nullptr;     // m: vrank of each adjp entry
    void *slot = nullptr;             // 2m * 16 B: per adjacency slot {w, vrank(w) | row flag, hubid(w), t}
};

// Launch one of this library's kernels on the context's stream and count it.
#define PGD_LAUNCH(ctx, kernel, grid, block, smem, ...)                            \
    do {                                                                           \
        kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);           \
        (ctx)->launches++;                                                         \
    } while (0)

// Error helpers: set ctx->err and return a status.
pgd_status pgd_fail(pgd_ctx *ctx, pgd_status s, const std::string &msg);
pgd_status pgd_cuda_fail(pgd_ctx *ctx, cudaError_t e, const char *what);

#define PGD_CUDA(ctx, call)                                          \
    do {                                                             \
        cudaError_t e__ = (call);                                    \
        if (e__ != cudaSuccess) return pgd_cuda_fail((ctx), e__, #call); \
    } while (0)

// Device memory owned by a graph (counted against the context budget).
pgd_status pgd_graph_alloc(pgd_graph *g, void **p, size_t bytes);
void pgd_graph_free(pgd_graph *g, void *p, size_t bytes);

// Stream-ordered temporaries (not counted against the budget).
pgd_status pgd_tmp_alloc(pgd_ctx *ctx, void **p, size_t bytes);
void pgd_tmp_free(pgd_ctx *ctx, void *p);

// Device stages (graph_build.cu).
pgd_status pgd_build_from_pairs(pgd_graph *g, const int32_t *h_src, const int32_t *h_dst, int64_t k,
                                int64_t n_min, bool dedup);
pgd_status pgd_build_from_device_pairs(pgd_graph *g, const int32_t *d_src, const int32_t *d_dst, int64_t k,
                                       int64_t n_min, bool dedup);
pgd_status pgd_build_from_csr(pgd_graph *g, const int64_t *h_off, const int32_t *h_adj, int64_t n);
// ingest.cu: a graph file parsed on the device with the reference reader's rules
pgd_status pgd_build_from_file(pgd_graph *g, const char *path, bool *mtx);
pgd_status pgd_dev_preprocess(pgd_graph *g, int neigh_kind, int s2l);
pgd_status pgd_dev_cores(pgd_graph *g);
pgd_status pgd_dev_assortativity(pgd_graph *g, double *r);
pgd_status pgd_dev_sort_edges(pgd_graph *g, int order_kind, int s2l);
pgd_status pgd_dev_sort_edges_sample(pgd_graph *g, int order_kind, int s2l, const int64_t *h_ids, int64_t k);
pgd_status pgd_dev_micro_out(pgd_graph *g, uint64_t *cols, int64_t *src1, int64_t *dst1);
// host memory the device can address directly (page-locked, mapped): its device address, else null
void *pgd_device_view(const void *host);
// host -> device copy on the context's stream: a kernel through the mapping when
// the source is page-locked host memory (every SM's bandwidth over the host
// link), else cudaMemcpyAsync
cudaError_t pgd_h2d(pgd_ctx *ctx, void *dst, const void *src, size_t bytes);
pgd_status pgd_dev_micro_ids(pgd_graph *g, int64_t *d_src1, int64_t *d_dst1);

// Decomposition (decompose.cu).
pgd_status pgd_dev_decompose(pgd_graph *g, bool micro, pgd_counts *out);
pgd_status pgd_dev_decompose_batch(pgd_ctx *ctx, pgd_graph *const *graphs, int k, bool micro, pgd_counts *out);
pgd_status pgd_dev_decompose_pairs_batch(pgd_ctx *ctx, int k, const int64_t *pair_off, const int32_t *src,
                                         const int32_t *dst, const int64_t *n_min, pgd_counts *out);

// Order kinds shared by host parsing and device keys.
enum pgd_order_kind {
    PGD_ORD_NATURAL = 0,
    PGD_ORD_DEG = 2,
    PGD_ORD_KCORE = 3,
    PGD_ORD_KCORE_DEG = 4,
    PGD_ORD_DEG_VOL = 5,
    PGD_ORD_KCORE_VOL = 6,
    PGD_ORD_KCORE_DEG_VOL = 7,
    PGD_ORD_DEG_U = 99,     // names mapped past VAR: key = degree of e_u
};
enum pgd_neigh_kind { PGD_NEIGH_ASREAD = 0, PGD_NEIGH_DEG = 1, PGD_NEIGH_KCORE = 2 };
