/*
 * pgd_gb300.h -- C ABI of the GB300-native exact graphlet decomposition.
 *
 * Drop-in replacement for the hot path of PGD (nkahmed/PGD): read graph ->
 * CSR -> order -> per-edge decomposition -> 17 global counts + per-edge
 * ("micro") counts.  Every entry point below names the reference interface it
 * replaces (file:line in the reference tree).  All compute runs on one CUDA
 * device; there is no CPU fallback: when the device or the kernels are not
 * available every call returns PGD_ECUDA.
 *
 * Conventions
 *   - Plain pointers and sizes only.  Host buffers are caller-owned; device
 *     state is owned by the pgd_ctx / pgd_graph objects and released by the
 *     matching *_destroy call.
 *   - Vertex ids are 0-based int32 inside the library.  Output rows print
 *     ids + 1, as the reference's writers do.
 *   - One context per host thread.  Calls on one context are serialised on
 *     the context's stream; they are not thread-safe.
 *   - Every call returns a pgd_status; pgd_last_error() gives the message of
 *     the last failure on that context.
 */
#ifndef PGD_GB300_H
#define PGD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGD_ABI_VERSION 1

typedef enum {
    PGD_OK = 0,
    PGD_EINVAL = 1,      /* bad argument or malformed input                  */
    PGD_ENOMEM = 2,      /* device/host allocation failed or budget refused  */
    PGD_ETIMEOUT = 3,    /* a bounded device wait gave up                    */
    PGD_ECUDA = 4,       /* CUDA runtime/driver error (device missing, ...)  */
    PGD_EIO = 5,         /* file could not be read                           */
    PGD_EUNSUPPORTED = 6 /* option the reference leaves undefined (e.g. rand)*/
} pgd_status;

typedef struct pgd_ctx pgd_ctx;
typedef struct pgd_graph pgd_graph;

/* Context options.  Zero-initialise and set what you need. */
typedef struct {
    int device;            /* CUDA device ordinal                           */
    int reserved0;
    uint64_t hbm_budget;   /* bytes the context may keep resident; 0 = 90 %
                              of the device's free memory at creation        */
    void *stream;          /* cudaStream_t to run on; NULL = own stream      */
} pgd_opts;

/* Number of the raw per-edge partial sums and of the global counts. */
#define PGD_NSUMS 15
#define PGD_NTOTALS 17
#define PGD_NMICRO 8

/* Global results of one decomposition.
 * totals[] follows the field order of graphlet_core.h:310-329:
 *   0 total_2_1edge  1 total_2_indep  2 total_3_tris  3 total_2_star
 *   4 total_3_1edge  5 total_3_indep  6 total_4_clique 7 total_4_chordcycle
 *   8 total_4_tailed_tris 9 total_4_cycle 10 total_3_star 11 total_4_path
 *  12 total_4_2edge 13 total_4_1edge 14 total_4_2star 15 total_4_tri
 *  16 total_4_indep
 * sums[] are the reduced per-edge terms before the closing identities
 * (graphlet_core.cpp:1326-1364): 0 sum t, 1 sum 2-star, 2 sum 3-node-1-edge,
 * 3 sum 4-clique, 4 sum 4-cycle, 5..14 N1..N10. */
typedef struct {
    uint64_t totals[PGD_NTOTALS];
    uint64_t sums[PGD_NSUMS];
    int64_t n;              /* vertices                                     */
    int64_t m;              /* undirected edges                             */
    float kernel_ms;        /* device time of the decomposition kernels     */
    float hub_ms;           /* of which the hub-anchored kernel (k_hub)     */
    float tri_ms;           /* of which the triangle pass (t of every edge) */
    float reserved;
} pgd_counts;

/* Graph summary (graphlet_core::basic_stats, graphlet_core.cpp:562-568). */
typedef struct {
    int64_t n, m;
    int32_t max_degree;
    int32_t avg_degree;     /* (int)((double)2m / n), graphlet_core.cpp:890 */
    int64_t self_loops;     /* dropped by the reader                        */
    int64_t duplicates;     /* dropped by the dedup step                    */
} pgd_info;

/* ---- context ----------------------------------------------------------
 * No reference counterpart: replaces the OpenMP runtime set-up of
 * params::params (graphlet_params.h:285, omp_set_num_threads). */
const char *pgd_status_string(pgd_status s);
pgd_status pgd_context_create(const pgd_opts *opts, pgd_ctx **out);
pgd_status pgd_context_destroy(pgd_ctx *ctx);
const char *pgd_last_error(const pgd_ctx *ctx);
/* Bytes currently held on the device by graphs of this context. */
uint64_t pgd_context_resident_bytes(const pgd_ctx *ctx);
/* Kernels of this library launched on the context so far (no reference
 * counterpart; lets a caller check that the CUDA path did the work). */
uint64_t pgd_context_kernel_launches(const pgd_ctx *ctx);

/* ---- graph construction ----------------------------------------------- */

/* Graph from a file with the reference reader's rules (ext "mtx" -> 1-based
 * ids, no dedup, n = 1 + largest id with an edge; anything else -> generic
 * edge list: delimiter sniffing, first-seen relabel, self loops dropped,
 * duplicate edges dropped).  Replaces graphlet_core::read_graph
 * (graphlet_core.cpp:259-283, read_edge_list :291-457, read_mtx :459-522,
 * remove_multiple_edges :530-556). */
pgd_status pgd_graph_from_file(pgd_ctx *ctx, const char *path, pgd_graph **out);

#define PGD_EDGES_DEDUP 1u   /* drop repeated pairs, keep the first (edge-list rule) */

/* Graph from k undirected pairs (0-based ids) already tokenised on the host.
 * The device symmetrises, drops self loops, sorts and (with
 * PGD_EDGES_DEDUP) removes duplicates, keeping each pair's first position
 * as its insertion rank, as the reader's adjacency map does
 * (graphlet_core.cpp:410-411, 448-455).  n = max(n_min, 1 + largest id with
 * an edge).  Without PGD_EDGES_DEDUP a repeated pair is an error, since the
 * reference's marking is ill-defined on multigraphs. */
pgd_status pgd_graph_from_edges(pgd_ctx *ctx, const int32_t *src, const int32_t *dst, int64_t k,
                                int64_t n_min, uint32_t flags, pgd_graph **out);

/* Graph from a CSR (offsets n+1, adjacency off[n]); row order is taken as
 * the insertion order.  Replaces the CSR constructor
 * graphlet_core(vector<long long> vs, vector<int> es) (graphlet_core.h:156-160). */
pgd_status pgd_graph_from_csr(pgd_ctx *ctx, const int64_t *off, const int32_t *adj, int64_t n,
                              pgd_graph **out);

pgd_status pgd_graph_destroy(pgd_graph *g);
pgd_status pgd_graph_info(const pgd_graph *g, pgd_info *info);
/* Device bytes held by this graph. */
uint64_t pgd_graph_resident_bytes(const pgd_graph *g);

/* ---- ordering ---------------------------------------------------------- */

/* Neighbour ordering + edge arrays.  Replaces graphlet_core::preprocess
 * (graphlet_core.cpp:77-93: order_vertex_neighbors :1910-1953,
 * create_edge_list_arrays :929-949).  neigh_order: "deg"/"degree", "kcore",
 * or any other name for "as read"; "rand" and the *_vol/deg_kcore variants
 * return PGD_EUNSUPPORTED (wall-clock seeded / out-of-bounds in the
 * reference).  The dense-adjacency switch of optimize_graph_ops
 * (:602-611) has no counterpart: it never changes a count. */
pgd_status pgd_preprocess(pgd_graph *g, const char *neigh_order, int small_to_large);

/* k-core numbers by parallel peeling.  Replaces graphlet_core::compute_cores
 * (graphlet_core.cpp:958-1018).  *max_core is the value the reference prints
 * as "K = " (its loop at :1012-1015 leaves the last vertex out). */
pgd_status pgd_compute_cores(pgd_graph *g, int32_t *max_core);

/* Copies core numbers in the reference's 1-based layout (n+1 entries,
 * kcore[x] = core number of vertex x-1, kcore[0] = 0). */
pgd_status pgd_get_kcore(pgd_graph *g, int32_t *kcore);

/* Degree assortativity.  Replaces graphlet_core::compute_assortativity
 * (graphlet_core.cpp:1029-1057), including its int products and its
 * -ffast-math build where the isnan() guard is compiled out. */
pgd_status pgd_assortativity(pgd_graph *g, double *r);

/* Edge (job) order.  Replaces graphlet_core::sort_edges (graphlet_core.cpp:
 * 854-867) with get_ordering_value (:774-834) and the Vertex comparators
 * (graphlet_vertex.h:57-75).  order: "natural"/"off", "deg"/"degree",
 * "kcore", "kcore_deg", "deg_vol", "kcore_vol", "kcore_deg_vol", or any name
 * the reference maps past VAR (key = degree of e_u).  "rand"/"var" return
 * PGD_EUNSUPPORTED. */
pgd_status pgd_sort_edges(pgd_graph *g, const char *order, int small_to_large);

/* Edge order over a sample of edges.  Replaces the E_s overload of
 * graphlet_core::sort_edges (graphlet_core.cpp:836-851): edge_ids[0..k) are
 * edge ids (0 <= id < m, repeats allowed, k <= m) and the natural key is the
 * position in the sample.  A following pgd_decompose decomposes only these
 * k edges (sums and closed forms over the sample, with the whole graph's n
 * and m; t of unsampled edges is still read), as the reference's
 * decomposition iterates over E_ordered.  Batches reject sampled orders. */
pgd_status pgd_sort_edges_sample(pgd_graph *g, const char *order, int small_to_large, const int64_t *edge_ids,
                                 int64_t k);

/* Length of E_ordered (m, or the sample size of pgd_sort_edges_sample; 0
 * before any sort): the number of rows pgd_get_micro and the order array of
 * pgd_get_edges hold.  No reference counterpart (E_ordered.size()). */
int64_t pgd_graph_order_length(const pgd_graph *g);

/* ---- decomposition ----------------------------------------------------- */

#define PGD_MICRO 1u         /* also compute and keep the per-edge counts */

/* Exact decomposition.  Replaces graphlet_core::graphlet_decomposition
 * (graphlet_core.cpp:1366-1474) and graphlet_decomposition_micro (:1483-1625).
 * Runs pgd_preprocess("deg")/pgd_sort_edges("deg") first if they were not
 * called, as the reference does (:1376-1378). */
pgd_status pgd_decompose(pgd_graph *g, uint32_t flags, pgd_counts *out);

/* Per-edge rows of the last PGD_MICRO decomposition in E_ordered order, as
 * write_micro_stats prints them (graphlet_core.cpp:1668-1761): src1/dst1 are
 * e_v+1 / e_u+1 (may be NULL), cols is L x 8 row-major (L =
 * pgd_graph_order_length, m unless the order is sampled): triangle, 2-star,
 * 4-clique, 4-chordal-cycle, 4-tailed-triangle, 4-cycle, 3-star, 4-path. */
pgd_status pgd_get_micro(pgd_graph *g, int64_t *src1, int64_t *dst1, uint64_t *cols);

/* Edge arrays e_v/e_u (graphlet_core.h:230, m entries) and E_ordered ids
 * (graphlet_core.h:206, pgd_graph_order_length entries); any pointer may be
 * NULL. */
pgd_status pgd_get_edges(pgd_graph *g, int64_t *ev, int64_t *eu, int32_t *order);

/* Closing identities on the host (graphlet_core.cpp:1449-1472,
 * graphlet_core.h:548-557), exposed for callers that reduce sums
 * themselves. */
void pgd_close_counts(const uint64_t sums[PGD_NSUMS], int64_t n, int64_t m,
                      uint64_t totals[PGD_NTOTALS]);

/* ---- batched decomposition (no reference counterpart) ------------------
 * Many independent graphs decomposed together: the batch becomes one
 * disjoint-union graph on the device and runs through the same persistent
 * work-queue kernels (work items are (anchor, edge chunk) and edge spans of
 * every graph); per-graph results are identical to pgd_decompose (closed
 * forms use each graph's own n and m, sums are kept per graph).  Graphs not
 * yet preprocessed/sorted get the "deg" defaults.  With PGD_MICRO each
 * graph's per-edge rows are written to that graph (read with
 * pgd_get_micro).  out has k entries; kernel_ms is the batch's. */
pgd_status pgd_decompose_batch(pgd_ctx *ctx, pgd_graph *const *graphs, int k, uint32_t flags,
                               pgd_counts *out);

/* Batched decomposition straight from host pair lists (no reference
 * counterpart): graph g is the pairs [pair_off[g], pair_off[g+1]) of
 * src/dst (0-based ids local to the graph; edge-list rules: symmetrised,
 * deduplicated, self loops dropped), with n = max(n_min[g], 1 + largest id
 * with an edge) (n_min may be NULL).  The whole batch is built as one device
 * CSR and decomposed in one pass; out[g] gets graph g's global counts,
 * identical to building and decomposing it alone. */
pgd_status pgd_decompose_pairs_batch(pgd_ctx *ctx, int k, const int64_t *pair_off, const int32_t *src,
                                     const int32_t *dst, const int64_t *n_min, pgd_counts *out);

/* ---- request server (no reference counterpart) ---------------------------
 * Continuous batching: submitted graphs queue; `workers` threads, each with
 * its own context and stream, repeatedly admit pending requests, oldest
 * first, that fit the HBM budget (at most max_batch requests and about 2M
 * pairs per batch), decompose them together with pgd_decompose_pairs_batch,
 * and publish each request's global counts.  A request that does not fit the
 * memory left is passed by later, smaller ones until it has waited
 * max_wait_ms; then it goes next.  Requests that arrive while a batch runs
 * join the next one; batches of different workers run on the device at the
 * same time.  A request whose own memory estimate exceeds the budget
 * completes with PGD_ENOMEM.  Latency quantiles come from fixed log-spaced
 * histograms (2 % resolution). */
typedef struct pgd_server pgd_server;
typedef struct {
    int device;
    int workers;           /* default 2                                     */
    int max_batch;         /* requests per batch, default 4096              */
    int max_wait_ms;       /* age after which a request is no longer passed, default 20 */
    uint64_t hbm_budget;   /* bytes of admitted work; 0 = half of the device's free memory */
} pgd_server_opts;
typedef struct {
    uint64_t submitted, completed, rejected, batches;
    uint64_t inflight_bytes, peak_bytes;
    double p50_ms, p99_ms, mean_ms;   /* submit -> result latency            */
    double graphs_per_s;              /* completed / (last completion - first submit) */
    double queue_p50_ms, queue_p99_ms;       /* submit -> admission into a batch */
    double service_p50_ms, service_p99_ms;   /* admission -> result             */
    uint64_t skipped_ahead;           /* requests admitted ahead of an older one */
} pgd_server_stat;
pgd_status pgd_server_create(const pgd_server_opts *opts, pgd_server **out);
pgd_status pgd_server_submit(pgd_server *sv, const int32_t *src, const int32_t *dst, int64_t k, int64_t n_min,
                             uint64_t *ticket);
/* *done = 1 when finished: out gets the counts, the ticket is released and
 * the request's own status is returned. */
pgd_status pgd_server_poll(pgd_server *sv, uint64_t ticket, pgd_counts *out, int *done);
/* Waits up to timeout_ms; PGD_ETIMEOUT if the request is still running. */
pgd_status pgd_server_wait(pgd_server *sv, uint64_t ticket, int timeout_ms, pgd_counts *out);
pgd_status pgd_server_stats(pgd_server *sv, pgd_server_stat *st);
/* Finishes the queued requests, then stops the workers. */
pgd_status pgd_server_destroy(pgd_server *sv);

/* ---- thresholds and autotuning (no reference counterpart) --------------
 * Three thresholds steer how the decomposition kernels split work; counts
 * never depend on them.  Until the caller sets them (here or through
 * pgd_autotune), graphs of more than 1.5·2^20 vertices are decomposed with
 * anchor_hub 128 and cache_hub 40, the faster pair on large power-law
 * graphs.  anchor_hub (2..256, default 64): anchors of degree
 * >= it are processed one CTA per anchor with N(p) as a bitmap, below it one
 * warp per edge with N(p) staged and searched.  cache_hub (>= 2, default
 * 32): W(w,p) comes from the anchor's histogram for neighbours of degree >=
 * it (16-bit counters from degree 256, 8-bit below), below it N(w) is
 * scanned per edge.  dense_max (0..2048, default 2048): in a batch,
 * graphs of at most this many vertices are decomposed with whole adjacency
 * rows as bitsets (one 2048-bit row per warp), larger ones with sorted
 * lists; those of average degree >= n/16 also get a 16-bit common-neighbour
 * matrix (about 2·n² bytes of device memory while the batch runs).
 * A fourth, tensor_min_degree (0 or 2..1088, default 64): in those
 * common-neighbour graphs, the edges (p, q) whose lower-degree endpoint q has
 * degree in [tensor_min_degree, 1088] get their 4-clique count from a
 * product of q's ego network on the tensor cores (e4m3 0/1 operands, fp32
 * sums, exact); 0 keeps every edge on the integer path.
 * pgd_autotune decomposes the given graphs `reps` times per
 * candidate -- first dense_max in {0, 256, 1024, 2048}, then
 * tensor_min_degree in {0, 64, 128, 256}, then 16 (anchor_hub, cache_hub)
 * pairs -- checks that every candidate gives identical counts, keeps the
 * fastest on the context and reports it. */
pgd_status pgd_set_thresholds(pgd_ctx *ctx, int anchor_hub, int cache_hub, int dense_max);
pgd_status pgd_get_thresholds(const pgd_ctx *ctx, int *anchor_hub, int *cache_hub, int *dense_max);
pgd_status pgd_set_tensor_min_degree(pgd_ctx *ctx, int tensor_min_degree);
pgd_status pgd_get_tensor_min_degree(const pgd_ctx *ctx, int *tensor_min_degree);
pgd_status pgd_autotune(pgd_ctx *ctx, pgd_graph *const *graphs, int k, int reps, int *anchor_hub, int *cache_hub,
                        int *dense_max, float *best_ms);

/* ---- allocation-free decomposition --------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they need counts: a host framework that hands its plugins a
 * fixed device workspace and forbids allocation (its memory manager owns the
 * device), and latency-critical loops that cannot afford cudaMalloc/cudaFree,
 * which can synchronise the whole device.
 *
 * Global counts of a graph already on the device as a CSR (d_off: n+1 int64,
 * d_adj: nnz int32; offsets from 0 to nnz, non-decreasing; rows sorted,
 * symmetric, no self loops or repeats; anything else is refused with
 * PGD_EINVAL), on `stream` of `device`.  Every intermediate lives in one
 * static device array of pgd_noalloc_scratch_bytes() bytes (64 MiB) that the
 * library reserves on every GPU it is loaded on; the call never allocates.
 * Graphs that need more scratch than that are refused with PGD_ENOMEM and a
 * message in err.  The first call on a device looks up the array's address.
 * All calls share the array and each
 * clears what must start at zero: calls that overlap on the GPU race and must
 * be serialised by the caller.  The call synchronises `stream` up to four
 * times, because later launch sizes (hub-anchored edges, work items) are read
 * back to the host, and it leaves the calling thread's current device as it
 * found it.  Results (totals, sums, n, m) go to the host struct *out; err
 * (errlen bytes, may be NULL) receives a message on failure. */
pgd_status pgd_decompose_csr_noalloc(const int64_t *d_off, const int32_t *d_adj, int64_t n, int64_t nnz,
                                     int device, void *stream, pgd_counts *out, char *err, size_t errlen);
uint64_t pgd_noalloc_scratch_bytes(void);

#ifdef __cplusplus
}
#endif
#endif /* PGD_GB300_H */
