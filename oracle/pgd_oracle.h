/*
 * pgd_oracle.h -- CPU oracle for PGD's edge-centric graphlet decomposition.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (nkahmed/PGD, graphlet_core.cpp) used as the checker for the GPU
 * product path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; the product library never links or calls it.
 *
 * Parity is pinned against the reference's own fixtures (sample_graph.csv
 * per-edge golden rows, the toy graphs in data/) and against the reference
 * compiled from its sources (oracle/Makefile -> oracle/_ref/).
 */
#ifndef PGD_ORACLE_H
#define PGD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct po_graph po_graph;

/* Number of raw per-edge partial sums kept by the decomposition (see
 * po_decompose): t, 2-star, 3-node-1-edge, 4-clique, 4-cycle, N1..N10. */
#define PO_NSUMS 15
/* Number of global motif counts (graphlet_core.h:310-329). */
#define PO_NTOTALS 17
/* Number of per-edge output columns (graphlet_core.cpp:1677-1684). */
#define PO_NMICRO 8

/* Readers.  Return NULL and fill err (if non-NULL, 256 bytes) on failure. */
po_graph *po_read_file(const char *path, char *err);
/* CSR as given (row order = "insertion order" of the reference's CSR ctor,
 * graphlet_core.h:156-160). */
po_graph *po_from_csr(int64_t n, const int64_t *off, const int32_t *adj, char *err);
/* Undirected pairs read the way read_mtx does (graphlet_core.cpp:459-522):
 * ids are 0-based here, self loops dropped, no dedup, n = 1 + max id that
 * has an edge (or n_min if larger). */
po_graph *po_from_pairs(int64_t k, const int32_t *src, const int32_t *dst, int64_t n_min,
                        int dedup, char *err);
void po_free(po_graph *g);

/* graphlet_core::preprocess (graphlet_core.cpp:77-93) minus the adj matrix:
 * neighbour ordering + e_v/e_u construction. */
int po_preprocess(po_graph *g, const char *neigh_order, int s2l);
/* graphlet_core::compute_cores (graphlet_core.cpp:958-1018). */
int po_compute_cores(po_graph *g);
/* graphlet_core::compute_assortativity (graphlet_core.cpp:1029-1057). */
double po_assortativity(po_graph *g);
/* graphlet_core::sort_edges (graphlet_core.cpp:854-867). */
int po_sort_edges(po_graph *g, const char *order, int s2l);
/* sort_edges over a sample of edge ids (graphlet_core.cpp:836-851); the
 * following po_decompose covers only those k positions. */
int po_sort_edges_sample(po_graph *g, const char *order, int s2l, const int64_t *ids, int64_t k);
/* graphlet_decomposition[_micro] (graphlet_core.cpp:1366-1625).  threads<=0
 * means all cores.  cheap_side!=0 scans the endpoint with the smaller 2-hop
 * volume instead of always e_u (same counts, less work on power-law graphs). */
int po_decompose(po_graph *g, int micro, int threads, int cheap_side);

/* Timing sample for the CPU baseline: runs the per-edge loop (global
 * counts) over E_ordered positions 0, stride, 2*stride, ... with all or
 * `threads` threads and returns the number of edges done; *seconds gets the
 * wall time of the loop alone.  Results are not kept. */
int64_t po_decompose_sample(po_graph *g, int threads, int cheap_side, int64_t stride, double *seconds);

/* t, k4, c4 of the edges (vs[i], us[i]), each by the reference's own
 * marking procedure (graphlet_core.cpp:1069-1240: mark N(v), scan N(u));
 * for checking sampled rows of graphs too large for a full oracle run.
 * Needs only the CSR. */
int po_edge_sample(po_graph *g, int64_t k, const int64_t *vs, const int64_t *us, uint64_t *t, uint64_t *k4,
                   uint64_t *c4, int threads);

/* The 8 per-edge columns of one edge (graphlet_core.cpp:1559-1575 and
 * graphlet_core.h:353-355) from its endpoint degrees and t, k4, c4. */
void po_micro_row(long long dv, long long du, uint64_t t, uint64_t k4, uint64_t c4, uint64_t row[PO_NMICRO]);

/* Closing identities (graphlet_core.cpp:1449-1472, graphlet_core.h:548-557). */
void po_close(const uint64_t sums[PO_NSUMS], int64_t n, int64_t m, uint64_t totals[PO_NTOTALS]);

/* Accessors. */
int64_t po_n(const po_graph *g);
int64_t po_m(const po_graph *g);
int64_t po_n_ord(const po_graph *g);   /* E_ordered length: m or the sample size */
int po_max_degree(const po_graph *g);
int po_max_core(const po_graph *g);
void po_get_csr(const po_graph *g, int64_t *off, int32_t *adj);
void po_get_edges(const po_graph *g, int64_t *ev, int64_t *eu);
void po_get_order(const po_graph *g, int32_t *ids);
void po_get_kcore(const po_graph *g, int32_t *kcore); /* n+1 entries, 1-based layout */
void po_get_sums(const po_graph *g, uint64_t *sums);
void po_get_totals(const po_graph *g, uint64_t *totals);
/* Rows in E_ordered order: src+1, dst+1 (as printed) and the 8 columns. */
void po_get_micro(const po_graph *g, int64_t *src1, int64_t *dst1, uint64_t *cols);
/* Per-edge values by edge id (undirected edge index of e_v/e_u):
 * t, k4, c4 -- convenient for keyed comparisons. */
void po_get_edge_tkc(const po_graph *g, uint64_t *t, uint64_t *k4, uint64_t *c4);

/* Seeded RMAT pairs (edge_factor << scale draws), identical to the product's
 * generator for the same arguments; src/dst hold edge_factor << scale ids. */
void po_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int32_t *src,
                 int32_t *dst);

#ifdef __cplusplus
}
#endif
#endif
