/*
 * pgd_gen.h -- seeded synthetic graph generators (no reference counterpart).
 *
 * Stand-ins for the graph shapes the benchmark configurations name: RMAT,
 * Erdos-Renyi G(n,p), Barabasi-Albert and 3-D random geometric graphs.  All
 * randomness comes from a counter-based mixer (the SplitMix64 output
 * function applied to seed and draw index), so every result is a pure
 * function of the arguments, independent of thread count and machine.
 * Outputs are undirected pairs (0-based ids) that may contain self loops and
 * repeats where the model produces them; pgd_graph_from_edges with
 * PGD_EDGES_DEDUP turns them into a simple graph.
 */
#ifndef PGD_GEN_H
#define PGD_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Uniform double in [0,1) for (seed, stream, index). */
double pgd_gen_u01(uint64_t seed, uint64_t stream, uint64_t index);

/* RMAT: k = edge_factor << scale draws; draw i picks one quadrant per level
 * l (bit l of src/dst) with probabilities a, b, c, 1-a-b-c (b sets the dst
 * bit, c the src bit).  src/dst must hold k entries. */
void pgd_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int32_t *src,
                  int32_t *dst);

/* G(n, p): pair (i, j), i < j, is an edge iff u01(seed, ER, index(i,j)) < p.
 * Writes at most cap pairs; returns the number of edges (which may exceed
 * cap, in which case only cap were written). */
int64_t pgd_gen_er(int64_t n, double p, uint64_t seed, int32_t *src, int32_t *dst, int64_t cap);

/* Barabasi-Albert: vertices 0..m0 start as a clique (m0 = m_attach); every
 * later vertex attaches to m_attach distinct earlier vertices chosen with
 * probability proportional to degree.  Returns the edge count (writes at
 * most cap). */
int64_t pgd_gen_ba(int64_t n, int m_attach, uint64_t seed, int32_t *src, int32_t *dst, int64_t cap);

/* 3-D random geometric graph: n points uniform in the unit cube, an edge
 * between every pair closer than radius.  Returns the edge count (writes at
 * most cap). */
int64_t pgd_gen_rgg3d(int64_t n, double radius, uint64_t seed, int32_t *src, int32_t *dst, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
