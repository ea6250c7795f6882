// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Drives the reference's own graphlet_core class (nkahmed/PGD, compiled from
// its unmodified sources by oracle/Makefile into oracle/_ref/) through its
// public C++ API, and exposes the results over a small C ABI so the Python
// tests can compare the CPU oracle and the GPU product against the real
// reference.  Nothing in the product links this file.
//
// Call sequence follows the reference's own driver (graphlet_driver.cpp:58-88)
// and, for CSR input, the route the CSR constructor needs
// (graphlet_core.h:156-160: initialize, vertex_degrees, preprocess).
#include "graphlet.h"

#include <stdint.h>
#include <string.h>

using namespace graphlet;

extern "C" {

void *ref_open_file(const char *path, const char *neigh, int s2l_neigh, int adj_limit, const char *rep) {
    return new graphlet_core(std::string(path), std::string(neigh), s2l_neigh != 0, adj_limit,
                             std::string(rep), 64);
}

void *ref_open_csr(int64_t n, const int64_t *off, const int32_t *adj, const char *neigh, int s2l_neigh,
                   int adj_limit, const char *rep) {
    // The CSR constructor (graphlet_core.h:156-160) runs vertex_degrees()
    // before initialize() has set block_size, so its OpenMP loop sees an
    // uninitialised chunk size.  The same state is reached without that by
    // the default constructor, initialize(), and the public CSR fields.
    graphlet_core *g = new graphlet_core();
    g->initialize();
    g->vertices.assign(off, off + n + 1);
    g->edges.assign(adj, adj + off[n]);
    g->vertex_degrees();
    g->preprocess(std::string(neigh), s2l_neigh != 0, adj_limit, std::string(rep));
    return g;
}

// Runs the driver's sequence: assortativity, cores, sort_edges, decomposition.
int ref_run(void *h, const char *order, int s2l, int micro, int workers) {
    graphlet_core *g = (graphlet_core *)h;
    g->compute_assortativity();
    g->compute_cores();
    g->sort_edges(std::string(order), s2l != 0);
    if (micro) g->graphlet_decomposition_micro(workers);
    else g->graphlet_decomposition(workers);
    return 0;
}

// Timing sample for the CPU baseline: the reference's own sampled edge order
// (sort_edges over a subset E_s, graphlet_core.cpp:837-851) holding every
// stride-th edge of the full order, then its decomposition over that subset.
// Returns the number of edges; *seconds is the decomposition's wall time.
long long ref_run_sample(void *h, const char *order, int s2l, int workers, long long stride, double *seconds) {
    graphlet_core *g = (graphlet_core *)h;
    g->compute_cores();
    g->E_ordered.clear();
    g->sort_edges(std::string(order), s2l != 0);
    std::vector<unsigned long> sample;
    for (size_t i = 0; i < g->E_ordered.size(); i += (size_t)stride) sample.push_back(g->E_ordered[i].get_id());
    g->E_ordered.clear();
    g->sort_edges(std::string(order), s2l != 0, sample);
    double t0 = get_time();
    g->graphlet_decomposition(workers);
    *seconds = get_time() - t0;
    return (long long)sample.size();
}

// The reference's own sampled path: sort_edges with E_s = ids[0..k), then the
// decomposition (per-edge rows too when micro).
void ref_run_ids(void *h, const char *order, int s2l, const int64_t *ids, long long k, int micro, int workers) {
    graphlet_core *g = (graphlet_core *)h;
    g->compute_cores();
    std::vector<unsigned long> sample((size_t)k);
    for (long long i = 0; i < k; i++) sample[(size_t)i] = (unsigned long)ids[i];
    g->E_ordered.clear();
    g->sort_edges(std::string(order), s2l != 0, sample);
    if (micro) g->graphlet_decomposition_micro(workers);
    else g->graphlet_decomposition(workers);
}

void ref_totals(void *h, uint64_t *out) {
    graphlet_core *g = (graphlet_core *)h;
    const unsigned long long v[17] = {
        g->total_2_1edge, g->total_2_indep, g->total_3_tris, g->total_2_star, g->total_3_1edge,
        g->total_3_indep, g->total_4_clique, g->total_4_chordcycle, g->total_4_tailed_tris,
        g->total_4_cycle, g->total_3_star, g->total_4_path, g->total_4_2edge, g->total_4_1edge,
        g->total_4_2star, g->total_4_tri, g->total_4_indep};
    for (int i = 0; i < 17; i++) out[i] = v[i];
}

int64_t ref_n(void *h) { return ((graphlet_core *)h)->num_vertices(); }
int64_t ref_m(void *h) { return ((graphlet_core *)h)->num_edges(); }
int ref_max_core(void *h) { return ((graphlet_core *)h)->get_max_core(); }
double ref_r(void *h) { return ((graphlet_core *)h)->get_assortativity(); }
int ref_is_adj(void *h) { return ((graphlet_core *)h)->is_adj_exists() ? 1 : 0; }

// Rows in E_ordered order, as write_micro_stats prints them
// (graphlet_core.cpp:1689-1701).
int64_t ref_n_ord(void *h) { return (int64_t)((graphlet_core *)h)->E_ordered.size(); }

void ref_micro(void *h, int64_t *src1, int64_t *dst1, uint64_t *cols) {
    graphlet_core *g = (graphlet_core *)h;
    for (long long e = 0; e < (long long)g->E_ordered.size(); e++) {
        long long id = g->E_ordered[e].get_id();
        long long v = g->e_v[id], u = g->e_u[id];
        long long dv = g->vertices[v + 1] - g->vertices[v], du = g->vertices[u + 1] - g->vertices[u];
        src1[e] = v + 1;
        dst1[e] = u + 1;
        uint64_t *r = cols + 8 * e;
        r[0] = g->tri[e];
        r[1] = g->get_2_star(e, dv, du);
        r[2] = g->local_4_clique[e];
        r[3] = g->local_4_chordal_cycle[e];
        r[4] = g->local_4_tailed_tris[e];
        r[5] = g->local_4_cycle[e];
        r[6] = g->local_3_star[e];
        r[7] = g->local_4_path[e];
    }
}

void ref_csr(void *h, int64_t *off, int32_t *adj) {
    graphlet_core *g = (graphlet_core *)h;
    for (size_t i = 0; i < g->vertices.size(); i++) off[i] = g->vertices[i];
    for (size_t i = 0; i < g->edges.size(); i++) adj[i] = g->edges[i];
}

void ref_close(void *h) { delete (graphlet_core *)h; }

}  // extern "C"
