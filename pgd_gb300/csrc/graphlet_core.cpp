// graphlet_core.cpp -- the graphlet_core mirror (graphlet_core.hpp) on the C ABI.
// Output formats follow the reference's writers: print_graphlet_counts
// (graphlet_core.cpp:2061-2084), get_graphlet_counts (:2138-2162),
// write_micro_stats (:1668-1761), get_micro_stats (:1772-1817), the GFD
// printers (:1955-2056) and basic_stats (:562-568).
#include "graphlet_core.hpp"

#include <stdio.h>
#include <stdlib.h>

#include <fstream>
#include <iostream>
#include <sstream>

namespace graphlet {

static void line_of(int n, const std::string &sym = "-") {
    for (int i = 0; i < n; ++i) std::cout << sym;
    std::cout << std::endl;
}

static pgd_ctx *shared_ctx() {
    static pgd_ctx *ctx = nullptr;
    if (!ctx) {
        pgd_status st = pgd_context_create(nullptr, &ctx);
        if (st != PGD_OK) {
            std::cerr << "[pgd] no usable CUDA device: " << pgd_status_string(st) << std::endl;
            exit(1);
        }
    }
    return ctx;
}

void graphlet_core::check(pgd_status st, const char *what) {
    if (st == PGD_OK) return;
    err_ = std::string(what) + ": " + pgd_status_string(st) + " -- " + pgd_last_error(ctx_);
    std::cerr << "[pgd] " << err_ << std::endl;
    exit(1);
}

graphlet_core::graphlet_core(const std::string &filename, std::string ordering_technique, bool is_small_to_large,
                             int adj_limit, std::string rep, int block_sz) {
    (void)adj_limit; (void)rep; (void)block_sz;
    ctx_ = shared_ctx();
    std::string ext;
    size_t dot = filename.rfind('.');
    if (dot != std::string::npos) ext = filename.substr(dot + 1);
    if (ext != "mtx") std::cout << "[reading generic edge list: read_edge_list func]  filename: " << filename << std::endl;
    // messages the reference's readers print about the first data line
    {
        std::ifstream f(filename.c_str());
        std::string line;
        bool banner = false;
        while (std::getline(f, line) && !line.empty() && (line[0] == '#' || line[0] == '%'))
            if (line.find("MatrixMarket matrix coordinate pattern symmetric") != std::string::npos) banner = true;
        if (ext == "mtx") {
            std::istringstream ss(line);
            long long rows = 0, cols = 0;
            ss >> rows >> cols;
            if (rows != cols) std::cout << "[pgd]  error: this is not a square matrix, attempting to proceed." << std::endl;
        } else {
            if (!banner && line.find(',') == std::string::npos && line.find('\t') == std::string::npos &&
                line.find("   ") != std::string::npos)
                printf("found tab-spaces delimiter \n");
            std::istringstream ss(line);
            std::string tok;
            int k = 0;
            while (ss >> tok) k++;
            if (k == 3) printf("weighted graph detected \n");
            fflush(stdout);
        }
    }
    check(pgd_graph_from_file(ctx_, filename.c_str(), &graph_), "read graph");
    vertex_degrees();
    basic_stats();
    preprocess(ordering_technique, is_small_to_large);
}

graphlet_core::graphlet_core(std::vector<long long> vs, std::vector<int> es) {
    ctx_ = shared_ctx();
    std::vector<int64_t> off(vs.begin(), vs.end());
    check(pgd_graph_from_csr(ctx_, off.data(), es.data(), (int64_t)off.size() - 1, &graph_), "CSR graph");
    vertex_degrees();
}

graphlet_core::~graphlet_core() {
    if (graph_) pgd_graph_destroy(graph_);
}

void graphlet_core::initialize() {
    max_degree = 0;
    avg_degree = 0;
    max_core = 0;
}

void graphlet_core::vertex_degrees() {
    pgd_info info;
    check(pgd_graph_info(graph_, &info), "graph info");
    n_ = info.n;
    m_ = info.m;
    max_degree = info.max_degree;
    avg_degree = info.avg_degree;
}

void graphlet_core::basic_stats(std::string prefix, std::string suffix) {
    std::cout << prefix << "|V|: " << num_vertices() << suffix;
    std::cout << prefix << "|E|: " << num_edges() << suffix;
    std::cout << prefix << "p: " << density() << suffix;
    std::cout << prefix << "d_max: " << get_max_degree() << suffix;
    std::cout << prefix << "d_avg: " << get_avg_degree() << suffix;
}

void graphlet_core::fetch_edges() {
    e_v.assign((size_t)m_, 0);
    e_u.assign((size_t)m_, 0);
    std::vector<int64_t> a((size_t)m_ + 1), b((size_t)m_ + 1);
    check(pgd_get_edges(graph_, a.data(), b.data(), nullptr), "edge arrays");
    for (int64_t i = 0; i < m_; i++) { e_v[i] = a[i]; e_u[i] = b[i]; }
}

void graphlet_core::preprocess(std::string ordering_csc_neighbor, bool is_small_to_large, int adj_limit,
                               std::string rep) {
    (void)adj_limit; (void)rep;
    check(pgd_preprocess(graph_, ordering_csc_neighbor.c_str(), is_small_to_large ? 1 : 0), "preprocess");
    preprocessed_ = true;
    fetch_edges();
}

void graphlet_core::compute_cores() {
    int32_t k = 0;
    check(pgd_compute_cores(graph_, &k), "compute_cores");
    max_core = k;
}

void graphlet_core::compute_assortativity() {
    double rr = 0;
    check(pgd_assortativity(graph_, &rr), "compute_assortativity");
    r = rr;
}

void graphlet_core::sort_edges(std::string edge_ordering, bool is_small_to_large) {
    check(pgd_sort_edges(graph_, edge_ordering.c_str(), is_small_to_large ? 1 : 0), "sort_edges");
    E_ordered.assign((size_t)pgd_graph_order_length(graph_), 0);
    check(pgd_get_edges(graph_, nullptr, nullptr, E_ordered.data()), "sort_edges");
}

void graphlet_core::sort_edges(std::string edge_ordering, bool is_small_to_large, std::vector<unsigned long> &E_s) {
    std::vector<int64_t> ids(E_s.begin(), E_s.end());
    check(pgd_sort_edges_sample(graph_, edge_ordering.c_str(), is_small_to_large ? 1 : 0, ids.data(),
                                (int64_t)ids.size()),
          "sort_edges");
    E_ordered.assign((size_t)pgd_graph_order_length(graph_), 0);
    check(pgd_get_edges(graph_, nullptr, nullptr, E_ordered.data()), "sort_edges");
}

void graphlet_core::decompose(bool micro) {
    if (!preprocessed_) preprocess();
    if (E_ordered.empty() && m_ > 0) sort_edges();
    pgd_counts c;
    check(pgd_decompose(graph_, micro ? PGD_MICRO : 0u, &c), "graphlet_decomposition");
    kernel_ms_ = c.kernel_ms;
    unsigned long long *f[PGD_NTOTALS] = {&total_2_1edge, &total_2_indep, &total_3_tris, &total_2_star,
                                          &total_3_1edge, &total_3_indep, &total_4_clique, &total_4_chordcycle,
                                          &total_4_tailed_tris, &total_4_cycle, &total_3_star, &total_4_path,
                                          &total_4_2edge, &total_4_1edge, &total_4_2star, &total_4_tri,
                                          &total_4_indep};
    for (int i = 0; i < PGD_NTOTALS; i++) *f[i] = c.totals[i];
    if (micro) {
        const int64_t rows = pgd_graph_order_length(graph_);
        std::vector<uint64_t> cols((size_t)rows * PGD_NMICRO + 1);
        check(pgd_get_micro(graph_, nullptr, nullptr, cols.data()), "micro counts");
        std::vector<unsigned long long> *dst[PGD_NMICRO] = {&tri, &two_star_, &local_4_clique,
                                                            &local_4_chordal_cycle, &local_4_tailed_tris,
                                                            &local_4_cycle, &local_3_star, &local_4_path};
        for (int c2 = 0; c2 < PGD_NMICRO; c2++) {
            dst[c2]->resize((size_t)rows);
            for (int64_t e = 0; e < rows; e++) (*dst[c2])[e] = cols[(size_t)e * PGD_NMICRO + c2];
        }
    }
}

void graphlet_core::graphlet_decomposition(int) { decompose(false); }
void graphlet_core::graphlet_decomposition_micro(int) { decompose(true); }

unsigned long long graphlet_core::get_2_star(long long e) const { return two_star_[(size_t)e]; }

void graphlet_core::print_graphlet_counts() {
    line_of(60, "*");
    std::cout << "total_2_1edge = " << total_2_1edge << std::endl;
    std::cout << "total_2_indep = " << total_2_indep << std::endl;
    line_of(40);
    std::cout << "total_3_tris = " << total_3_tris << std::endl;
    std::cout << "total_2_star = " << total_2_star << std::endl;
    std::cout << "total_3_1edge = " << total_3_1edge << std::endl;
    std::cout << "total_3_indep = " << total_3_indep << std::endl;
    line_of(40);
    std::cout << "total_4_clique = " << total_4_clique << std::endl;
    std::cout << "total_4_chordcycle = " << total_4_chordcycle << std::endl;
    std::cout << "total_4_tailed_tris = " << total_4_tailed_tris << std::endl;
    std::cout << "total_4_cycle = " << total_4_cycle << std::endl;
    std::cout << "total_3_star = " << total_3_star << std::endl;
    std::cout << "total_4_path = " << total_4_path << std::endl;
    line_of(40);
    std::cout << "total_4_1edge = " << total_4_1edge << std::endl;
    std::cout << "total_4_2edge = " << total_4_2edge << std::endl;
    std::cout << "total_4_2star = " << total_4_2star << std::endl;
    std::cout << "total_4_tri = " << total_4_tri << std::endl;
    std::cout << "total_4_indep = " << total_4_indep << std::endl;
    line_of(60, "*");
}

std::string graphlet_core::get_graphlet_counts() {
    std::ostringstream s;
    s << "total_2_1edge = " << total_2_1edge << "\n";
    s << "total_2_indep = " << total_2_indep << "\n";
    s << "total_3_tris = " << total_3_tris << "\n";
    s << "total_2_star = " << total_2_star << "\n";
    s << "total_3_1edge = " << total_3_1edge << "\n";
    s << "total_3_indep = " << total_3_indep << "\n";
    s << "total_4_clique = " << total_4_clique << "\n";
    s << "total_4_chordcycle = " << total_4_chordcycle << "\n";
    s << "total_4_tailed_tris = " << total_4_tailed_tris << "\n";
    s << "total_4_cycle = " << total_4_cycle << "\n";
    s << "total_3_star = " << total_3_star << "\n";
    s << "total_4_path = " << total_4_path << "\n";
    s << "total_4_1edge = " << total_4_1edge << "\n";
    s << "total_4_2edge = " << total_4_2edge << "\n";
    s << "total_4_2star = " << total_4_2star << "\n";
    s << "total_4_tri = " << total_4_tri << "\n";
    s << "total_4_indep = " << total_4_indep << "\n";
    return s.str();
}

void graphlet_core::write_macro_stats(std::string filename) {
    std::ofstream f(filename.c_str());
    f << get_graphlet_counts();
}

static const char *kMicroHeader =
    "triangle,2-star,4-clique,4-chordal-cycle,4-tailed-triangle,4-cycle,3-star,4-path";

static void micro_row(std::ostream &os, const graphlet_core &g, long long e, bool output_id, const std::string &d) {
    if (output_id) {
        long long id = g.E_ordered[(size_t)e];
        os << (g.e_v[(size_t)id] + 1) << d << (g.e_u[(size_t)id] + 1) << d;
    }
    os << g.tri[(size_t)e] << d << g.get_2_star(e) << d << g.local_4_clique[(size_t)e] << d
       << g.local_4_chordal_cycle[(size_t)e] << d << g.local_4_tailed_tris[(size_t)e] << d
       << g.local_4_cycle[(size_t)e] << d << g.local_3_star[(size_t)e] << d << g.local_4_path[(size_t)e];
}

void graphlet_core::write_micro_stats(std::string &filename, bool output_id, unsigned int) {
    std::ofstream f(filename.c_str());
    std::ostringstream s;
    s << "% ";
    if (output_id) s << "src,dst,";
    s << kMicroHeader << "\n";
    f << s.str();
    for (long long e = 0; e < (long long)tri.size(); e++) {
        micro_row(f, *this, e, output_id, ",");
        f << "\n";
    }
}

std::string graphlet_core::get_micro_stats(bool output_id, std::string delim) {
    std::ostringstream s;
    if (output_id) s << "src" << delim << "dst" << delim;
    s << "triangle" << delim << "2-star" << delim << "4-clique" << delim << "4-chordal-cycle" << delim
      << "4-tailed-triangle" << delim << "4-cycle" << delim << "3-star" << delim << "4-path" << "\n";
    for (long long e = 0; e < (long long)tri.size(); e++) {
        micro_row(s, *this, e, output_id, delim);
        s << "\n";
    }
    return s.str();
}

void graphlet_core::print_micro_stats(bool output_id, std::string delim) {
    line_of(80);
    std::cout << "\n\nMicro graphlet statistics" << std::endl;
    line_of(80);
    std::cout << get_micro_stats(output_id, delim) << std::endl;
}

static std::string gfd_block(const std::vector<unsigned long long> &g, const char *const *names, bool guard_zero,
                             bool last_is_rest, std::vector<double> &out) {
    std::ostringstream os;
    unsigned long long sum = 0;
    for (size_t i = 0; i < g.size(); i++) sum += g[i];
    double cum = 0;
    std::vector<double> d(g.size(), 0);
    for (size_t i = 0; i < g.size(); i++) {
        if (!guard_zero || sum > 0) d[i] = (double)g[i] / (double)sum;
        else d[i] = 0;
        os << names[i] << "\t" << d[i] << "\n";
        cum += d[i];
    }
    if (last_is_rest) d[g.size() - 1] = 1.0 - cum;
    os << "\n";
    out = d;
    return os.str();
}

std::string graphlet_core::compute_GFD() {
    static const char *names[] = {"4-clique     ", "4-chordal-cycle", "4-tailed-tri", "4-cycle       ",
                                  "3-star       ", "4-path       ", "4-node-1-tri   ", "4-node-2-star  ",
                                  "4-node-2-edge", "4-node-1-edge  ", "4-node-indep  "};
    std::vector<unsigned long long> g = {total_4_clique, total_4_chordcycle, total_4_tailed_tris, total_4_cycle,
                                         total_3_star, total_4_path, total_4_tri, total_4_2star,
                                         total_4_2edge, total_4_1edge, total_4_indep};
    return gfd_block(g, names, false, true, GFD);
}

std::string graphlet_core::compute_connected_GFD() {
    static const char *names[] = {"4-clique     ", "4-chordal-cycle", "4-tailed-tri", "4-cycle       ",
                                  "3-star       ", "4-path       "};
    std::vector<unsigned long long> g = {total_4_clique, total_4_chordcycle, total_4_tailed_tris,
                                         total_4_cycle, total_3_star, total_4_path};
    return gfd_block(g, names, true, false, connected_GFD);
}

std::string graphlet_core::compute_disconnected_GFD() {
    static const char *names[] = {"4-node-1-tri   ", "4-node-2-star", "4-node-2-edge  ", "4-node-1-edge  ",
                                  "4-node-indep  "};
    std::vector<unsigned long long> g = {total_4_tri, total_4_2star, total_4_2edge, total_4_1edge, total_4_indep};
    return gfd_block(g, names, true, true, disconnected_GFD);
}

void graphlet_core::print_GFD() {
    line_of(80);
    std::cout << "Graphlet Frequency Distribution (GFD)\n";
    line_of(80);
    std::cout << compute_GFD() << std::endl;
}

void graphlet_core::print_connected_GFD() {
    line_of(80);
    std::cout << "Connected Motif Graphlet Frequency Distribution (GFD)\n";
    line_of(80);
    std::cout << compute_connected_GFD() << std::endl;
}

void graphlet_core::print_disconnected_GFD() {
    line_of(80);
    std::cout << "Disconnected Motif Graphlet Frequency Distribution (GFD)\n";
    line_of(80);
    std::cout << compute_disconnected_GFD() << std::endl;
}

}  // namespace graphlet
