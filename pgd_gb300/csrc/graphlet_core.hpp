// graphlet_core.hpp -- C++ interface mirroring the reference's
// graphlet::graphlet_core (graphlet_core.h:54-702) for the decomposition path,
// implemented on the C ABI (include/pgd_gb300.h).  Code written against the
// reference's class for this path -- construct, preprocess, compute_cores,
// sort_edges, graphlet_decomposition[_micro], read total_* and the per-edge
// vectors, print or write them -- compiles and runs unchanged against this
// header; the work runs on the GPU.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "pgd_gb300.h"

namespace graphlet {

class graphlet_core {
   public:
    // graphlet_core.h:152-160
    explicit graphlet_core(const std::string &filename, std::string ordering_technique = "degree",
                           bool is_small_to_large = false, int adj_limit = 10000, std::string rep = "auto",
                           int block_sz = 64);
    graphlet_core(std::vector<long long> vs, std::vector<int> es);
    ~graphlet_core();
    graphlet_core(const graphlet_core &) = delete;
    graphlet_core &operator=(const graphlet_core &) = delete;

    // pipeline (graphlet_core.h:164, 207-209, 559-560, 659, 679)
    void initialize();
    void vertex_degrees();
    void preprocess(std::string ordering_csc_neighbor = "degree", bool is_small_to_large = false,
                    int adj_limit = 10000, std::string rep = "auto");
    void compute_cores();
    void compute_assortativity();
    void sort_edges(std::string edge_ordering = "degree", bool is_small_to_large = false);
    // the E_s overload (graphlet_core.h:208-209): order and decompose only the sampled edge ids
    void sort_edges(std::string edge_ordering, bool is_small_to_large, std::vector<unsigned long> &E_s);
    void graphlet_decomposition(int max_num_workers = 1);
    void graphlet_decomposition_micro(int max_num_workers = 1);

    // graph properties
    int num_vertices() const { return (int)n_; }
    int num_edges() const { return (int)m_; }
    int get_max_degree() const { return max_degree; }
    double get_avg_degree() const { return avg_degree; }
    double density() const { return (double)num_edges() / (num_vertices() * (num_vertices() - 1.0) / 2.0); }
    int get_max_core() const { return max_core; }
    double get_assortativity() const { return r; }
    void basic_stats(std::string prefix = "", std::string suffix = "\n");

    // output (graphlet_core.h:454-508, 512-538)
    void print_graphlet_counts();
    std::string get_graphlet_counts();
    void write_macro_stats(std::string filename);
    void write_micro_stats(std::string &filename, bool output_id = true, unsigned int buffer_size = 0);
    std::string get_micro_stats(bool output_id = true, std::string delim = ",");
    void print_micro_stats(bool output_id = true, std::string delim = ",");
    std::string compute_GFD();
    std::string compute_connected_GFD();
    std::string compute_disconnected_GFD();
    void print_GFD();
    void print_connected_GFD();
    void print_disconnected_GFD();
    unsigned long long get_2_star(long long e) const;

    bool ok() const { return graph_ != nullptr; }
    const std::string &error() const { return err_; }
    float last_kernel_ms() const { return kernel_ms_; }

    // public state as in the reference
    int max_degree = 0, avg_degree = 0, max_core = 0;
    double r = 0;
    std::vector<long long> e_v, e_u;
    std::vector<int> E_ordered;   // edge ids in processing order
    unsigned long long total_2_1edge = 0, total_2_indep = 0, total_3_tris = 0, total_2_star = 0,
                       total_3_1edge = 0, total_3_indep = 0, total_4_clique = 0, total_4_chordcycle = 0,
                       total_4_tailed_tris = 0, total_4_cycle = 0, total_3_star = 0, total_4_path = 0,
                       total_4_2edge = 0, total_4_1edge = 0, total_4_2star = 0, total_4_tri = 0, total_4_indep = 0;
    std::vector<unsigned long long> tri, local_4_clique, local_4_chordal_cycle, local_4_tailed_tris, local_4_cycle,
        local_3_star, local_4_path;
    std::vector<double> GFD, connected_GFD, disconnected_GFD;

   private:
    void check(pgd_status st, const char *what);
    void fetch_edges();
    void decompose(bool micro);
    pgd_ctx *ctx_ = nullptr;
    pgd_graph *graph_ = nullptr;
    int64_t n_ = 0, m_ = 0;
    std::string err_;
    bool preprocessed_ = false;
    std::vector<long long> row_deg_sum_;  // deg(e_v)+deg(e_u) per row, for get_2_star
    std::vector<unsigned long long> two_star_;
    float kernel_ms_ = 0;
};

}  // namespace graphlet
