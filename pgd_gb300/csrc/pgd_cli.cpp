// pgd_cli.cpp -- the drop-in `pgd` command line tool.
//
// Same flags and the same run sequence as the reference's driver
// (graphlet_driver.cpp:53-92, flags graphlet_params.h:216-287): read the
// graph, print basic stats, assortativity (r) and max k-core (K), order the
// edges, decompose (global or with -m per edge), print the 17 counts, the
// per-edge table (-m), the timing line, write -c/-m files, print the three
// graphlet frequency distributions and (-m) the summary of per-edge 4-clique
// counts.  -w/-b/-r/-l/-a are accepted and have no effect: the GPU kernels
// pick their own work split and representation, and none of these change a
// count in the reference either.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <sys/time.h>

#include <algorithm>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "graphlet_core.hpp"

namespace {

struct Params {
    std::string algorithm = "exact", graph = "sample_graph.csv", macro_file, micro_file;
    std::string ordering = "deg", neigh_ordering = "deg", rep;
    int workers = 1, block_size = 64, adj_limit = 10000;
    bool verbose = false, help = false, s2l = false, s2l_neigh = false;
};

void usage(const char *argv0) {
    fprintf(stderr,
            "Usage: %s -f path [options]\n"
            "  exact 3- and 4-node graphlet decomposition on one GPU\n"
            "  -f, --file, --graph, -g FILE   input graph (.mtx, or an edge list: csv/tab/space)\n"
            "  -m, --micro FILE               also compute per-edge counts and write them to FILE\n"
            "  -c, --counts, --macro FILE     write the global counts to FILE\n"
            "  -o, --ordering, --order NAME   edge order: deg (default), kcore, natural, kcore_deg, ...\n"
            "      --s2l                      order smallest to largest\n"
            "  -n, --neigh_ordering NAME      neighbour order: deg (default), kcore, natural\n"
            "      --s2l_neigh                neighbour order smallest to largest\n"
            "  -w, -b, -r, -l, -a VALUE       accepted for compatibility; no effect on the GPU\n"
            "  -v, --verbose                  print the parameters\n"
            "  -h, -?, --help                 this text\n",
            argv0);
    exit(-1);
}

double now() {
    struct timeval t;
    gettimeofday(&t, 0);
    return t.tv_sec * 1.0 + t.tv_usec / 1000000.0;
}

void print_line(int n, const std::string &sym = "-") {
    for (int i = 0; i < n; ++i) std::cout << sym;
    std::cout << std::endl;
}

Params parse(int argc, char **argv) {
    if (argc <= 1) usage(argv[0]);
    Params p;
    std::map<std::string, int *> ints;
    ints["-w"] = ints["--workers"] = ints["--threads"] = ints["--cores"] = &p.workers;
    ints["-b"] = ints["--block_size"] = &p.block_size;
    ints["-l"] = ints["--adj_limit"] = ints["--adj_size"] = &p.adj_limit;
    std::map<std::string, bool *> bools;
    bools["-?"] = bools["-h"] = bools["--help"] = &p.help;
    bools["-v"] = bools["--verbose"] = &p.verbose;
    bools["--s2l"] = bools["--small_to_large"] = &p.s2l;
    bools["--s2l_neigh"] = bools["--small_to_large_neigh"] = &p.s2l_neigh;
    std::map<std::string, std::string *> strs;
    strs["-f"] = strs["--graph"] = strs["--file"] = strs["-g"] = &p.graph;
    strs["-a"] = strs["--algorithm"] = strs["--alg"] = &p.algorithm;
    strs["-c"] = strs["--counts"] = strs["--macro"] = &p.macro_file;
    strs["-m"] = strs["--micro"] = &p.micro_file;
    strs["-r"] = strs["--rep"] = &p.rep;
    strs["-o"] = strs["--ordering"] = strs["--order"] = &p.ordering;
    strs["-n"] = strs["--neigh_ordering"] = strs["--neigh_order"] = strs["--csc_ordering"] =
        strs["--neighbor_ordering"] = &p.neigh_ordering;
    for (int i = 1; i < argc; ++i) {
        std::string flag(argv[i]);
        if (bools.count(flag)) { *bools[flag] = true; continue; }
        if (i + 1 < argc) {
            if (ints.count(flag)) *ints[flag] = atoi(argv[++i]);
            else if (strs.count(flag)) *strs[flag] = std::string(argv[++i]);
            else printf("Invalid argument %s, ignoring.\n", flag.c_str());
        }
    }
    if (p.help) usage(argv[0]);
    if (p.workers <= 0) p.workers = 1;
    FILE *f = fopen(p.graph.c_str(), "r");
    if (!f) usage(argv[0]);
    fclose(f);
    if (p.verbose) {
        print_line(80, "=");
        std::cout << "GB300 graphlet decomposition (pgd)" << std::endl;
        print_line(80, "=");
        std::cout << "file: " << p.graph << std::endl;
        std::cout << "ordering: " << p.ordering << (p.s2l ? ", smallest to largest" : ", largest to smallest") << std::endl;
        std::cout << "csc/neighbor ordering: " << p.neigh_ordering
                  << (p.s2l_neigh ? ", smallest to largest" : ", largest to smallest") << std::endl;
        std::cout << "macro (per graph counts) output: " << p.macro_file << std::endl;
        std::cout << "micro (per edge counts)  output: " << p.micro_file << std::endl;
        print_line(80);
        std::cout << std::endl;
    }
    return p;
}

// Summary of per-edge 4-clique counts printed after a -m run, computed as
// univar_stats does (graphlet_univar_stats.h:75-108): integer mean and
// median of even-sized data, min starting (and staying) at 0.
std::string univar(const std::vector<unsigned long long> &data) {
    double sum_sq = 0;
    unsigned long long sum = 0, mx = 0, mn = 0, count = 0;
    for (size_t i = 0; i < data.size(); i++) {
        sum_sq += (double)(data[i] * data[i]);
        sum += data[i];
        if (data[i] > mx) mx = data[i];
        if (data[i] < mn) mn = data[i];
        count++;
    }
    double mean = count ? (double)(sum / count) : 0;
    double var = (sum_sq / (double)count) - (mean * mean);
    double sd = sqrt(var);
    unsigned long long range = mx - mn;
    std::vector<unsigned long long> arr = data;
    std::sort(arr.begin(), arr.end());
    unsigned long long med_idx = count / 2, q_idx = count / 4;
    double median = 0, q1 = 0, q3 = 0;
    if (count) {
        median = (double)arr[med_idx];
        if (arr.size() % 2 == 0) median = (double)((arr[med_idx - 1] + arr[med_idx]) / 2);
        q1 = (double)arr[med_idx - q_idx];
        q3 = (double)arr[med_idx + q_idx];
    }
    double iqr = q3 - q1;
    std::ostringstream os;
    os << "mean\t= " << mean << "\n";
    os << "median\t= " << median << "\n";
    os << "max\t= " << mx << "\n";
    os << "min\t= " << mn << "\n";
    os << "range\t= " << range << "\n";
    os << "std\t= " << sd << "\n";
    os << "var\t= " << var << "\n";
    os << "iqr\t= " << iqr << "\n";
    os << "q1\t= " << q1 << "\n";
    os << "q3\t= " << q3 << "\n";
    return os.str();
}

}  // namespace

int main(int argc, char *argv[]) {
    Params p = parse(argc, argv);
    if (p.verbose) std::cout << "graph file: " << p.graph << std::endl;
    graphlet::graphlet_core G(p.graph, p.neigh_ordering, p.s2l_neigh, p.adj_limit, p.rep, p.block_size);

    G.compute_assortativity();
    if (std::isnan(G.get_assortativity())) std::cout << "r = -nan" << std::endl;  // as printed on x86-64
    else std::cout << "r = " << G.get_assortativity() << std::endl;
    G.compute_cores();
    std::cout << "K = " << G.get_max_core() << std::endl;

    bool micro = !p.micro_file.empty();
    double s = now();
    G.sort_edges(p.ordering, p.s2l);
    if (micro) G.graphlet_decomposition_micro(p.workers);
    else G.graphlet_decomposition(p.workers);
    s = now() - s;
    G.print_graphlet_counts();
    if (micro) G.print_micro_stats();
    std::cout << "graphlet decomposition time: " << s << " sec" << std::endl;
    if (p.verbose) std::cout << "decomposition kernels: " << G.last_kernel_ms() << " ms" << std::endl;

    if (!p.macro_file.empty()) G.write_macro_stats(p.macro_file);
    if (micro) G.write_micro_stats(p.micro_file);
    G.print_GFD();
    G.print_connected_GFD();
    G.print_disconnected_GFD();
    if (micro) std::cout << univar(G.local_4_clique) << std::endl;
    return 0;
}
