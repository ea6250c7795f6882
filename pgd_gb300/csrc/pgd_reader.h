// pgd_reader.h -- host tokenisation of graph files (reader.cpp).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

struct ReadResult {
    std::vector<int32_t> src, dst;  // undirected pairs in file order, 0-based ids
    bool is_mtx = false;            // mtx: no dedup; edge list: dedup
    int64_t self_loops = 0;
    std::string error;
};

bool pgd_read_graph_file(const std::string &path, ReadResult &r);
