// reader.cpp -- host-side tokenisation of graph files with the reference
// reader's rules.  The resulting pairs go to the device, which symmetrises,
// sorts and deduplicates them (graph_build.cu).
//
//   read_graph dispatch        graphlet_core.cpp:259-283  (extension after the last '.')
//   read_edge_list             graphlet_core.cpp:291-457
//   read_mtx                   graphlet_core.cpp:459-522
//   get_token / detect_delim   graphlet_core.cpp:196-241
#include <stdint.h>
#include <stdlib.h>

#include <cctype>
#include <climits>
#include <fstream>
#include <string>
#include <vector>

#include "pgd_reader.h"

namespace {

// std::string::find based tokenizer of the reference (get_token): a value is
// assigned only when a non-empty token is found, so an empty field keeps the
// previous line's value.
void next_token(const std::string &line, const std::string &delim, size_t &prev, int &v) {
    size_t pos = line.find(delim, prev);
    if (pos != std::string::npos) {
        if (pos > prev) v = atoi(line.substr(prev, pos - prev).c_str());
        prev = pos + 1;
    } else if (prev < line.length()) {
        v = atoi(line.substr(prev).c_str());
    }
}

// `stream >> int` on one line with the C++11 library rule: leading white
// space skipped; end of input leaves the target alone; a non-number stores
// 0; either failure stops later extractions.
struct LineStream {
    const std::string &s;
    size_t i = 0;
    bool failed = false;
    explicit LineStream(const std::string &str) : s(str) {}
    void get(int &v) {
        if (failed) return;
        while (i < s.size() && isspace((unsigned char)s[i])) i++;
        if (i >= s.size()) { failed = true; return; }
        size_t j = i;
        if (s[j] == '+' || s[j] == '-') j++;
        if (j >= s.size() || !isdigit((unsigned char)s[j])) { v = 0; failed = true; return; }
        char *end = nullptr;
        long val = strtol(s.c_str() + i, &end, 10);
        if (val > INT_MAX) val = INT_MAX;
        if (val < INT_MIN) val = INT_MIN;
        v = (int)val;
        i = (size_t)(end - s.c_str());
    }
};

std::string extension(const std::string &path) {
    size_t dot = path.rfind('.');
    return dot == std::string::npos ? std::string() : path.substr(dot + 1);
}

bool is_comment(const std::string &l) { return !l.empty() && (l[0] == '%' || l[0] == '#'); }

bool read_mtx(const std::string &path, ReadResult &r) {
    std::ifstream f(path.c_str());
    if (!f) { r.error = "file not found: " + path; return false; }
    std::string line;
    bool have = false;
    while (std::getline(f, line)) {
        if (is_comment(line)) continue;
        have = true;
        break;
    }
    int v = -1, u = -1;
    bool fix_start = true;
    if (have && !line.empty()) {
        LineStream ls(line);
        ls.get(v);
        ls.get(u);
        if (v == 0 || u == 0) fix_start = false;
    }
    while (have && fix_start && std::getline(f, line)) {
        if (line.empty() || is_comment(line)) continue;
        LineStream ls(line);
        ls.get(v);
        ls.get(u);
        v--;
        u--;
        if (v == u) { r.self_loops++; continue; }
        if (v < 0 || u < 0) { r.error = "vertex id < 1 in mtx file"; return false; }
        r.src.push_back(v);
        r.dst.push_back(u);
    }
    r.is_mtx = true;
    return true;
}

bool read_edge_list(const std::string &path, ReadResult &r) {
    std::ifstream f(path.c_str());
    if (!f) { r.error = "file not found: " + path; return false; }
    std::string line, delim;
    // comment block at the top; an "MatrixMarket ... symmetric" banner forces
    // a space delimiter
    bool have = false;
    while (std::getline(f, line)) {
        if (is_comment(line)) {
            if (line.find("MatrixMarket matrix coordinate pattern symmetric") != std::string::npos) delim = " ";
            continue;
        }
        have = true;
        break;
    }
    if (!have) line.clear();
    if (delim.empty()) {
        if (line.find(',') != std::string::npos) delim = ",";
        else if (line.find('\t') != std::string::npos) delim = "\t";
        else if (line.find("   ") != std::string::npos) delim = "   ";
        else if (line.find(' ') != std::string::npos) delim = " ";
    }
    if (delim.empty()) {
        std::string ext = extension(path);
        delim = ext == "csv" ? "," : (ext == "tab" ? "\t" : " ");
    }
    int v = -1, u = -1;
    bool fix_start = true;
    long long max_id = 0;
    if (!line.empty()) {
        LineStream ls(line);
        ls.get(v);
        ls.get(u);
        if (v == 0 || u == 0) fix_start = false;
        if (!is_comment(line)) {
            // the first data line's ids also size the relabel table here
            size_t prev = 0;
            int a = v, b = u;
            next_token(line, delim, prev, a);
            next_token(line, delim, prev, b);
            if (a > max_id) max_id = a;
            if (b > max_id) max_id = b;
        }
    }
    while (std::getline(f, line)) {
        if (line.empty() || is_comment(line)) continue;
        size_t prev = 0;
        next_token(line, delim, prev, v);
        next_token(line, delim, prev, u);
        if (v == 0 || u == 0) fix_start = false;
        if (v < 0 || u < 0) { r.error = "negative vertex id"; return false; }
        if (v > max_id) max_id = v;
        if (u > max_id) max_id = u;
    }
    f.close();
    std::ifstream g(path.c_str());
    if (!g) { r.error = "file not found: " + path; return false; }
    std::vector<int32_t> lookup((size_t)max_id + 2, -1);
    int32_t next_id = 0;
    while (std::getline(g, line)) {
        if (line.empty() || is_comment(line)) continue;
        size_t prev = 0;
        next_token(line, delim, prev, v);
        next_token(line, delim, prev, u);
        if (fix_start) { v--; u--; }
        if (v == u) { r.self_loops++; continue; }
        if (v < 0 || u < 0 || v > max_id || u > max_id) { r.error = "vertex id out of range"; return false; }
        if (lookup[v] == -1) lookup[v] = next_id++;
        v = lookup[v];
        if (lookup[u] == -1) lookup[u] = next_id++;
        u = lookup[u];
        r.src.push_back(v);
        r.dst.push_back(u);
    }
    r.is_mtx = false;
    return true;
}

}  // namespace

bool pgd_read_graph_file(const std::string &path, ReadResult &r) {
    if (extension(path) == "mtx") return read_mtx(path, r);
    return read_edge_list(path, r);
}
