// ingest.cu -- graph files parsed on the device, with the reference reader's
// rules.
//
//   read_graph dispatch        graphlet_core.cpp:259-283  (extension after the last '.')
//   read_edge_list             graphlet_core.cpp:291-457  (two passes: ids and 0/1 base, then first-seen relabel)
//   read_mtx                   graphlet_core.cpp:459-522  (1-based ids, no dedup)
//   get_token / detect_delim   graphlet_core.cpp:196-241
//
// The host reads the file's bytes once and copies them to the device; the
// host only looks at the header (the comment block and the first data line,
// which decide the delimiter and, for mtx, whether any edge is read).  On the
// device: the newline positions are selected, every line is tokenised by one
// thread with the reference's token rules, the reader's checks and the
// first-seen relabel are data-parallel (first occurrence of an id = minimum
// position, relabel = rank of first occurrences by a scan), and the pairs go
// straight into the device CSR build.
//
// One quirk of the reference resists that: a line whose id field is empty or
// missing keeps the previous line's value, and in the relabel pass that value
// has already been decremented and relabelled.  Files with such a line are
// read by a single device thread that follows the reference's loops line by
// line (slow, exact); well-formed files never take it.
#include <stdio.h>
#include <string.h>

#include <climits>
#include <cub/cub.cuh>
#include <string>
#include <vector>

#include "pgd_internal.h"

namespace {

constexpr int kThreads = 256;

inline int grid_for(int64_t n, int per_block = kThreads, int cap = 1 << 20) {
    int64_t g = (n + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

// ---------------------------------------------------------------------------
// Token rules, shared by the host (header) and the device (every line).

__host__ __device__ __forceinline__ bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}
__host__ __device__ __forceinline__ bool is_digit(char c) { return c >= '0' && c <= '9'; }

// strtol(s, &end, 10) over [p, e) from its first character: optional sign,
// digits; the magnitude saturates at LONG_MAX / LONG_MIN.  *end = first
// character not consumed.  Returns 0 with *end = p when there is no digit.
__host__ __device__ inline long long parse_long(const char *p, const char *e, const char **end) {
    const char *q = p;
    bool neg = false;
    if (q < e && (*q == '+' || *q == '-')) {
        neg = *q == '-';
        q++;
    }
    if (q >= e || !is_digit(*q)) {
        *end = p;
        return 0;
    }
    const unsigned long long limit = neg ? (1ull << 63) : (1ull << 63) - 1;
    unsigned long long mag = 0;
    while (q < e && is_digit(*q)) {
        const unsigned d = (unsigned)(*q - '0');
        mag = mag > (limit - d) / 10 ? limit : mag * 10 + d;
        q++;
    }
    *end = q;
    return neg ? (long long)(0ull - mag) : (long long)mag;
}

// atoi over [p, e): white space skipped, then strtol, then the int
// conversion keeps the low 32 bits (as glibc's atoi does).
__host__ __device__ inline int atoi_range(const char *p, const char *e) {
    while (p < e && is_space(*p)) p++;
    const char *end;
    const long long v = parse_long(p, e, &end);
    return (int)(uint32_t)(unsigned long long)v;
}

// line.find(delim, from) for a 1- or 3-character delimiter; -1 if absent.
__host__ __device__ inline int64_t find_delim(const char *s, int64_t len, const char *d, int dl, int64_t from) {
    for (int64_t i = from; i + dl <= len; i++) {
        bool ok = true;
        for (int k = 0; k < dl; k++) ok = ok && s[i + k] == d[k];
        if (ok) return i;
    }
    return -1;
}

// get_token: a value is assigned only when a non-empty token is found.
__host__ __device__ inline bool next_token(const char *s, int64_t len, const char *d, int dl, int64_t &prev, int &v) {
    const int64_t pos = find_delim(s, len, d, dl, prev);
    if (pos >= 0) {
        const bool set = pos > prev;
        if (set) v = atoi_range(s + prev, s + pos);
        prev = pos + 1;
        return set;
    }
    if (prev < len) {
        v = atoi_range(s + prev, s + len);
        return true;
    }
    return false;
}

// `stream >> int` on one line (C++11 rules): white space skipped; end of
// line leaves v alone; a non-number stores 0; either failure stops later
// extractions.  Values beyond int saturate.  Returns whether v was assigned.
struct LineInts {
    const char *s;
    int64_t len, i = 0;
    bool failed = false;
    __host__ __device__ LineInts(const char *s_, int64_t len_) : s(s_), len(len_) {}
    __host__ __device__ bool get(int &v) {
        if (failed) return false;
        while (i < len && is_space(s[i])) i++;
        if (i >= len) {
            failed = true;
            return false;
        }
        int64_t j = i;
        if (s[j] == '+' || s[j] == '-') j++;
        if (j >= len || !is_digit(s[j])) {
            v = 0;
            failed = true;
            return true;
        }
        const char *end;
        long long x = parse_long(s + i, s + len, &end);
        if (x > INT_MAX) x = INT_MAX;
        if (x < INT_MIN) x = INT_MIN;
        v = (int)x;
        i = end - s;
        return true;
    }
};

__host__ __device__ __forceinline__ bool is_comment(const char *s, int64_t len) {
    return len > 0 && (s[0] == '%' || s[0] == '#');
}

// ---------------------------------------------------------------------------
// Device passes.

// Newlines of 1 KiB chunks, one warp per chunk: counted, then (after a scan
// of the counts) written in order.
constexpr int kChunk = 1024;

__global__ void k_nl_count(const char *buf, int64_t bytes, int64_t nchunks, unsigned long long *counts) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; c < nchunks; c += nw) {
        unsigned n = 0;
        for (int r = 0; r < kChunk / 32; r++) {
            const int64_t i = c * kChunk + r * 32 + lane;
            n += __popc(__ballot_sync(0xffffffffu, i < bytes && buf[i] == '\n'));
        }
        if (lane == 0) counts[c] = n;
    }
}

__global__ void k_nl_write(const char *buf, int64_t bytes, int64_t nchunks, const unsigned long long *offs,
                           int64_t *nl) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; c < nchunks; c += nw) {
        int64_t at = (int64_t)offs[c];
        for (int r = 0; r < kChunk / 32; r++) {
            const int64_t i = c * kChunk + r * 32 + lane;
            const bool is_nl = i < bytes && buf[i] == '\n';
            const unsigned m = __ballot_sync(0xffffffffu, is_nl);
            if (is_nl) nl[at + __popc(m & ((1u << lane) - 1))] = i;
            at += __popc(m);
        }
    }
}

struct Lines {
    const char *buf;        // the region's bytes
    int64_t bytes;
    const int64_t *nl;      // positions of its newlines
    int64_t nnl;
    int64_t count;          // lines: nnl, plus one when the region does not end with a newline
    __device__ void span(int64_t j, int64_t &s, int64_t &e) const {
        s = j ? nl[j - 1] + 1 : 0;
        e = j < nnl ? nl[j] : bytes;
    }
};

// Per line: flags bit0 data line, bit1 first id assigned, bit2 second id
// assigned; a, b the ids (edge lists: get_token twice; mtx: stream >> int twice).
__global__ void k_parse_lines(Lines L, int mtx, char d0, char d1, char d2, int dl, uint8_t *flags, int32_t *a,
                              int32_t *b) {
    const char d[3] = {d0, d1, d2};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < L.count; j += (int64_t)gridDim.x * blockDim.x) {
        int64_t s, e;
        L.span(j, s, e);
        const char *p = L.buf + s;
        const int64_t len = e - s;
        uint8_t f = 0;
        int va = 0, vb = 0;
        if (len > 0 && !is_comment(p, len)) {
            f = 1;
            if (mtx) {
                LineInts li(p, len);
                if (li.get(va)) f |= 2;
                if (li.get(vb)) f |= 4;
            } else {
                int64_t prev = 0;
                if (next_token(p, len, d, dl, prev, va)) f |= 2;
                if (next_token(p, len, d, dl, prev, vb)) f |= 4;
            }
        }
        flags[j] = f;
        a[j] = va;
        b[j] = vb;
    }
}

// st: [0] data lines with an id missing, [1] any zero id in lines j >= j0,
// [2] any negative id there, [3] their max id (as int, >= 0).  j0 = 1 when
// line 0 is the header's first data line (checked on the host), else 0.
__global__ void k_edge_pass1(const uint8_t *flags, const int32_t *a, const int32_t *b, int64_t count, int64_t j0,
                             unsigned long long *st) {
    unsigned long long incomplete = 0, zero = 0, neg = 0;
    int mx = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t f = flags[j];
        if (!(f & 1)) continue;
        if ((f & 6) != 6) incomplete++;
        if (j < j0) continue;   // the first data line is checked by the host
        const int x = a[j], y = b[j];
        zero |= (x == 0 || y == 0);
        neg |= (x < 0 || y < 0);
        mx = max(mx, max(x, y));
    }
    if (incomplete) atomicAdd(st, incomplete);
    if (zero) atomicOr(st + 1, 1ull);
    if (neg) atomicOr(st + 2, 1ull);
    atomicMax((int *)(st + 3), mx);
}

// relabel pass: ids decremented when the file is 1-based, self loops
// dropped (counted), ids range-checked, and the first position of every id
// (2 j for the first id of line j, 2 j + 1 for the second) kept by atomicMin.
// st: [4] self loops, [5] ids out of range
__global__ void k_edge_pass2(const uint8_t *flags, const int32_t *a, const int32_t *b, int64_t count, int fix,
                             int max_id, uint64_t *first, uint32_t *keep, unsigned long long *st) {
    unsigned long long loops = 0, bad = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x) {
        uint32_t k = 0;
        if (flags[j] & 1) {
            const int v = a[j] - fix, u = b[j] - fix;
            if (v == u) loops++;
            else if (v < 0 || u < 0 || v > max_id || u > max_id) bad++;
            else {
                k = 1;
                atomicMin((unsigned long long *)first + v, (unsigned long long)(2 * j));
                atomicMin((unsigned long long *)first + u, (unsigned long long)(2 * j + 1));
            }
        }
        keep[j] = k;
    }
    if (loops) atomicAdd(st + 4, loops);
    if (bad) atomicAdd(st + 5, bad);
}

// position p = 2 j + side of a kept line is a first occurrence
__global__ void k_first_flags(const uint32_t *keep, const int32_t *a, const int32_t *b, int64_t count, int fix,
                              const uint64_t *first, uint32_t *pflag) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x) {
        uint32_t fa = 0, fb = 0;
        if (keep[j]) {
            fa = first[a[j] - fix] == (uint64_t)(2 * j);
            fb = first[b[j] - fix] == (uint64_t)(2 * j + 1);
        }
        pflag[2 * j] = fa;
        pflag[2 * j + 1] = fb;
    }
}

// new id of a first occurrence = number of first occurrences before it
__global__ void k_relabel_table(const uint32_t *keep, const int32_t *a, const int32_t *b, int64_t count, int fix,
                                const uint32_t *pflag, const uint32_t *prank, int32_t *lookup) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x) {
        if (!keep[j]) continue;
        if (pflag[2 * j]) lookup[a[j] - fix] = (int32_t)prank[2 * j];
        if (pflag[2 * j + 1]) lookup[b[j] - fix] = (int32_t)prank[2 * j + 1];
    }
}

// kept lines to pairs, in file order; relabelled (edge lists) or as read (mtx)
__global__ void k_emit_pairs(const uint32_t *keep, const uint32_t *kpos, const int32_t *a, const int32_t *b,
                             int64_t count, int fix, const int32_t *lookup, int32_t *src, int32_t *dst) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x) {
        if (!keep[j]) continue;
        const int v = a[j] - fix, u = b[j] - fix;
        src[kpos[j]] = lookup ? lookup[v] : v;
        dst[kpos[j]] = lookup ? lookup[u] : u;
    }
}

// mtx lines: ids minus one, self loops dropped (counted), negative ids
// counted as errors.  st: [0] lines with an id missing, [4] self loops,
// [5] negative ids
__global__ void k_mtx_pass(const uint8_t *flags, const int32_t *a, const int32_t *b, int64_t count, uint32_t *keep,
                           unsigned long long *st) {
    unsigned long long incomplete = 0, loops = 0, bad = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x) {
        uint32_t k = 0;
        const uint8_t f = flags[j];
        if (f & 1) {
            if ((f & 6) != 6) incomplete++;
            const int v = a[j] - 1, u = b[j] - 1;
            if (v == u) loops++;
            else if (v < 0 || u < 0) bad++;
            else k = 1;
        }
        keep[j] = k;
    }
    if (incomplete) atomicAdd(st, incomplete);
    if (loops) atomicAdd(st + 4, loops);
    if (bad) atomicAdd(st + 5, bad);
}

// The reference's loops, line by line, for files with a missing id field
// (values carry over from the previous line).  One thread.
// Edge list, pass 1: st[1] zero seen, st[2] negative seen, st[3] max id,
// st[6] / st[7] the ids carried out of the pass.
__global__ void k_seq_edge_pass1(const uint8_t *flags, const int32_t *a, const int32_t *b, int64_t count, int64_t j0,
                                 int v0, int u0, unsigned long long *st) {
    if (blockIdx.x || threadIdx.x) return;
    int v = v0, u = u0;
    int mx = 0;
    bool zero = false, neg = false;
    for (int64_t j = j0; j < count; j++) {
        const uint8_t f = flags[j];
        if (!(f & 1)) continue;
        if (f & 2) v = a[j];
        if (f & 4) u = b[j];
        zero |= (v == 0 || u == 0);
        if (v < 0 || u < 0) { neg = true; break; }
        mx = max(mx, max(v, u));
    }
    st[1] = zero;
    st[2] = neg;
    st[3] = (unsigned long long)(unsigned)mx;
    st[6] = (unsigned long long)(unsigned)v;
    st[7] = (unsigned long long)(unsigned)u;
}

// Edge list, pass 2 (relabel), carrying the decremented and relabelled ids.
// lookup: max_id + 2 entries set to -1.  st[4] self loops, st[5] error,
// st[8] pairs written.
__global__ void k_seq_edge_pass2(const uint8_t *flags, const int32_t *a, const int32_t *b, int64_t count, int v0,
                                 int u0, int fix, int max_id, int32_t *lookup, int32_t *src, int32_t *dst,
                                 unsigned long long *st) {
    if (blockIdx.x || threadIdx.x) return;
    int v = v0, u = u0;
    int32_t next_id = 0;
    unsigned long long loops = 0, k = 0, err = 0;
    for (int64_t j = 0; j < count; j++) {
        const uint8_t f = flags[j];
        if (!(f & 1)) continue;
        if (f & 2) v = a[j];
        if (f & 4) u = b[j];
        if (fix) { v--; u--; }
        if (v == u) { loops++; continue; }
        if (v < 0 || u < 0 || v > max_id || u > max_id) { err = 1; break; }
        if (lookup[v] == -1) lookup[v] = next_id++;
        v = lookup[v];
        if (lookup[u] == -1) lookup[u] = next_id++;
        u = lookup[u];
        src[k] = v;
        dst[k] = u;
        k++;
    }
    st[4] = loops;
    st[5] = err;
    st[8] = k;
}

// mtx, carrying the decremented ids of the previous line.  st[4] self loops,
// st[5] negative id, st[8] pairs written.
__global__ void k_seq_mtx(const uint8_t *flags, const int32_t *a, const int32_t *b, int64_t count, int v0, int u0,
                          int32_t *src, int32_t *dst, unsigned long long *st) {
    if (blockIdx.x || threadIdx.x) return;
    int v = v0, u = u0;
    unsigned long long loops = 0, k = 0, err = 0;
    for (int64_t j = 0; j < count; j++) {
        const uint8_t f = flags[j];
        if (!(f & 1)) continue;
        if (f & 2) v = a[j];
        if (f & 4) u = b[j];
        v--;
        u--;
        if (v == u) { loops++; continue; }
        if (v < 0 || u < 0) { err = 1; break; }
        src[k] = v;
        dst[k] = u;
        k++;
    }
    st[4] = loops;
    st[5] = err;
    st[8] = k;
}

// ---------------------------------------------------------------------------
// Host side.

std::string file_extension(const std::string &path) {
    const size_t dot = path.rfind('.');
    return dot == std::string::npos ? std::string() : path.substr(dot + 1);
}

// What the host learns from the header.
struct Header {
    bool mtx = false;
    int64_t region = 0;        // byte offset where the device's lines start
    bool any = false;          // a non-comment line exists
    bool first_data = false;   // ... and it is not empty (edge list: the first data line)
    char delim[4] = {0, 0, 0, 0};
    int dl = 0;
    int v = -1, u = -1;        // ids after the header's `stream >> int`
    bool fix = true;           // ids 1-based (edge list) / edges to read (mtx)
    int first_max = 0;         // edge list: max of the first line's get_token values
};

Header read_header(const char *buf, int64_t n, const std::string &path) {
    Header h;
    h.mtx = file_extension(path) == "mtx";
    bool banner = false;
    int64_t pos = 0, ls = 0, le = 0;
    while (pos < n) {
        int64_t e = pos;
        while (e < n && buf[e] != '\n') e++;
        ls = pos;
        le = e;
        pos = e + 1;
        if (is_comment(buf + ls, le - ls)) {
            const std::string line(buf + ls, (size_t)(le - ls));
            if (line.find("MatrixMarket matrix coordinate pattern symmetric") != std::string::npos) banner = true;
            continue;
        }
        h.any = true;
        break;
    }
    if (!h.any) {
        ls = le = n;
        pos = n;
    }
    const char *line = buf + ls;
    const int64_t len = le - ls;
    if (h.mtx) {
        // the size line: a 0 among its first two numbers means no edge is read
        if (h.any && len > 0) {
            LineInts li(line, len);
            li.get(h.v);
            li.get(h.u);
            if (h.v == 0 || h.u == 0) h.fix = false;
        }
        h.region = std::min(pos, n);
        return h;
    }
    std::string d = banner ? " " : "";
    if (d.empty()) {
        const std::string l(line, (size_t)len);
        if (l.find(',') != std::string::npos) d = ",";
        else if (l.find('\t') != std::string::npos) d = "\t";
        else if (l.find("   ") != std::string::npos) d = "   ";
        else if (l.find(' ') != std::string::npos) d = " ";
    }
    if (d.empty()) {
        const std::string ext = file_extension(path);
        d = ext == "csv" ? "," : (ext == "tab" ? "\t" : " ");
    }
    h.dl = (int)d.size();
    memcpy(h.delim, d.data(), d.size());
    h.first_data = h.any && len > 0;
    if (h.first_data) {
        LineInts li(line, len);
        li.get(h.v);
        li.get(h.u);
        if (h.v == 0 || h.u == 0) h.fix = false;
        int a = h.v, b = h.u;
        int64_t prev = 0;
        next_token(line, len, h.delim, h.dl, prev, a);
        next_token(line, len, h.delim, h.dl, prev, b);
        h.first_max = std::max(0, std::max(a, b));
        h.region = ls;   // the first data line is the device's line 0
    } else {
        h.region = std::min(pos, n);   // an empty first line: nothing special follows
    }
    return h;
}

struct Tmp {
    pgd_ctx *ctx;
    std::vector<void *> held;
    explicit Tmp(pgd_ctx *c) : ctx(c) {}
    Tmp(const Tmp &) = delete;
    Tmp &operator=(const Tmp &) = delete;
    ~Tmp() {
        for (void *p : held) pgd_tmp_free(ctx, p);
    }
    template <typename T>
    pgd_status alloc(T **out, size_t bytes) {
        void *p = nullptr;
        const pgd_status st = pgd_tmp_alloc(ctx, &p, bytes ? bytes : 1);
        if (st == PGD_OK) {
            held.push_back(p);
            *out = (T *)p;
        }
        return st;
    }
};

template <typename In, typename Out>
pgd_status exclusive_scan(pgd_ctx *ctx, In in, Out out, int64_t count) {
    size_t tb = 0;
    void *tmp = nullptr;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, in, out, count, ctx->stream);
    pgd_status st = pgd_tmp_alloc(ctx, &tmp, tb ? tb : 1);
    if (st) return st;
    cub::DeviceScan::ExclusiveSum(tmp, tb, in, out, count, ctx->stream);
    pgd_tmp_free(ctx, tmp);
    return PGD_OK;
}

}  // namespace

// Reads `path` with the reference reader's rules, parsing on the device, and
// builds the graph's CSR from the resulting pairs.  *mtx tells the caller
// which rules applied.
pgd_status pgd_build_from_file(pgd_graph *g, const char *path, bool *mtx) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    FILE *f = fopen(path, "rb");
    if (!f) return pgd_fail(ctx, PGD_EIO, std::string("file not found: ") + path);
    fseek(f, 0, SEEK_END);
    const long size = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (size < 0) {
        fclose(f);
        return pgd_fail(ctx, PGD_EIO, std::string("cannot read ") + path);
    }
    char *hbuf = nullptr;
    if (cudaHostAlloc((void **)&hbuf, (size_t)size + 1, cudaHostAllocDefault) != cudaSuccess) {
        fclose(f);
        cudaGetLastError();
        return pgd_fail(ctx, PGD_ENOMEM, "cannot allocate a pinned buffer for the file");
    }
    const size_t got = fread(hbuf, 1, (size_t)size, f);
    fclose(f);
    struct HostFree {
        char *p;
        ~HostFree() { cudaFreeHost(p); }
    } host_free{hbuf};
    if (got != (size_t)size) return pgd_fail(ctx, PGD_EIO, std::string("cannot read ") + path);
    const Header h = read_header(hbuf, size, path);
    *mtx = h.mtx;
    const int64_t bytes = size - h.region;
    Tmp tmp(ctx);
    unsigned long long *stats = ctx->d_ctr;   // [0..8] pass results
    PGD_CUDA(ctx, cudaMemsetAsync(stats, 0, 10 * sizeof(unsigned long long), s));
    if ((h.mtx && !h.fix) || bytes <= 0) return pgd_build_from_device_pairs(g, nullptr, nullptr, 0, 0, !h.mtx);

    // ---- lines of the region -------------------------------------------------
    char *dbuf = nullptr;
    if ((st = tmp.alloc(&dbuf, (size_t)bytes))) return st;
    PGD_CUDA(ctx, cudaMemcpyAsync(dbuf, hbuf + h.region, (size_t)bytes, cudaMemcpyHostToDevice, s));
    // newline positions: counted per chunk, scanned, written in order
    const int64_t nchunks = (bytes + kChunk - 1) / kChunk;
    unsigned long long *ccount = nullptr, *coff = nullptr;
    if ((st = tmp.alloc(&ccount, (size_t)(nchunks + 1) * sizeof(unsigned long long)))) return st;
    if ((st = tmp.alloc(&coff, (size_t)(nchunks + 1) * sizeof(unsigned long long)))) return st;
    PGD_CUDA(ctx, cudaMemsetAsync(ccount + nchunks, 0, sizeof(unsigned long long), s));
    PGD_LAUNCH(ctx, k_nl_count, grid_for(32 * nchunks), kThreads, 0, dbuf, bytes, nchunks, ccount);
    if ((st = exclusive_scan(ctx, ccount, coff, nchunks + 1))) return st;
    unsigned long long h_nnl = 0;
    PGD_CUDA(ctx, cudaMemcpyAsync(&h_nnl, coff + nchunks, sizeof(h_nnl), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    const int64_t nnl = (int64_t)h_nnl;
    int64_t *nl = nullptr;
    if ((st = tmp.alloc(&nl, (size_t)(nnl + 1) * sizeof(int64_t)))) return st;
    PGD_LAUNCH(ctx, k_nl_write, grid_for(32 * nchunks), kThreads, 0, dbuf, bytes, nchunks, coff, nl);
    Lines L;
    L.buf = dbuf;
    L.bytes = bytes;
    L.nl = nl;
    L.nnl = nnl;
    L.count = nnl + (hbuf[size - 1] != '\n' ? 1 : 0);
    const int64_t count = L.count;
    uint8_t *flags = nullptr;
    int32_t *a = nullptr, *b = nullptr;
    uint32_t *keep = nullptr, *kpos = nullptr;
    if ((st = tmp.alloc(&flags, (size_t)count))) return st;
    if ((st = tmp.alloc(&a, (size_t)count * sizeof(int32_t)))) return st;
    if ((st = tmp.alloc(&b, (size_t)count * sizeof(int32_t)))) return st;
    if ((st = tmp.alloc(&keep, (size_t)(count + 1) * sizeof(uint32_t)))) return st;
    if ((st = tmp.alloc(&kpos, (size_t)(count + 1) * sizeof(uint32_t)))) return st;
    PGD_LAUNCH(ctx, k_parse_lines, grid_for(count), kThreads, 0, L, h.mtx ? 1 : 0, h.delim[0], h.delim[1], h.delim[2],
               h.dl, flags, a, b);
    int32_t *src = nullptr, *dst = nullptr;
    if ((st = tmp.alloc(&src, (size_t)count * sizeof(int32_t)))) return st;
    if ((st = tmp.alloc(&dst, (size_t)count * sizeof(int32_t)))) return st;
    unsigned long long hs[10];
    auto read_stats = [&]() -> pgd_status {
        PGD_CUDA(ctx, cudaMemcpyAsync(hs, stats, sizeof(hs), cudaMemcpyDeviceToHost, s));
        PGD_CUDA(ctx, cudaStreamSynchronize(s));
        return PGD_OK;
    };
    int64_t npairs = 0;

    if (h.mtx) {
        // ---- mtx: ids minus one, no relabel, no dedup ----------------------
        PGD_LAUNCH(ctx, k_mtx_pass, grid_for(count), kThreads, 0, flags, a, b, count, keep, stats);
        if ((st = read_stats())) return st;
        if (hs[0]) {
            PGD_LAUNCH(ctx, k_seq_mtx, 1, 1, 0, flags, a, b, count, h.v, h.u, src, dst, stats);
            if ((st = read_stats())) return st;
            if (hs[5]) return pgd_fail(ctx, PGD_EINVAL, "vertex id < 1 in mtx file");
            npairs = (int64_t)hs[8];
        } else {
            if (hs[5]) return pgd_fail(ctx, PGD_EINVAL, "vertex id < 1 in mtx file");
            PGD_CUDA(ctx, cudaMemsetAsync(keep + count, 0, sizeof(uint32_t), s));
            if ((st = exclusive_scan(ctx, keep, kpos, count + 1))) return st;
            PGD_LAUNCH(ctx, k_emit_pairs, grid_for(count), kThreads, 0, keep, kpos, a, b, count, 1,
                       (const int32_t *)nullptr, src, dst);
            npairs = count - (int64_t)hs[4];
            uint32_t k32 = 0;
            PGD_CUDA(ctx, cudaMemcpyAsync(&k32, kpos + count, sizeof(k32), cudaMemcpyDeviceToHost, s));
            PGD_CUDA(ctx, cudaStreamSynchronize(s));
            npairs = k32;
        }
        st = pgd_build_from_device_pairs(g, src, dst, npairs, 0, false);
        g->self_loops = (int64_t)hs[4];
        return st;
    }

    // ---- edge list: pass 1 (ids, 0/1 base), pass 2 (relabel) ----------------
    const int64_t j0 = h.first_data ? 1 : 0;
    PGD_LAUNCH(ctx, k_edge_pass1, grid_for(count), kThreads, 0, flags, a, b, count, j0, stats);
    if ((st = read_stats())) return st;
    const bool sequential = hs[0] != 0;
    int fix = h.fix ? 1 : 0;
    int max_id = h.first_max;
    int v_carry = h.v, u_carry = h.u;
    if (sequential) {
        PGD_LAUNCH(ctx, k_seq_edge_pass1, 1, 1, 0, flags, a, b, count, j0, h.v, h.u, stats);
        if ((st = read_stats())) return st;
        if (hs[2]) return pgd_fail(ctx, PGD_EINVAL, "negative vertex id");
        if (hs[1]) fix = 0;
        max_id = std::max(max_id, (int)(unsigned)hs[3]);
        v_carry = (int)(unsigned)hs[6];
        u_carry = (int)(unsigned)hs[7];
    } else {
        if (hs[2]) return pgd_fail(ctx, PGD_EINVAL, "negative vertex id");
        if (hs[1]) fix = 0;
        max_id = std::max(max_id, (int)(unsigned)hs[3]);
    }
    int32_t *lookup = nullptr;
    if ((st = tmp.alloc(&lookup, ((size_t)max_id + 2) * sizeof(int32_t)))) return st;
    if (sequential) {
        PGD_CUDA(ctx, cudaMemsetAsync(lookup, 0xff, ((size_t)max_id + 2) * sizeof(int32_t), s));
        PGD_LAUNCH(ctx, k_seq_edge_pass2, 1, 1, 0, flags, a, b, count, v_carry, u_carry, fix, max_id, lookup, src,
                   dst, stats);
        if ((st = read_stats())) return st;
        if (hs[5]) return pgd_fail(ctx, PGD_EINVAL, "vertex id out of range");
        npairs = (int64_t)hs[8];
    } else {
        uint64_t *first = nullptr;
        uint32_t *pflag = nullptr, *prank = nullptr;
        if ((st = tmp.alloc(&first, ((size_t)max_id + 2) * sizeof(uint64_t)))) return st;
        if ((st = tmp.alloc(&pflag, (size_t)(2 * count + 1) * sizeof(uint32_t)))) return st;
        if ((st = tmp.alloc(&prank, (size_t)(2 * count + 1) * sizeof(uint32_t)))) return st;
        PGD_CUDA(ctx, cudaMemsetAsync(first, 0xff, ((size_t)max_id + 2) * sizeof(uint64_t), s));
        PGD_LAUNCH(ctx, k_edge_pass2, grid_for(count), kThreads, 0, flags, a, b, count, fix, max_id, first, keep,
                   stats);
        PGD_LAUNCH(ctx, k_first_flags, grid_for(count), kThreads, 0, keep, a, b, count, fix, first, pflag);
        PGD_CUDA(ctx, cudaMemsetAsync(pflag + 2 * count, 0, sizeof(uint32_t), s));
        if ((st = exclusive_scan(ctx, pflag, prank, 2 * count + 1))) return st;
        PGD_LAUNCH(ctx, k_relabel_table, grid_for(count), kThreads, 0, keep, a, b, count, fix, pflag, prank, lookup);
        PGD_CUDA(ctx, cudaMemsetAsync(keep + count, 0, sizeof(uint32_t), s));
        if ((st = exclusive_scan(ctx, keep, kpos, count + 1))) return st;
        PGD_LAUNCH(ctx, k_emit_pairs, grid_for(count), kThreads, 0, keep, kpos, a, b, count, fix,
                   (const int32_t *)lookup, src, dst);
        if ((st = read_stats())) return st;
        if (hs[5]) return pgd_fail(ctx, PGD_EINVAL, "vertex id out of range");
        uint32_t k32 = 0;
        PGD_CUDA(ctx, cudaMemcpyAsync(&k32, kpos + count, sizeof(k32), cudaMemcpyDeviceToHost, s));
        PGD_CUDA(ctx, cudaStreamSynchronize(s));
        npairs = k32;
    }
    st = pgd_build_from_device_pairs(g, src, dst, npairs, 0, true);
    g->self_loops = (int64_t)hs[4];
    return st;
}
