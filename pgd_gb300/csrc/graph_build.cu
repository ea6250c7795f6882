// graph_build.cu -- device-side graph construction and ordering.
//
// Replaces, on the GPU, the reference's host-side preparation of the graph:
//   read_* + remove_multiple_edges (graphlet_core.cpp:291-556)  -> pgd_build_from_pairs
//   the CSR constructor (graphlet_core.h:156-160)                -> pgd_build_from_csr
//   vertex_degrees (graphlet_core.cpp:877-891)                   -> k_degrees
//   order_vertex_neighbors + create_edge_list_arrays (:929-949, :1846-1953) -> pgd_dev_preprocess
//   compute_cores (:958-1018)                                    -> pgd_dev_cores (parallel peeling)
//   compute_assortativity (:1029-1057)                           -> pgd_dev_assortativity
//   sort_edges + get_ordering_value (:774-867)                   -> pgd_dev_sort_edges
//
// The compute CSR keeps every row sorted by neighbour id (what the
// decomposition kernels search).  The reference's own neighbour order only
// decides edge ids and hence the E_ordered tie-break; it is reproduced as a
// per-entry "insertion rank" and a segmented sort, never materialised.
#include <cub/cub.cuh>
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
// Edge-pair intake.

__global__ void k_pair_stats(const int32_t *src, const int32_t *dst, int64_t k, int *max_id,
                             unsigned long long *self_loops, unsigned long long *bad) {
    int local_max = -1;
    unsigned long long loops = 0, nbad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x) {
        int a = src[i], b = dst[i];
        if (a < 0 || b < 0) { nbad++; continue; }
        if (a == b) { loops++; continue; }
        local_max = max(local_max, max(a, b));
    }
    for (int o = 16; o > 0; o >>= 1) {
        local_max = max(local_max, __shfl_xor_sync(0xffffffffu, local_max, o));
        loops += __shfl_xor_sync(0xffffffffu, loops, o);
        nbad += __shfl_xor_sync(0xffffffffu, nbad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (local_max >= 0) atomicMax(max_id, local_max);
        if (loops) atomicAdd(self_loops, loops);
        if (nbad) atomicAdd(bad, nbad);
    }
}

// Pair i -> directed entries 2i (a->b) and 2i+1 (b->a), both carrying i as
// their insertion rank.  Self loops get a key that sorts after every edge.
__global__ void k_make_entries(const int32_t *src, const int32_t *dst, int64_t k, uint64_t sentinel,
                               uint64_t *keys, uint32_t *vals) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t a = (uint32_t)src[i], b = (uint32_t)dst[i];
        uint64_t k0 = sentinel, k1 = sentinel;
        if (a != b) {
            k0 = ((uint64_t)a << 32) | b;
            k1 = ((uint64_t)b << 32) | a;
        }
        keys[2 * i] = k0;
        keys[2 * i + 1] = k1;
        vals[2 * i] = (uint32_t)i;
        vals[2 * i + 1] = (uint32_t)i;
    }
}

// CSR input -> entries (row<<32 | col), rank = position in the input.
__global__ void k_csr_entries(const int64_t *off, const int32_t *adj, int64_t n, int64_t nnz, uint64_t *keys,
                              uint32_t *vals, unsigned long long *bad) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        // row of position j: last r with off[r] <= j
        int64_t lo = 0, hi = n;  // off[lo] <= j < off[hi]
        while (hi - lo > 1) {
            int64_t mid = (lo + hi) >> 1;
            if (off[mid] <= j) lo = mid; else hi = mid;
        }
        int32_t c = adj[j];
        if (c < 0 || c >= n || c == lo) atomicAdd(bad, 1ull);
        keys[j] = ((uint64_t)(uint32_t)lo << 32) | (uint32_t)c;
        vals[j] = (uint32_t)j;
    }
}

// first-of-run flags over the sorted valid prefix
__global__ void k_unique_flags(const uint64_t *keys, int64_t valid, uint32_t *flags) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < valid; i += (int64_t)gridDim.x * blockDim.x)
        flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

__global__ void k_scatter_unique(const uint64_t *keys, const uint32_t *vals, const uint32_t *flags,
                                 const uint32_t *pos, int64_t valid, int32_t *adj, int64_t *rank, int32_t *row) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < valid; i += (int64_t)gridDim.x * blockDim.x) {
        if (!flags[i]) continue;
        uint32_t p = pos[i];
        adj[p] = (int32_t)(uint32_t)(keys[i] & 0xffffffffu);
        row[p] = (int32_t)(keys[i] >> 32);
        rank[p] = vals[i];
    }
}

// off[r] = first entry of row r; rows without entries point at the next one.
__global__ void k_offsets(const int32_t *row, int64_t nnz, int64_t n, int64_t *off) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= nnz; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = (i < nnz) ? row[i] : n;
        int64_t rp = (i == 0) ? -1 : row[i - 1];
        for (int64_t x = rp + 1; x <= r; x++) off[x] = i;
    }
}

__global__ void k_degrees(const int64_t *off, int64_t n, int32_t *deg) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        deg[v] = (int32_t)(off[v + 1] - off[v]);
}

// Per-vertex sum over neighbours of f(x), one warp per vertex.
// mode 0: degree (2-hop volume), 1: kcore1, 2: degree * kcore1.
__global__ void k_neigh_sum(const int64_t *off, const int32_t *adj, const int32_t *deg, const int32_t *core,
                            int64_t n, int mode, uint64_t *out) {
    int lane = threadIdx.x & 31;
    int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = w; v < n; v += nw) {
        uint64_t s = 0;
        for (int64_t j = off[v] + lane; j < off[v + 1]; j += 32) {
            int32_t x = adj[j];
            long long d = deg[x];
            long long k1 = (mode == 0) ? 0 : (x >= 1 ? core[x - 1] : 0);
            s += (uint64_t)(mode == 0 ? d : (mode == 1 ? k1 : d * k1));
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[v] = s;
    }
}

// Symmetry check for CSR input: (r,c) needs (c,r).
__global__ void k_check_symmetric(const int64_t *off, const int32_t *adj, const int32_t *row, int64_t nnz,
                                  unsigned long long *bad) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        int32_t r = row[j], c = adj[j];
        int64_t lo = off[c], hi = off[c + 1];
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if (adj[mid] < r) lo = mid + 1; else hi = mid;
        }
        if (lo >= off[c + 1] || adj[lo] != r) atomicAdd(bad, 1ull);
    }
}

__global__ void k_rows_of(const int64_t *off, int64_t n, int64_t nnz, int32_t *row) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = n;
        while (hi - lo > 1) {
            int64_t mid = (lo + hi) >> 1;
            if (off[mid] <= j) lo = mid; else hi = mid;
        }
        row[j] = (int32_t)lo;
    }
}

// ---------------------------------------------------------------------------
// Neighbour order and edge ids.

// Composite within-row sort key: (neighbour key, insertion rank).  The
// reference's stable counting sort followed by a reversal
// (graphlet_core.cpp:1867-1875) orders a row by key descending with ties in
// reverse insertion order; --s2l_neigh keeps key ascending, ties in order.
__global__ void k_neigh_keys(const int32_t *adj, const int64_t *rank, const int32_t *deg, const int32_t *core,
                             int64_t nnz, int kind, uint64_t *keys, uint32_t *idx) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        int32_t c = adj[j];
        uint32_t key = 0;
        if (kind == PGD_NEIGH_DEG) key = (uint32_t)deg[c];
        else if (kind == PGD_NEIGH_KCORE) key = (uint32_t)(c >= 1 ? core[c - 1] : 0);
        keys[j] = ((uint64_t)key << 33) | (uint64_t)rank[j];
        idx[j] = (uint32_t)j;
    }
}

__global__ void k_edge_flags(const int32_t *row, const int32_t *adj, const uint32_t *perm, int64_t nnz,
                             uint32_t *flags) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        flags[j] = (row[j] < adj[perm[j]]) ? 1u : 0u;
}

// create_edge_list_arrays (graphlet_core.cpp:929-949): e_v is the endpoint
// with the smaller degree, ties go to the larger id.
__global__ void k_edge_arrays(const int32_t *row, const int32_t *adj, const int32_t *deg, const uint32_t *perm,
                              const uint32_t *flags, const uint32_t *ids, int64_t nnz, int32_t *ev, int32_t *eu) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        if (!flags[j]) continue;
        int32_t r = row[j], c = adj[perm[j]];
        uint32_t id = ids[j];
        if (deg[r] < deg[c]) { ev[id] = r; eu[id] = c; }
        else { ev[id] = c; eu[id] = r; }
    }
}

// ---------------------------------------------------------------------------
// k-core peeling.  core[v] = -1 while v is alive.

__global__ void k_core_init(const int32_t *deg, int64_t n, int32_t *cur, int32_t *core, int32_t *alive) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        cur[v] = deg[v];
        core[v] = -1;
        alive[v] = (int32_t)v;
    }
}

__global__ void k_max_core(const int32_t *core, int64_t n_minus_1, int *out) {
    int local = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n_minus_1; v += (int64_t)gridDim.x * blockDim.x)
        local = max(local, core[v]);
    for (int o = 16; o > 0; o >>= 1) local = max(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0 && local > 0) atomicMax(out, local);
}

// ---------------------------------------------------------------------------
// Assortativity: int degree products as in the reference, double sums in a
// fixed order (block partials, then one block), so the result is repeatable.

__global__ void k_assort_partial(const int32_t *ev, const int32_t *eu, const int32_t *deg, int64_t m,
                                 double *partial) {
    __shared__ double s[3][kThreads / 32];
    double mu = 0, jd = 0, psi = 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        unsigned dv = (unsigned)deg[ev[e]], du = (unsigned)deg[eu[e]];
        int p = (int)(dv * du);
        int q = (int)(dv * dv + du * du);
        mu += (double)p;
        jd += 0.5 * (double)(int)(dv + du);
        psi += 0.5 * (double)q;
    }
    for (int o = 16; o > 0; o >>= 1) {
        mu += __shfl_xor_sync(0xffffffffu, mu, o);
        jd += __shfl_xor_sync(0xffffffffu, jd, o);
        psi += __shfl_xor_sync(0xffffffffu, psi, o);
    }
    int wid = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { s[0][wid] = mu; s[1][wid] = jd; s[2][wid] = psi; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0;
        for (int i = 0; i < kThreads / 32; i++) t += s[threadIdx.x][i];
        partial[3 * blockIdx.x + threadIdx.x] = t;
    }
}

// ---------------------------------------------------------------------------
// Edge keys for sort_edges (graphlet_core.cpp:774-834).  The key is stored as
// int (Vertex, graphlet_vertex.h:42); order is key then id, id always
// descending (decr_bound / incr_bound, graphlet_vertex.h:57-75).

// Keys of the edges to order: every edge (ids == null, count == m) or the
// sampled edge ids ids[0..count) (sort_edges with E_s, graphlet_core.cpp:
// 836-851), whose natural key is the position in the sample.
__global__ void k_edge_keys(const int32_t *ev, const int32_t *eu, const int32_t *deg, const int32_t *core,
                            const uint64_t *vsum, const int32_t *ids, int64_t count, int kind, int s2l,
                            uint64_t *keys) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = ids ? ids[i] : i;
        int32_t v = ev[e], u = eu[e];
        long long val = i;
        // core[] exists only for the k-core keys
        const bool kc = kind == PGD_ORD_KCORE || kind == PGD_ORD_KCORE_DEG;
        int kv = (kc && v >= 1) ? core[v - 1] : 0, ku = (kc && u >= 1) ? core[u - 1] : 0;
        switch (kind) {
        case PGD_ORD_DEG: val = deg[u] + deg[v]; break;
        case PGD_ORD_KCORE: val = ku + kv; break;
        case PGD_ORD_KCORE_DEG: val = (int)((unsigned)(deg[u] + deg[v]) * (unsigned)(ku + kv)); break;
        case PGD_ORD_DEG_VOL:
        case PGD_ORD_KCORE_VOL:
        case PGD_ORD_KCORE_DEG_VOL: val = (long long)(vsum[u] + vsum[v]); break;
        case PGD_ORD_DEG_U: val = deg[u]; break;
        default: break;
        }
        uint32_t k32 = (uint32_t)(int32_t)val ^ 0x80000000u;
        uint32_t id = (uint32_t)e;
        keys[i] = ((uint64_t)k32 << 32) | (s2l ? (0xffffffffu - id) : id);
    }
}

__global__ void k_keys_to_ids(const uint64_t *keys, int64_t m, int s2l, int32_t *order) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        uint32_t lo = (uint32_t)(keys[e] & 0xffffffffu);
        order[e] = (int32_t)(s2l ? (0xffffffffu - lo) : lo);
    }
}

int bit_length(uint64_t x) {
    int b = 0;
    while (x) { b++; x >>= 1; }
    return b;
}

}  // namespace

// ---------------------------------------------------------------------------

static pgd_status finish_csr(pgd_graph *g, uint64_t *keys, uint32_t *vals, int64_t valid, bool dedup,
                             bool csr_input) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    uint32_t *flags = nullptr, *pos = nullptr;
    int32_t *row = nullptr;
    pgd_status st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&flags, (valid + 1) * sizeof(uint32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&pos, (valid + 1) * sizeof(uint32_t)))) return st;
    PGD_LAUNCH(ctx, k_unique_flags, grid_for(valid), kThreads, 0, keys, valid, flags);
    size_t tb = 0;
    void *tmp = nullptr;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, flags, pos, (int64_t)valid + 1, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    // flags[valid] is scratch: clear it so pos[valid] = number of unique
    PGD_CUDA(ctx, cudaMemsetAsync(flags + valid, 0, sizeof(uint32_t), s));
    cub::DeviceScan::ExclusiveSum(tmp, tb, flags, pos, (int64_t)valid + 1, s);
    pgd_tmp_free(ctx, tmp);
    uint32_t nnz32 = 0;
    PGD_CUDA(ctx, cudaMemcpyAsync(&nnz32, pos + valid, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    int64_t nnz = nnz32;
    if (nnz != valid) {
        if (!dedup) {
            pgd_tmp_free(ctx, flags); pgd_tmp_free(ctx, pos);
            return pgd_fail(ctx, PGD_EINVAL, csr_input ? "CSR row lists a neighbour twice"
                                                       : "repeated pair without PGD_EDGES_DEDUP (multigraph input)");
        }
        g->duplicates = (valid - nnz) / 2;
    }
    g->m = nnz / 2;
    if ((st = pgd_graph_alloc(g, (void **)&g->adj, (nnz + 1) * sizeof(int32_t)))) return st;
    if ((st = pgd_graph_alloc(g, (void **)&g->rank, (nnz + 1) * sizeof(int64_t)))) return st;
    if ((st = pgd_graph_alloc(g, (void **)&g->off, (g->n + 1) * sizeof(int64_t)))) return st;
    if ((st = pgd_graph_alloc(g, (void **)&g->deg, (g->n + 1) * sizeof(int32_t)))) return st;
    if ((st = pgd_graph_alloc(g, (void **)&g->vol2, (g->n + 1) * sizeof(uint64_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&row, (nnz + 1) * sizeof(int32_t)))) return st;
    PGD_LAUNCH(ctx, k_scatter_unique, grid_for(valid), kThreads, 0, keys, vals, flags, pos, valid, g->adj, g->rank, row);
    PGD_LAUNCH(ctx, k_offsets, grid_for(nnz + 1), kThreads, 0, row, nnz, g->n, g->off);
    PGD_LAUNCH(ctx, k_degrees, grid_for(g->n), kThreads, 0, g->off, g->n, g->deg);
    if (csr_input && nnz > 0) {
        unsigned long long *bad = ctx->d_ctr;
        PGD_CUDA(ctx, cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s));
        PGD_LAUNCH(ctx, k_check_symmetric, grid_for(nnz), kThreads, 0, g->off, g->adj, row, nnz, bad);
        unsigned long long h_bad = 0;
        PGD_CUDA(ctx, cudaMemcpyAsync(&h_bad, bad, sizeof(h_bad), cudaMemcpyDeviceToHost, s));
        PGD_CUDA(ctx, cudaStreamSynchronize(s));
        if (h_bad) {
            pgd_tmp_free(ctx, flags); pgd_tmp_free(ctx, pos); pgd_tmp_free(ctx, row);
            return pgd_fail(ctx, PGD_EINVAL, "CSR is not symmetric (undirected graphs list each edge both ways)");
        }
    }
    pgd_tmp_free(ctx, flags);
    pgd_tmp_free(ctx, pos);
    pgd_tmp_free(ctx, row);
    // max degree and 2-hop volumes
    int *d_max = (int *)ctx->d_ctr;
    PGD_CUDA(ctx, cudaMemsetAsync(d_max, 0, sizeof(int), s));
    if (g->n > 0) {
        size_t tb2 = 0;
        cub::DeviceReduce::Max(nullptr, tb2, g->deg, d_max, g->n, s);
        if ((st = pgd_tmp_alloc(ctx, &tmp, tb2))) return st;
        cub::DeviceReduce::Max(tmp, tb2, g->deg, d_max, g->n, s);
        pgd_tmp_free(ctx, tmp);
        PGD_LAUNCH(ctx, k_neigh_sum, grid_for(g->n * 32), kThreads, 0, g->off, g->adj, g->deg, nullptr, g->n, 0, g->vol2);
    }
    int h_max = 0;
    PGD_CUDA(ctx, cudaMemcpyAsync(&h_max, d_max, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    g->max_degree = h_max;
    PGD_CUDA(ctx, cudaGetLastError());
    return PGD_OK;
}

// 16-byte words from a mapped host source, then the tail bytes
__global__ void k_copy_mapped(const uint4 *src, uint4 *dst, int64_t n16, const uint8_t *src_tail, uint8_t *dst_tail,
                              int tail) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = src[i];
    if (blockIdx.x == 0 && threadIdx.x < tail) dst_tail[threadIdx.x] = src_tail[threadIdx.x];
}

cudaError_t pgd_h2d(pgd_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (!bytes) return cudaSuccess;
    const void *v = pgd_device_view(src);
    if (!v || ((uintptr_t)v & 15) || ((uintptr_t)dst & 15))
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
    const int64_t n16 = (int64_t)(bytes / 16);
    const int tail = (int)(bytes % 16);
    k_copy_mapped<<<ctx->num_sms * 8, kThreads, 0, ctx->stream>>>((const uint4 *)v, (uint4 *)dst, n16,
                                                                   (const uint8_t *)v + 16 * n16,
                                                                   (uint8_t *)dst + 16 * n16, tail);
    ctx->launches++;
    return cudaGetLastError();
}

pgd_status pgd_build_from_pairs(pgd_graph *g, const int32_t *h_src, const int32_t *h_dst, int64_t k, int64_t n_min,
                                bool dedup) {
    pgd_ctx *ctx = g->ctx;
    if (k < 0 || k > (int64_t)0x7fffffff) return pgd_fail(ctx, PGD_EINVAL, "pair count out of range (0..2^31-1)");
    pgd_status st;
    int32_t *d_src = nullptr, *d_dst = nullptr;
    const int64_t k1 = k > 0 ? k : 1;
    if ((st = pgd_tmp_alloc(ctx, (void **)&d_src, k1 * sizeof(int32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&d_dst, k1 * sizeof(int32_t)))) {
        pgd_tmp_free(ctx, d_src);
        return st;
    }
    cudaError_t e = cudaSuccess;
    if (k > 0) {
        e = pgd_h2d(ctx, d_src, h_src, k * sizeof(int32_t));
        if (e == cudaSuccess) e = pgd_h2d(ctx, d_dst, h_dst, k * sizeof(int32_t));
    }
    st = e == cudaSuccess ? pgd_build_from_device_pairs(g, d_src, d_dst, k, n_min, dedup)
                          : pgd_cuda_fail(ctx, e, "upload of the pairs");
    pgd_tmp_free(ctx, d_src);
    pgd_tmp_free(ctx, d_dst);
    return st;
}

pgd_status pgd_build_from_device_pairs(pgd_graph *g, const int32_t *d_src, const int32_t *d_dst, int64_t k,
                                       int64_t n_min, bool dedup) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    if (k < 0 || k > (int64_t)0x7fffffff) return pgd_fail(ctx, PGD_EINVAL, "pair count out of range (0..2^31-1)");
    pgd_status st;
    uint64_t *keys = nullptr, *keys2 = nullptr;
    uint32_t *vals = nullptr, *vals2 = nullptr;
    const int64_t k1 = k > 0 ? k : 1;
    // stats: [0] max id (int), [1] self loops, [2] bad ids
    unsigned long long *stats = ctx->d_ctr;
    PGD_CUDA(ctx, cudaMemsetAsync(stats, 0, 4 * sizeof(unsigned long long), s));
    PGD_CUDA(ctx, cudaMemsetAsync(stats, 0xff, sizeof(int), s));  // max id = -1
    if (k > 0)
        PGD_LAUNCH(ctx, k_pair_stats, grid_for(k), kThreads, 0, d_src, d_dst, k, (int *)stats, stats + 1, stats + 2);
    unsigned long long h_stats[3];
    PGD_CUDA(ctx, cudaMemcpyAsync(h_stats, stats, sizeof(h_stats), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    const int max_id = (int)(h_stats[0] & 0xffffffffu);
    if (h_stats[2]) return pgd_fail(ctx, PGD_EINVAL, "negative vertex id in edge list");
    g->self_loops = (int64_t)h_stats[1];
    g->n = std::max<int64_t>(n_min, (int64_t)max_id + 1);
    const int64_t valid = 2 * (k - g->self_loops);
    const int64_t ne = 2 * k1;
    if ((st = pgd_tmp_alloc(ctx, (void **)&keys, ne * sizeof(uint64_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&keys2, ne * sizeof(uint64_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&vals, ne * sizeof(uint32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&vals2, ne * sizeof(uint32_t)))) return st;
    const uint64_t sentinel = (uint64_t)(uint32_t)(max_id + 1) << 32;
    if (k > 0) PGD_LAUNCH(ctx, k_make_entries, grid_for(k), kThreads, 0, d_src, d_dst, k, sentinel, keys, vals);
    const int end_bit = 32 + bit_length((uint64_t)(max_id + 1));
    if (k > 0) {
        size_t tb = 0;
        void *tmp = nullptr;
        cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, keys2, vals, vals2, (int64_t)(2 * k), 0, end_bit, s);
        if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
        cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, vals2, (int64_t)(2 * k), 0, end_bit, s);
        pgd_tmp_free(ctx, tmp);
    }
    pgd_tmp_free(ctx, keys);
    pgd_tmp_free(ctx, vals);
    st = finish_csr(g, keys2, vals2, valid, dedup, false);
    pgd_tmp_free(ctx, keys2);
    pgd_tmp_free(ctx, vals2);
    return st;
}

pgd_status pgd_build_from_csr(pgd_graph *g, const int64_t *h_off, const int32_t *h_adj, int64_t n) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    if (n < 0 || n > (int64_t)0x7ffffffe) return pgd_fail(ctx, PGD_EINVAL, "vertex count out of range");
    if (h_off[0] != 0) return pgd_fail(ctx, PGD_EINVAL, "CSR offsets must start at 0");
    for (int64_t v = 0; v < n; v++)
        if (h_off[v + 1] < h_off[v]) return pgd_fail(ctx, PGD_EINVAL, "CSR offsets must not decrease");
    int64_t nnz = h_off[n];
    if (nnz > (int64_t)0x7fffffff) return pgd_fail(ctx, PGD_EINVAL, "too many CSR entries");
    g->n = n;
    pgd_status st;
    int64_t *d_off = nullptr;
    int32_t *d_adj = nullptr;
    uint64_t *keys = nullptr, *keys2 = nullptr;
    uint32_t *vals = nullptr, *vals2 = nullptr;
    int64_t nz1 = nnz > 0 ? nnz : 1;
    if ((st = pgd_tmp_alloc(ctx, (void **)&d_off, (n + 1) * sizeof(int64_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&d_adj, nz1 * sizeof(int32_t)))) return st;
    PGD_CUDA(ctx, cudaMemcpyAsync(d_off, h_off, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    if (nnz) PGD_CUDA(ctx, cudaMemcpyAsync(d_adj, h_adj, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    if ((st = pgd_tmp_alloc(ctx, (void **)&keys, nz1 * sizeof(uint64_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&keys2, nz1 * sizeof(uint64_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&vals, nz1 * sizeof(uint32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&vals2, nz1 * sizeof(uint32_t)))) return st;
    unsigned long long *bad = ctx->d_ctr;
    PGD_CUDA(ctx, cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s));
    if (nnz) PGD_LAUNCH(ctx, k_csr_entries, grid_for(nnz), kThreads, 0, d_off, d_adj, n, nnz, keys, vals, bad);
    unsigned long long h_bad = 0;
    PGD_CUDA(ctx, cudaMemcpyAsync(&h_bad, bad, sizeof(h_bad), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    pgd_tmp_free(ctx, d_off);
    pgd_tmp_free(ctx, d_adj);
    if (h_bad) {
        pgd_tmp_free(ctx, keys); pgd_tmp_free(ctx, keys2); pgd_tmp_free(ctx, vals); pgd_tmp_free(ctx, vals2);
        return pgd_fail(ctx, PGD_EINVAL, "CSR neighbour id out of range or a self loop");
    }
    if (nnz) {
        int end_bit = 32 + bit_length((uint64_t)n);
        size_t tb = 0;
        void *tmp = nullptr;
        cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, keys2, vals, vals2, nnz, 0, end_bit, s);
        if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
        cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, vals2, nnz, 0, end_bit, s);
        pgd_tmp_free(ctx, tmp);
    }
    pgd_tmp_free(ctx, keys);
    pgd_tmp_free(ctx, vals);
    st = finish_csr(g, keys2, vals2, nnz, false, true);
    pgd_tmp_free(ctx, keys2);
    pgd_tmp_free(ctx, vals2);
    return st;
}

pgd_status pgd_dev_preprocess(pgd_graph *g, int neigh_kind, int s2l) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    int64_t nnz = 2 * g->m;
    if (!g->ev) {
        if ((st = pgd_graph_alloc(g, (void **)&g->ev, (g->m + 1) * sizeof(int32_t)))) return st;
        if ((st = pgd_graph_alloc(g, (void **)&g->eu, (g->m + 1) * sizeof(int32_t)))) return st;
    }
    if (nnz == 0) { g->preprocessed = true; return PGD_OK; }
    int32_t *row = nullptr;
    uint64_t *keys = nullptr, *keys2 = nullptr;
    uint32_t *idx = nullptr, *perm = nullptr, *flags = nullptr, *ids = nullptr;
    if ((st = pgd_tmp_alloc(ctx, (void **)&row, nnz * sizeof(int32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&keys, nnz * sizeof(uint64_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&keys2, nnz * sizeof(uint64_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&idx, nnz * sizeof(uint32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&perm, nnz * sizeof(uint32_t)))) return st;
    PGD_LAUNCH(ctx, k_rows_of, grid_for(nnz), kThreads, 0, g->off, g->n, nnz, row);
    PGD_LAUNCH(ctx, k_neigh_keys, grid_for(nnz), kThreads, 0, g->adj, g->rank, g->deg, g->core, nnz, neigh_kind, keys, idx);
    bool descending = (neigh_kind != PGD_NEIGH_ASREAD) && !s2l;
    size_t tb = 0;
    void *tmp = nullptr;
    if (descending)
        cub::DeviceSegmentedSort::SortPairsDescending(nullptr, tb, keys, keys2, idx, perm, nnz, g->n, g->off,
                                                      g->off + 1, s);
    else
        cub::DeviceSegmentedSort::SortPairs(nullptr, tb, keys, keys2, idx, perm, nnz, g->n, g->off, g->off + 1, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    if (descending)
        cub::DeviceSegmentedSort::SortPairsDescending(tmp, tb, keys, keys2, idx, perm, nnz, g->n, g->off,
                                                      g->off + 1, s);
    else
        cub::DeviceSegmentedSort::SortPairs(tmp, tb, keys, keys2, idx, perm, nnz, g->n, g->off, g->off + 1, s);
    pgd_tmp_free(ctx, tmp);
    pgd_tmp_free(ctx, keys);
    pgd_tmp_free(ctx, keys2);
    pgd_tmp_free(ctx, idx);
    if ((st = pgd_tmp_alloc(ctx, (void **)&flags, nnz * sizeof(uint32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&ids, nnz * sizeof(uint32_t)))) return st;
    PGD_LAUNCH(ctx, k_edge_flags, grid_for(nnz), kThreads, 0, row, g->adj, perm, nnz, flags);
    tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, flags, ids, nnz, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    cub::DeviceScan::ExclusiveSum(tmp, tb, flags, ids, nnz, s);
    pgd_tmp_free(ctx, tmp);
    PGD_LAUNCH(ctx, k_edge_arrays, grid_for(nnz), kThreads, 0, row, g->adj, g->deg, perm, flags, ids, nnz, g->ev, g->eu);
    pgd_tmp_free(ctx, row);
    pgd_tmp_free(ctx, perm);
    pgd_tmp_free(ctx, flags);
    pgd_tmp_free(ctx, ids);
    PGD_CUDA(ctx, cudaGetLastError());
    g->preprocessed = true;
    g->sorted = false;
    g->has_micro = false;
    return PGD_OK;
}

// Device-driven peeling: the state machine below replaces a host loop with
// one round trip per level and per peel round.  Each step is a work kernel
// (a level scan or a peel round, chosen from the state) and a one-thread
// control kernel that applies the transition; a block of kCoreSteps steps is
// captured once as a CUDA graph and replayed until the control kernel
// reports that every vertex has a core number.  A level scan reads only the
// vertices still alive at the previous scan (a compacted list, rewritten by
// each scan), so the scans shrink as the peeling goes inward.
namespace {

struct CoreState {
    int level, mode, sel, done, failed, min_rest;
    unsigned int cnt[2];          // frontier sizes of buffers 0 and 1
    long long removed, steps, max_steps;
    int asel;                     // alive list read by the next scan
    unsigned int acnt[2];         // alive list sizes
};

constexpr int kCoreSteps = 64;
enum { kCoreScan = 0, kCorePeel = 1 };

__global__ void k_core_work(const int64_t *off, const int32_t *adj, int32_t *cur, int32_t *core, int64_t n,
                            int32_t *f0, int32_t *f1, int32_t *a0, int32_t *a1, CoreState *st) {
    if (st->done) return;
    const int mode = st->mode, level = st->level, sel = st->sel;
    int32_t *fin = sel ? f1 : f0, *fout = sel ? f0 : f1;
    if (mode == kCoreScan) {
        // every alive vertex with cur <= level leaves now; the others are
        // kept in the next alive list, and the smallest cur among them lets
        // the control kernel skip empty levels
        const int asel = st->asel;
        const int32_t *ain = asel ? a1 : a0;
        int32_t *aout = asel ? a0 : a1;
        const unsigned int na = st->acnt[asel];
        int local_min = INT_MAX;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < na; i += (int64_t)gridDim.x * blockDim.x) {
            const int32_t v = ain[i];
            if (core[v] != -1) continue;
            const int c = cur[v];
            if (c <= level) {
                core[v] = level;
                fin[atomicAdd(&st->cnt[sel], 1u)] = v;
            } else {
                local_min = min(local_min, c);
                aout[atomicAdd(&st->acnt[asel ^ 1], 1u)] = v;
            }
        }
        for (int o = 16; o > 0; o >>= 1) local_min = min(local_min, __shfl_xor_sync(0xffffffffu, local_min, o));
        if ((threadIdx.x & 31) == 0 && local_min != INT_MAX) atomicMin(&st->min_rest, local_min);
    } else {
        // remove the frontier: each alive neighbour loses one; the one whose
        // count drops to `level` joins the next frontier (one warp per vertex)
        const int lane = threadIdx.x & 31;
        const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
        const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
        const unsigned int fsize = st->cnt[sel];
        for (int64_t f = w; f < fsize; f += nw) {
            const int32_t v = fin[f];
            for (int64_t j = off[v] + lane; j < off[v + 1]; j += 32) {
                const int32_t x = adj[j];
                if (core[x] != -1) continue;
                const int old = atomicSub(&cur[x], 1);
                if (old == level + 1) {
                    core[x] = level;
                    fout[atomicAdd(&st->cnt[sel ^ 1], 1u)] = x;
                }
            }
        }
    }
}

__global__ void k_core_ctrl(CoreState *st, int64_t n) {
    if (st->done) return;
    const int sel = st->sel;
    if (st->mode == kCoreScan) {
        // the scan's survivors are the next alive list
        st->asel ^= 1;
        st->acnt[st->asel ^ 1] = 0;
        const unsigned int f = st->cnt[sel];
        if (f == 0) {
            // nobody at this level: jump to the smallest remaining count
            st->level = max(st->level + 1, st->min_rest);
            st->min_rest = INT_MAX;
        } else {
            st->removed += f;
            st->mode = kCorePeel;
            st->cnt[sel ^ 1] = 0;
        }
    } else {
        const unsigned int nf = st->cnt[sel ^ 1];
        st->removed += nf;
        if (nf == 0) {
            st->level += 1;
            st->mode = kCoreScan;
            st->cnt[sel] = 0;
            st->min_rest = INT_MAX;
        } else {
            st->sel = sel ^ 1;
            st->cnt[sel] = 0;   // the buffer written next
        }
    }
    st->steps += 1;
    if (st->removed >= n) st->done = 1;
    else if (st->steps >= st->max_steps) {
        st->done = 1;
        st->failed = 1;
    }
}

}  // namespace

pgd_status pgd_dev_cores(pgd_graph *g) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    int64_t n = g->n;
    if (!g->core) {
        if ((st = pgd_graph_alloc(g, (void **)&g->core, (n + 1) * sizeof(int32_t)))) return st;
    }
    if (n == 0) { g->has_cores = true; g->max_core = 0; return PGD_OK; }
    int32_t *cur = nullptr, *fa = nullptr, *fb = nullptr, *aa = nullptr, *ab = nullptr;
    CoreState *d_st = nullptr;
    if ((st = pgd_tmp_alloc(ctx, (void **)&cur, n * sizeof(int32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&fa, n * sizeof(int32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&fb, n * sizeof(int32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&aa, n * sizeof(int32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&ab, n * sizeof(int32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&d_st, sizeof(CoreState)))) return st;
    auto release = [&]() {
        pgd_tmp_free(ctx, cur);
        pgd_tmp_free(ctx, fa);
        pgd_tmp_free(ctx, fb);
        pgd_tmp_free(ctx, aa);
        pgd_tmp_free(ctx, ab);
        pgd_tmp_free(ctx, d_st);
    };
    PGD_LAUNCH(ctx, k_core_init, grid_for(n), kThreads, 0, g->deg, n, cur, g->core, aa);
    // every step removes a vertex or raises the level (at most max_degree + 1
    // levels), so 2 (n + max_degree) + 4 steps always suffice
    CoreState h{};
    h.min_rest = INT_MAX;
    h.max_steps = 2 * (n + (long long)g->max_degree) + 4;
    h.asel = 0;
    h.acnt[0] = (unsigned int)n;   // every vertex alive at the first scan
    h.acnt[1] = 0;
    PGD_CUDA(ctx, cudaMemcpyAsync(d_st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    const int work_grid = grid_for(32 * (int64_t)ctx->num_sms * 64);
    // capture kCoreSteps steps once, replay until done
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (int i = 0; i < kCoreSteps; i++) {
            k_core_work<<<work_grid, kThreads, 0, s>>>(g->off, g->adj, cur, g->core, n, fa, fb, aa, ab, d_st);
            k_core_ctrl<<<1, 1, 0, s>>>(d_st, n);
        }
        e = cudaStreamEndCapture(s, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        release();
        return pgd_cuda_fail(ctx, e, "k-core step graph");
    }
    int done = 0;
    while (!done) {
        e = cudaGraphLaunch(exec, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&done, &d_st->done, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) break;
        ctx->launches += 2 * kCoreSteps;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        release();
        return pgd_cuda_fail(ctx, e, "k-core peeling");
    }
    PGD_CUDA(ctx, cudaMemcpyAsync(&h, d_st, sizeof(h), cudaMemcpyDeviceToHost, s));
    int *d_mc = (int *)d_st;
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    if (h.failed) {
        release();
        return pgd_fail(ctx, PGD_EINVAL, "k-core peeling did not converge");
    }
    PGD_CUDA(ctx, cudaMemsetAsync(d_mc, 0, sizeof(int), s));
    if (n > 1) PGD_LAUNCH(ctx, k_max_core, grid_for(n - 1), kThreads, 0, g->core, n - 1, d_mc);
    int mc = 0;
    PGD_CUDA(ctx, cudaMemcpyAsync(&mc, d_mc, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    release();
    PGD_CUDA(ctx, cudaGetLastError());
    g->max_core = mc;
    g->has_cores = true;
    return PGD_OK;
}

pgd_status pgd_dev_assortativity(pgd_graph *g, double *r) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    int64_t m = g->m;
    int blocks = grid_for(m, kThreads, 4 * ctx->num_sms);
    double *partial = nullptr;
    if ((st = pgd_tmp_alloc(ctx, (void **)&partial, 3 * blocks * sizeof(double)))) return st;
    PGD_LAUNCH(ctx, k_assort_partial, blocks, kThreads, 0, g->ev, g->eu, g->deg, m, partial);
    double *h = (double *)malloc(3 * blocks * sizeof(double));
    PGD_CUDA(ctx, cudaMemcpyAsync(h, partial, 3 * blocks * sizeof(double), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    pgd_tmp_free(ctx, partial);
    double mu = 0, jd = 0, psi = 0;
    for (int b = 0; b < blocks; b++) { mu += h[3 * b]; jd += h[3 * b + 1]; psi += h[3 * b + 2]; }
    free(h);
    double dm = (double)m;
    double tau = (jd / dm) * (jd / dm);
    double rr = ((mu / dm) - tau) / ((psi / dm) - tau);
    // The reference's isnan() guard is compiled out by -ffast-math
    // (graphlet_core.cpp:1054), so a NaN stays NaN; the range check cannot
    // fire on NaN either.
    if (rr < -1 || rr > 1.0) rr = 1;
    if (m == 0) rr = 0.0;
    *r = rr;
    return PGD_OK;
}

// Orders every edge (d_ids == null, count == m) or the sample d_ids[0..count)
// (device array of edge ids in [0, m)); E_ordered gets count entries.
static pgd_status sort_edges_impl(pgd_graph *g, int kind, int s2l, const int32_t *d_ids, int64_t count) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    int64_t m = g->m;
    if (!g->order) {
        if ((st = pgd_graph_alloc(g, (void **)&g->order, (m + 1) * sizeof(int32_t)))) return st;
    }
    g->sorted = false;
    g->has_micro = false;
    g->norder = count;
    if (count == 0) { g->sorted = true; return PGD_OK; }
    uint64_t *vsum = nullptr;
    if (kind == PGD_ORD_DEG_VOL) {
        vsum = g->vol2;
    } else if (kind == PGD_ORD_KCORE_VOL || kind == PGD_ORD_KCORE_DEG_VOL) {
        if ((st = pgd_tmp_alloc(ctx, (void **)&vsum, g->n * sizeof(uint64_t)))) return st;
        PGD_LAUNCH(ctx, k_neigh_sum, grid_for(g->n * 32), kThreads, 0, g->off, g->adj, g->deg, g->core, g->n,
                                                              kind == PGD_ORD_KCORE_VOL ? 1 : 2, vsum);
    }
    uint64_t *keys = nullptr, *keys2 = nullptr;
    if ((st = pgd_tmp_alloc(ctx, (void **)&keys, count * sizeof(uint64_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&keys2, count * sizeof(uint64_t)))) return st;
    PGD_LAUNCH(ctx, k_edge_keys, grid_for(count), kThreads, 0, g->ev, g->eu, g->deg, g->core, vsum, d_ids, count, kind,
               s2l, keys);
    size_t tb = 0;
    void *tmp = nullptr;
    if (s2l) cub::DeviceRadixSort::SortKeys(nullptr, tb, keys, keys2, count, 0, 64, s);
    else cub::DeviceRadixSort::SortKeysDescending(nullptr, tb, keys, keys2, count, 0, 64, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    if (s2l) cub::DeviceRadixSort::SortKeys(tmp, tb, keys, keys2, count, 0, 64, s);
    else cub::DeviceRadixSort::SortKeysDescending(tmp, tb, keys, keys2, count, 0, 64, s);
    pgd_tmp_free(ctx, tmp);
    PGD_LAUNCH(ctx, k_keys_to_ids, grid_for(count), kThreads, 0, keys2, count, s2l, g->order);
    pgd_tmp_free(ctx, keys);
    pgd_tmp_free(ctx, keys2);
    if (vsum && vsum != g->vol2) pgd_tmp_free(ctx, vsum);
    PGD_CUDA(ctx, cudaGetLastError());
    g->sorted = true;
    return PGD_OK;
}

pgd_status pgd_dev_sort_edges(pgd_graph *g, int kind, int s2l) { return sort_edges_impl(g, kind, s2l, nullptr, g->m); }

pgd_status pgd_dev_sort_edges_sample(pgd_graph *g, int kind, int s2l, const int64_t *h_ids, int64_t k) {
    pgd_ctx *ctx = g->ctx;
    pgd_status st;
    if (k < 0 || k > g->m) return pgd_fail(ctx, PGD_EINVAL, "sample size must be between 0 and m");
    for (int64_t i = 0; i < k; i++)
        if (h_ids[i] < 0 || h_ids[i] >= g->m) return pgd_fail(ctx, PGD_EINVAL, "sampled edge id out of range");
    std::vector<int32_t> ids32((size_t)k + 1);
    for (int64_t i = 0; i < k; i++) ids32[(size_t)i] = (int32_t)h_ids[i];
    int32_t *d_ids = nullptr;
    if ((st = pgd_tmp_alloc(ctx, (void **)&d_ids, (k + 1) * sizeof(int32_t)))) return st;
    cudaError_t e = cudaMemcpyAsync(d_ids, ids32.data(), k * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);   // ids32 is a host temporary
    if (e != cudaSuccess) {
        pgd_tmp_free(ctx, d_ids);
        return pgd_cuda_fail(ctx, e, "copy of the sampled edge ids");
    }
    st = sort_edges_impl(g, kind, s2l, d_ids, k);
    pgd_tmp_free(ctx, d_ids);
    return st;
}

// ---------------------------------------------------------------------------
// Row ids of the per-edge output (the writer's id+1 convention,
// graphlet_core.cpp:1694-1701): row e is edge order[e].

__global__ void k_micro_ids(const int32_t *ev, const int32_t *eu, const int32_t *order, int64_t m, int64_t *src1,
                            int64_t *dst1) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t id = order[e];
        if (src1) src1[e] = (int64_t)ev[id] + 1;
        if (dst1) dst1[e] = (int64_t)eu[id] + 1;
    }
}

// The per-edge rows and their ids written straight into host memory that the
// device can address (page-locked and mapped): one pass of every SM over the
// host link, 16-byte stores.  Any of the three outputs may be null.
__global__ void k_micro_out(const uint4 *micro, const int32_t *ev, const int32_t *eu, const int32_t *order,
                            int64_t m, uint4 *cols, int64_t *src1, int64_t *dst1) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (cols)   // a row is 8 x 8 bytes = 4 x 16 bytes
        for (int64_t i = t0; i < m * (PGD_NMICRO / 2); i += stride) cols[i] = micro[i];
    if (src1 || dst1)
        for (int64_t e = t0; e < m; e += stride) {
            const int32_t id = order[e];
            if (src1) src1[e] = (int64_t)ev[id] + 1;
            if (dst1) dst1[e] = (int64_t)eu[id] + 1;
        }
}

pgd_status pgd_dev_micro_out(pgd_graph *g, uint64_t *cols, int64_t *src1, int64_t *dst1) {
    pgd_ctx *ctx = g->ctx;
    if (g->norder > 0)
        PGD_LAUNCH(ctx, k_micro_out, ctx->num_sms * 8, kThreads, 0, (const uint4 *)g->micro, g->ev, g->eu, g->order,
                   g->norder, (uint4 *)cols, src1, dst1);
    PGD_CUDA(ctx, cudaGetLastError());
    return PGD_OK;
}

pgd_status pgd_dev_micro_ids(pgd_graph *g, int64_t *d_src1, int64_t *d_dst1) {
    pgd_ctx *ctx = g->ctx;
    if (g->norder > 0)
        PGD_LAUNCH(ctx, k_micro_ids, grid_for(g->norder), kThreads, 0, g->ev, g->eu, g->order, g->norder, d_src1, d_dst1);
    PGD_CUDA(ctx, cudaGetLastError());
    return PGD_OK;
}
