// decompose.cu -- the per-edge graphlet decomposition kernels.
//
// Replaces the OpenMP edge loop of graphlet_decomposition[_micro]
// (graphlet_core.cpp:1408-1424 and :1549-1577) and its helpers
// mark_neighbors / triangles_and_wedges / cycle / clique (:1069-1240),
// solve_graphlet_equations (:1326-1364) and the serial thread-sum reduction
// (:1431-1448).  Results are identical to the reference's; only the way the
// per-edge numbers are obtained differs.
//
// Per edge e the reference needs
//   t   = |T|, T = N(u) n N(v)              (triangles through e)
//   k4  = #edges inside T                   (4-cliques through e)
//   c4  = #edges between S_u and S_v        (induced 4-cycles through e),
//         S_u = N(u) \ T \ {v}, S_v = N(v) \ T \ {u}
// and it scans N(w) for every w in S_u u T.  On power-law graphs that rescans
// the lists of the same hubs for every edge that touches them.  Here every
// edge is handed to its anchor p, the endpoint of higher (degree, id), and
// the other endpoint q is scanned:
//   * c4 comes from an exact identity.  With W(w,p) = |N(w) n N(p)| and
//     t(x,q) the triangle count of edge (x,q),
//        c4 = sum_{w in S_q} W(w,p) - |S_q| - sum_{x in T} t(x,q) + 2*k4 + t,
//     because |N(w) n S_p| = W(w,p) - |N(w) n T| - 1 for w in S_q, and the
//     edges between S_q and T number sum_{x in T} t(x,q) - 2*k4 - t.
//     W(w,p) of every hub w comes from one histogram per anchor (the hub
//     neighbours of N(p), counted), not from a scan of N(w) per edge; t(x,q)
//     is read from a per-slot array filled by a triangle pass.
//   * k4 counts each edge inside T once, from its lower endpoint, as
//     |N+(x) n T| for every x in T, with N+(x) the degree-oriented list
//     (neighbours of higher degree).  For the highest-ranked x, N+(x) is also
//     kept as a bitmap over degree ranks, and |N+(x) n T| is AND + popc of
//     that row with T's rank bitmap whenever the row is shorter than the list.
// Anchors of degree >= kAnchorHub are processed by one CTA per (anchor,
// edge chunk) with N(p) as a bitmap in shared memory (or in a per-CTA global
// slice when n does not fit); the others by one warp per edge with N(p)
// staged and labelled in shared memory.  Every scan is flattened over the
// warp (one list entry per lane, owner found by a 5-step search over the
// warp's prefix sums), so short and long lists keep all lanes busy.
//
// All per-edge arithmetic is integer; the reference's "/ 2.0" round trips
// are reproduced with explicitly rounded double intrinsics.  Partial sums
// are uint64 and wrap exactly like the reference's (addition mod 2^64 is
// order independent, so the reduction order does not matter).
#include <string.h>

#include <cub/cub.cuh>
#include <mutex>
#include <string>
#include <vector>

#include "pgd_internal.h"
#include "pgd_kernels.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kHubWarps = 32;            // hub-anchor CTA: 1024 threads (latency-bound gathers want warps)
constexpr int kLightWarps = 8;           // light path: 256 threads, one edge per warp
constexpr int kAnchorHub = 128;          // default: anchors of degree >= this take the bitmap path
constexpr int kCacheHub = 64;            // allocation-free path: W(w,p) from the histogram for degree >= this
constexpr int kWideHub = 256;            // hubs of lower degree get 8-bit histogram counters (W(w,p) <= degree)
constexpr int kLightStageMax = 256;      // largest warp/block threshold the light path can stage
constexpr int kChunk = 8192;             // edges of one anchor per CTA work item (target; measured
                                         // 2048: +9 %, 6144-12288: flat)
constexpr int kMaxChunks = 8;            // ... but an anchor is split into at most this many items, since
                                         // every item rebuilds the anchor's bitmap and W histogram
constexpr int kMaxDynSmem = 156 * 1024;  // k_hub dynamic shared memory: bitmap, then the W histogram
constexpr int kMaxTslotSmem = 200 * 1024;  // k_tslot_hub dynamic shared memory: rank bitmap
constexpr int kTHigh = 4096;             // T members of rank >= kRankBits listed per warp (beyond: search N(q))
constexpr int kTWin = 1 << 18;           // T members of rank in [kRankBits, kTWin) also marked in a per-warp
                                         // global bitmap (30 KB), so membership there is one load
constexpr int kRankBits = 16384;         // T members of degree rank below this are marked in a per-warp bitmap;
                                         // vertices of rank below this get a rank-bitmap row of N+(x)

inline int grid_for(int64_t n, int per_block = kThreads, int cap = 1 << 20) {
    int64_t g = (n + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

struct DevGraph {
    const int64_t *off;
    const int32_t *adj;
    const int32_t *deg;
    const int64_t *offp;
    const int32_t *adjp;
    const int32_t *hubid;
    const int32_t *adj_rank;    // vrank of each adjacency entry
    const int4 *slot;           // per adjacency slot: {w, vrank(w) | row flag << 31, hubid(w), t of the slot's edge}
    const int32_t *ev;
    const int32_t *eu;
    const int32_t *order;
    long long n, m;
    long long npos;             // E_ordered positions to decompose: m, or the sample size
    uint64_t *micro;
    unsigned long long *sums;   // PGD_NSUMS, or PGD_NSUMS per graph when batched
    const int32_t *egraph;      // batched: graph of each E_ordered position, else null
    const long long *gnm;       // batched: n and m of each graph
    const uint8_t *gdense;      // batched: graph decomposed by the row-bitset kernel
    const int32_t *vrank;       // rank of each vertex by (degree desc, id desc)
    const int32_t *adjp_rank;   // vrank of each entry of adjp
    const int64_t *offh;        // hub-neighbour lists (hub ids)
    const int32_t *adjh;
    const uint32_t *toprows;    // rank-bitmap rows of N+(x) for vertices of rank < top_r
    const int4 *vrec;           // per vertex, 32 B: {off, offp} then {deg, |N+|, vrank, hubid}
    int top_r;
    int anchor_hub;             // anchors of degree >= this take the bitmap path
};

// Graph of a union id: last g in [0, k) with base[g] <= x (base non-decreasing).
__device__ __forceinline__ int batch_find(const int64_t *base, int k, int64_t x) {
    int lo = 0, hi = k;  // last g with base[g] <= x
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (base[mid] <= x) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool dense_edge(const DevGraph &G, int64_t e) {
    return G.gdense && G.gdense[G.egraph[e]];
}

__device__ __forceinline__ bool ranks_above(int32_t a, int32_t b, const int32_t *deg) {
    int da = deg[a], db = deg[b];
    return da > db || (da == db && a > b);
}

// ---------------------------------------------------------------------------
// per-graph structures

__global__ void k_rows(const int64_t *off, int64_t n, int64_t nnz, int32_t *row) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = n;
        while (hi - lo > 1) {
            int64_t mid = (lo + hi) >> 1;
            if (off[mid] <= j) lo = mid; else hi = mid;
        }
        row[j] = (int32_t)lo;
    }
}

__global__ void k_oriented_flags(const int32_t *row, const int32_t *adj, const int32_t *deg, int64_t nnz,
                                 uint32_t *flag) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        flag[j] = ranks_above(adj[j], row[j], deg) ? 1u : 0u;
}

__global__ void k_oriented_fill(const int64_t *off, const int32_t *adj, const uint32_t *flag, const uint32_t *pos,
                                int64_t n, int64_t nnz, int64_t *offp, int32_t *adjp) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        if (flag[j]) adjp[pos[j]] = adj[j];
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v <= n; v += (int64_t)gridDim.x * blockDim.x)
        offp[v] = pos[v < n ? off[v] : nnz];
}

// degree rank: position in the order (degree descending, id descending), so
// that vrank[a] < vrank[b] exactly when ranks_above(a, b): every entry of
// N+(x) has a smaller rank than x
__global__ void k_rank_keys(const int32_t *deg, int64_t n, uint64_t *keys) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        keys[v] = ((uint64_t)(uint32_t)(0x7fffffff - deg[v]) << 32) | (uint32_t)(0x7fffffff - v);
}

__global__ void k_rank_scatter(const uint64_t *sorted, int64_t n, int32_t *vrank) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        vrank[0x7fffffff - (uint32_t)(sorted[i] & 0xffffffffu)] = (int32_t)i;
}

// Hub-neighbour lists: for every vertex the hub ids of its neighbours that
// are hubs, in list order.
__global__ void k_hubnb_flags(const int32_t *adj, const int32_t *hubid, int64_t nnz, uint32_t *flag) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        flag[j] = hubid[adj[j]] >= 0 ? 1u : 0u;
}

__global__ void k_hubnb_fill(const int64_t *off, const int32_t *adj, const int32_t *hubid, const uint32_t *flag,
                             const uint32_t *pos, int64_t n, int64_t nnz, int64_t *offh, int32_t *adjh) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        if (flag[j]) adjh[pos[j]] = hubid[adj[j]];
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v <= n; v += (int64_t)gridDim.x * blockDim.x)
        offh[v] = pos[v < n ? off[v] : nnz];
}

__global__ void k_gather_rank(const int32_t *adjp, const int32_t *vrank, int64_t m, int32_t *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = vrank[adjp[i]];
}

// Rank-bitmap rows: the vertex of rank r < top_r gets a row of (r >> 6) + 1
// 64-bit words (2 ((r >> 6) + 1) 32-bit words) with bit r_y set for every y in
// N+(x) (all of rank < r).  Rows are stored back to back in rank order, each
// 8-byte aligned: row r starts at 64-bit word sum_{r' < r} ((r' >> 6) + 1) =
// (a + 1) * (32 a + b) for r = 64 a + b; returned here in 32-bit words.
__host__ __device__ __forceinline__ int64_t top_row_base(int64_t r) {
    const int64_t a = r >> 6, b = r & 63;
    return 2 * (a + 1) * (32 * a + b);
}

// 32-bit words of row r
__host__ __device__ __forceinline__ int top_row_words(int32_t r) { return 2 * ((r >> 6) + 1); }

__global__ void k_top_rows(const int64_t *offp, const int32_t *adjp_rank, const int32_t *vrank, int64_t n, int top_r,
                           uint32_t *rows) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t x = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; x < n; x += nw) {
        const int32_t r = vrank[x];
        if (r >= top_r) continue;
        uint32_t *row = rows + top_row_base(r);
        for (int64_t j = offp[x] + lane; j < offp[x + 1]; j += 32) {
            const int32_t ry = adjp_rank[j];
            if (ry < r) atomicOr(row + (ry >> 5), 1u << (ry & 31));
        }
    }
}

// One 32-byte record per vertex with what a scan of N(q) needs to know about
// each neighbour w, so that one sector load replaces six dependent ones.
__global__ void k_vrec(const int64_t *off, const int64_t *offp, const int32_t *deg, const int32_t *vrank,
                       const int32_t *hubid, int64_t n, int4 *vrec) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = off[v], op = offp[v];
        vrec[2 * v] = make_int4((int)(uint32_t)o, (int)(o >> 32), (int)(uint32_t)op, (int)(op >> 32));
        vrec[2 * v + 1] = make_int4(deg[v], (int)(offp[v + 1] - op), vrank[v], hubid[v]);
    }
}

// Per adjacency slot j (entry w = adj[j]): {w, vrank(w), hubid(w), t}, with
// bit 31 of the rank set when |N+(w) n T| is taken from w's rank-bitmap row
// (rank below top_r and the row shorter than N+(w)).  t is filled by k_tslot.
__global__ void k_slot_fill(const int32_t *adj, const int32_t *vrank, const int32_t *hubid, const int64_t *offp,
                            int64_t nnz, int top_r, int4 *slot) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t w = adj[j], r = vrank[w];
        const bool row = r < top_r && top_row_words(r) < (int)(offp[w + 1] - offp[w]);
        slot[j] = make_int4(w, (int)((uint32_t)r | (row ? 0x80000000u : 0u)), hubid[w], 0);
    }
}

__global__ void k_hub_flags(const int32_t *deg, int64_t n, int cache_hub, uint32_t *flag) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        flag[v] = deg[v] >= cache_hub ? 1u : 0u;
}

__global__ void k_hub_ids(const uint32_t *flag, const uint32_t *pos, int64_t n, int32_t *hubid) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        hubid[v] = flag[v] ? (int32_t)pos[v] : -1;
}

// Hub ids in two tiers of the W histogram: vertices of degree >= wide (16- or
// 32-bit counters) get ids 0..nA-1, those of degree in [cache_hub, wide)
// (8-bit counters: W(w,p) <= deg(w) < 256) get nA.. in id order.
__global__ void k_hub_tier_flags(const int32_t *deg, int64_t n, int cache_hub, int wide, uint32_t *flag_a,
                                 uint32_t *flag_b) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int d = deg[v];
        flag_a[v] = d >= cache_hub && d >= wide ? 1u : 0u;
        flag_b[v] = d >= cache_hub && d < wide ? 1u : 0u;
    }
}

__global__ void k_hub_tier_ids(const uint32_t *flag_a, const uint32_t *pos_a, const uint32_t *flag_b,
                               const uint32_t *pos_b, int64_t n, int32_t *hubid) {
    const uint32_t na = pos_a[n];
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        hubid[v] = flag_a[v] ? (int32_t)pos_a[v] : (flag_b[v] ? (int32_t)(na + pos_b[v]) : -1);
}

// t of every edge (or of the edges at the E_ordered positions listed in pos),
// written to both of its CSR slots (the slot records' last field).  One warp
// per edge: the shorter list's entries are searched in the longer one.
__global__ void k_tslot(DevGraph G, int4 *slot, const int32_t *pos, int64_t count) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t total = pos ? count : G.m;
    for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < total; i += nw) {
        const int64_t id = pos ? G.order[pos[i]] : i;
        // in a batch each graph's edge ids and E_ordered positions cover the
        // same range, so egraph[id] is the edge's graph
        if (dense_edge(G, id)) continue;
        const int32_t a = G.ev[id], b = G.eu[id];
        const int da = G.deg[a], db = G.deg[b];
        const int32_t s = da <= db ? a : b, l = da <= db ? b : a;
        const int ds = da <= db ? da : db, dl = da <= db ? db : da;
        const int32_t *Ns = G.adj + G.off[s], *Nl = G.adj + G.off[l];
        unsigned long long t = 0;
        for (int i = lane; i < ds; i += 32) t += pgd_contains(Nl, dl, __ldg(Ns + i)) ? 1 : 0;
        t = pgd_warp_sum(t);
        if (lane == 0) slot[G.off[a] + pgd_lower_bound(G.adj + G.off[a], da, b)].w = (int)t;
        if (lane == 1) slot[G.off[b] + pgd_lower_bound(G.adj + G.off[b], db, a)].w = (int)t;
    }
}

// ---------------------------------------------------------------------------
// work plan: hub-anchored edges grouped by anchor, light edges listed

// Sort keys of the work plan, with the E_ordered position as the value.
// Hub-anchored edges: (rank(anchor) << eb | position), so one sort groups
// them by anchor, highest-degree anchors first (the largest work items are
// handed out first).  (Heaviest-edge-first within an anchor shortens the
// items' tails but was measured slower: all warps then gather hub lists at
// once.)  Dense-graph edges (batches only) get class n, the rest n + 1, so
// the sorted order is [hub-anchored, by anchor][dense][light].  eb bits hold
// a position; the sort needs eb + bits(n + 2) key bits.
__global__ void k_plan_keys(DevGraph G, uint64_t *keys, int32_t *vals, unsigned long long *counts, int eb) {
    unsigned long long hubs = 0, dense = 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < G.npos; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t id = G.order[e];
        const int32_t v = G.ev[id], u = G.eu[id];
        const int32_t p = ranks_above(v, u, G.deg) ? v : u;
        const bool d = dense_edge(G, e);
        const bool hub = !d && G.deg[p] >= G.anchor_hub;
        const uint64_t cls = d ? (uint64_t)G.n : (hub ? (uint64_t)G.vrank[p] : (uint64_t)G.n + 1);
        keys[e] = (cls << eb) | (uint64_t)e;
        vals[e] = (int32_t)e;
        hubs += hub;
        dense += d;
    }
    hubs = pgd_warp_sum(hubs);
    dense = pgd_warp_sum(dense);
    if ((threadIdx.x & 31) == 0) {
        if (hubs) atomicAdd(counts, hubs);
        if (dense) atomicAdd(counts + 3, dense);
    }
}

// item i starts a chunk: the first edge of an anchor's run of L edges, or
// every c-th of it, c = ceil(L / min(ceil(L / kChunk), kMaxChunks))
__global__ void k_item_flags(const uint64_t *keys, int64_t nh, uint32_t *flag, int eb) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t p = keys[i] >> eb;
        // first index of this anchor's run
        int64_t lo = 0, hi = i;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if ((keys[mid] >> eb) < p) lo = mid + 1; else hi = mid;
        }
        // one past its last index
        int64_t lo2 = i + 1, hi2 = nh;
        while (lo2 < hi2) {
            int64_t mid = (lo2 + hi2) >> 1;
            if ((keys[mid] >> eb) <= p) lo2 = mid + 1; else hi2 = mid;
        }
        const int64_t L = lo2 - lo;
        const int64_t chunks = min((L + kChunk - 1) / kChunk, (int64_t)kMaxChunks);
        const int64_t c = (L + chunks - 1) / chunks;
        flag[i] = ((i - lo) % c == 0) ? 1u : 0u;
    }
}

// Per hub-anchored plan position i: {E_ordered position e, the non-anchor
// endpoint q}, so that k_hub starts an edge with one load instead of a chain
// of four (position -> edge id -> endpoints -> q).
__global__ void k_hub_recs(DevGraph G, const int32_t *hpos, int64_t nh, int2 *hrec) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t e = hpos[i];
        const int32_t id = G.order[e];
        const int32_t v = G.ev[id], u = G.eu[id];
        hrec[i] = make_int2(e, ranks_above(v, u, G.deg) ? u : v);
    }
}

__global__ void k_item_fill(const uint32_t *flag, const uint32_t *pos, int64_t nh, int64_t *items) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh; i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) items[pos[i]] = i;
    if (blockIdx.x == 0 && threadIdx.x == 0) items[pos[nh]] = nh;
}


// ---------------------------------------------------------------------------
// shared per-edge epilogue

__device__ __forceinline__ void flush_graph(const DevGraph &G, unsigned long long *acc, int g) {
    unsigned long long *dst = G.sums + (int64_t)g * PGD_NSUMS;
#pragma unroll
    for (int i = 0; i < PGD_NSUMS; i++) {
        if (acc[i]) atomicAdd(dst + i, acc[i]);
        acc[i] = 0;
    }
}

// Closed forms, sums and the per-edge row of one edge.  Batched runs keep
// the sums of the current graph in acc and flush them when the warp moves
// on to another graph (cur_g).
__device__ __forceinline__ void edge_epilogue_d(const DevGraph &G, unsigned long long *acc, int &cur_g, int64_t e,
                                                long long dv, long long du, unsigned long long t,
                                                unsigned long long k4, unsigned long long c4, int lane) {
    long long n = G.n, m = G.m;
    if (G.egraph) {
        const int g = G.egraph[e];
        if (g != cur_g) {
            if (lane == 0 && cur_g >= 0) flush_graph(G, acc, cur_g);
            cur_g = g;
        }
        n = G.gnm[2 * g];
        m = G.gnm[2 * g + 1];
    }
    if (lane == 0) {
        pgd_edge_sums(acc, dv, du, t, m, n);
        acc[3] += k4;
        acc[4] += c4;
    }
    if (G.micro && lane < PGD_NMICRO) G.micro[e * PGD_NMICRO + lane] = pgd_micro_col(lane, dv, du, t, k4, c4);
}

// The closed forms are symmetric in the two endpoints: only their degrees matter.
__device__ __forceinline__ void edge_epilogue(const DevGraph &G, unsigned long long *acc, int &cur_g, int64_t e,
                                              int32_t v, int32_t u, unsigned long long t, unsigned long long k4,
                                              unsigned long long c4, int lane) {
    edge_epilogue_d(G, acc, cur_g, e, G.deg[v], G.deg[u], t, k4, c4, lane);
}

__device__ __forceinline__ void block_flush(const DevGraph &G, unsigned long long *acc, int cur_g,
                                            unsigned long long (*red)[PGD_NSUMS], int nwarps) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (G.egraph) {
        if (lane == 0 && cur_g >= 0) flush_graph(G, acc, cur_g);
        return;
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < PGD_NSUMS; i++) red[wid][i] = acc[i];
    }
    __syncthreads();
    if (threadIdx.x < PGD_NSUMS) {
        unsigned long long s = 0;
        for (int w = 0; w < nwarps; w++) s += red[w][threadIdx.x];
        atomicAdd(G.sums + threadIdx.x, s);
    }
}

// Owner lane of flattened item `it`: the first lane whose inclusive prefix
// exceeds it (all 32 lanes must call).
__device__ __forceinline__ int owner_of(int incl, int it) {
    int lo = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        int pre = __shfl_sync(0xffffffffu, incl, lo + step - 1);
        if (pre <= it) lo += step;
    }
    return lo;
}


// N(p) as a bitmap over degree ranks: ranks below `split` in shared memory,
// the rest in this CTA's global slice.  Queries are weighted by degree, so
// almost all of them land in the shared part.
struct RankBits {
    uint32_t *s;       // shared words (ranks < split)
    uint32_t *g;       // global slice (indexed by rank >> 5; only ranks >= split are used)
    int32_t split;     // multiple of 32
    __device__ __forceinline__ bool test(int32_t r) const {
        return r < split ? (s[r >> 5] >> (r & 31)) & 1u : (__ldcg(g + (r >> 5)) >> (r & 31)) & 1u;
    }
    __device__ __forceinline__ void set(int32_t r) const {
        if (r < split) atomicOr(s + (r >> 5), 1u << (r & 31));
        else atomicOr(g + (r >> 5), 1u << (r & 31));
    }
    __device__ __forceinline__ void clear_word(int32_t r) const {
        if (r < split) s[r >> 5] = 0;
        else g[r >> 5] = 0;
    }
};

// ---------------------------------------------------------------------------
// Hub anchors: one CTA per (anchor, chunk of its edges).
//
// Per work item: (1) N(p) goes into the rank bitmap and, in the same pass, the
// hub-neighbour lists of N(p) are histogrammed: afterwards hist[h] =
// |N(w_h) n N(p)| = W(w_h, p) for every hub w_h, whatever q needs it.
// (2) The chunk's edges are decomposed, one warp each, fetched dynamically.
// Per edge the warp first collects T (marked by degree rank in a per-warp
// bitmap), t, sum t(x,q) and the W's of hub neighbours, then scans what is
// left: N(w) of non-hub w in S_q (W by bit tests of its entries' ranks) and, for
// k4, |N+(x) n T| of x in T, either from x's oriented list or, for the
// highest-ranked x, as AND + popc of x's rank-bitmap row with the T bitmap.
// Lists of 64 or more entries are read warp-cooperatively; shorter ones are
// flattened across the warp, two loads in flight per lane.  Each neighbour w
// of q is described by one 32-byte record (offsets, |N+(w)|, rank, hub id);
// for q of degree <= 32, the first pass keeps what the second scans in
// registers.

struct HubArgs {
    DevGraph G;
    const int32_t *hpos;      // E_ordered positions of hub-anchored edges, grouped by anchor
    const int2 *hrec;         // per position: {E_ordered position, non-anchor endpoint q}
    const int64_t *items;     // chunk starts into hpos, nitems+1 entries
    int64_t nitems;
    uint32_t *ghist;          // per CTA histogram slices (hstride words each) when not in shared memory
    int32_t nhubs;
    int32_t nwide;            // hub ids below this: wide counters; the rest 8-bit, four per word
    int64_t wide_words;       // words of the wide tier (the 8-bit tier follows)
    int64_t hstride;
    int smem_hist;
    int hist16;               // wide counters of 16 bits, two per word (every W < 65536: max degree below that)
    uint32_t *gbitmap;        // per CTA rank-bitmap slices (nwords each) when split < n
    int64_t nwords;
    int32_t split;            // ranks below this are kept in shared memory
    unsigned long long *next;
    int4 *slot_out;           // k_tslot_hub: slot records whose t it writes
    int32_t *thigh;           // k_hub: per-warp lists of T's high-rank members (kTHigh each)
    uint32_t *twin;           // k_hub: per-warp bitmaps of T's members of rank in [kRankBits, kRankBits + 32 twin_words)
    int32_t twin_words;
};

// |{r in L[0..len) : r in N(p)}| for a list of ranks, warp-cooperative,
// 4 loads in flight per lane.
__device__ __forceinline__ unsigned count_bits(const RankBits &bm, const int32_t *L, int len, int lane) {
    unsigned c = 0;
    int i = lane;
    for (; i + 96 < len; i += 128) {
        const int32_t x0 = __ldg(L + i), x1 = __ldg(L + i + 32), x2 = __ldg(L + i + 64), x3 = __ldg(L + i + 96);
        c += bm.test(x0) + bm.test(x1) + bm.test(x2) + bm.test(x3);
    }
    for (; i < len; i += 32) c += bm.test(__ldg(L + i));
    return c;
}

// sum over the row's words of popc(row & Rw), warp-cooperative, 64 bits per
// load (rows and the T bitmap are 8-byte aligned; words is even)
__device__ __forceinline__ unsigned row_and_count(const uint32_t *row, const uint32_t *Rw, int words, int lane) {
    const unsigned long long *r64 = (const unsigned long long *)row;
    const unsigned long long *t64 = (const unsigned long long *)Rw;
    const int w64 = words >> 1;
    unsigned c = 0;
    int i = lane;
    for (; i + 32 < w64; i += 64) c += __popcll(__ldg(r64 + i) & t64[i]) + __popcll(__ldg(r64 + i + 32) & t64[i + 32]);
    if (i < w64) c += __popcll(__ldg(r64 + i) & t64[i]);
    return c;
}

// y in T = N(p) n N(q).  Almost every y tested is a high-degree vertex, so
// T's members of degree rank < kRankBits are marked in a per-warp bitmap and
// the test is one shared-memory bit; other y fall back to the N(p) bitmap and
// a search of N(q).
// T's members of rank >= kRankBits, in id order, kept by the warp in pass 1
// (a per-warp global slice that stays in L1) when there are at most kTHigh.
struct THigh {
    const int32_t *ids;
    int count;       // -1: more than kTHigh, search N(q) instead
};

// T's members of rank in [kRankBits, kRankBits + 32 twin_words), marked by
// the warp in pass 1 in its global bitmap (written by atomics, so read past
// L1).  Addressed from the kernel parameters so that no register holds it.
__device__ __forceinline__ uint32_t *twin_of(const HubArgs &A) {
    return A.twin + ((int64_t)blockIdx.x * kHubWarps + (threadIdx.x >> 5)) * A.twin_words;
}

// y (rank ry, id at *yp, loaded only when needed) in T?
__device__ __forceinline__ bool in_t(const uint32_t *Rw, const HubArgs &A, const RankBits &bm, const int32_t *Nq,
                                     int dq, const int32_t *yp, int32_t ry, const THigh &th) {
    if (ry < kRankBits) return (Rw[ry >> 5] >> (ry & 31)) & 1u;
    if (ry < kRankBits + 32 * A.twin_words) return (__ldcg(twin_of(A) + ((ry - kRankBits) >> 5)) >> (ry & 31)) & 1u;
    if (!bm.test(ry)) return false;
    const int32_t y = __ldg(yp);
    return th.count >= 0 ? pgd_contains(th.ids, th.count, y) : pgd_contains(Nq, dq, y);
}

__device__ __forceinline__ int64_t rec_off(const int4 &ra) { return (int64_t)(((uint64_t)(uint32_t)ra.y << 32) | (uint32_t)ra.x); }
__device__ __forceinline__ int64_t rec_offp(const int4 &ra) { return (int64_t)(((uint64_t)(uint32_t)ra.w << 32) | (uint32_t)ra.z); }

// What pass 2 scans for neighbour w of q (slot record sr): for w in T, N+(w)
// as a rank-bitmap row (kind 2, from the rank alone) or as a list of ranks
// (kind 1, with the ids beside them for the rare test that needs one); for a
// non-hub w outside N(p), N(w)'s ranks (kind 0); nothing otherwise (len 0).
// Lists need w's offsets: one 32-byte vertex record.
__device__ __forceinline__ void plan_entry(const DevGraph &G, bool inT, const int4 &sr, int &len, int &kind,
                                           const int32_t *&list, const int32_t *&rlist) {
    const int32_t w = sr.x;
    if (inT) {
        const int32_t r = sr.y & 0x7fffffff;
        if (sr.y < 0) {
            kind = 2;
            len = top_row_words(r);
            list = (const int32_t *)(G.toprows + top_row_base(r));
        } else {
            const int4 ra = __ldg(G.vrec + 2 * (int64_t)w), rb = __ldg(G.vrec + 2 * (int64_t)w + 1);
            const int64_t o = rec_offp(ra);
            kind = 1;
            len = rb.y;
            list = G.adjp_rank + o;
            rlist = G.adjp + o;
        }
    } else if (sr.z < 0) {
        const int4 ra = __ldg(G.vrec + 2 * (int64_t)w), rb = __ldg(G.vrec + 2 * (int64_t)w + 1);
        kind = 0;
        len = rb.x;
        list = G.adj_rank + rec_off(ra);   // ranks: tested against the N(p) rank bitmap
    }
}

// Shared-memory scratch of walk_lists: 1024 inclusive prefix sums, 1024
// list starts and 32 warp totals (k_hub lends its per-warp T bitmaps, which
// are idle while an item's histogram is built; 3,104 words in all).
struct WalkScratch {
    int *pre;               // [1024]
    const int32_t **ptr;    // [1024]
    int *wtot;              // [32]
};
constexpr int kWalkScratchWords = 1024 + 2 * 1024 + 32;

// First t in [0, 1024) with pre[t] > i (pre non-decreasing; pre[1023] > i).
__device__ __forceinline__ int walk_owner_search(const int *pre, int i) {
    int lo = 0;
#pragma unroll
    for (int step = 512; step > 0; step >>= 1)
        if (pre[lo + step - 1] <= i) lo += step;
    return lo;
}

// Applies fn(h) to every entry h of the hub-neighbour lists of N(p) (and, when
// bm is given, marks N(p) in the rank bitmap), balanced over the whole CTA:
// the lists of 1024 entries of N(p) at a time are concatenated, and each warp
// takes an equal contiguous share of their entries, so that a few long lists
// no longer keep the other warps waiting at the item's barrier.  Inside a
// share, the owner list of each entry is found from 32 prefix sums held one
// per lane (a 5-step search), two entries per lane in flight.  All threads of
// the CTA must call; returns the number of entries visited.
template <typename Fn>
__device__ __forceinline__ long long walk_lists(const DevGraph &G, const int32_t *Np, const int32_t *Rp, int dp,
                                                const RankBits *bm, const WalkScratch &W, Fn fn) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long visited = 0;
    for (int c0 = 0; c0 < dp; c0 += kHubWarps * 32) {
        const int j = c0 + (int)threadIdx.x;
        int len = 0;
        const int32_t *list = nullptr;
        if (j < dp) {
            const int32_t x = __ldg(Np + j);
            if (bm) bm->set(__ldg(Rp + j));
            const int64_t o = G.offh[x];
            len = (int)(G.offh[x + 1] - o);
            list = G.adjh + o;
        }
        const int incl = pgd_warp_incl_scan(len);
        if (lane == 31) W.wtot[wid] = incl;
        __syncthreads();
        const int wt = W.wtot[lane];
        const int wincl = pgd_warp_incl_scan(wt);
        const int total = __shfl_sync(0xffffffffu, wincl, 31);
        W.pre[threadIdx.x] = __shfl_sync(0xffffffffu, wincl - wt, wid) + incl;
        W.ptr[threadIdx.x] = list;
        __syncthreads();
        visited += total;
        const int share = (total + kHubWarps - 1) / kHubWarps;
        const int lo = min(total, wid * share), hi = min(total, lo + share);
        int base = lo < hi ? walk_owner_search(W.pre, lo) : 0;
        for (int s = lo; s < hi;) {
            // most entries sit in long lists: while one list covers the next
            // 128 (or 64) entries, take them straight, coalesced, 4 (2) per lane
            const int own_end = W.pre[base];
            if (own_end - s >= 64 && hi - s >= 64) {
                const int32_t *L = W.ptr[base] + (s - (base ? W.pre[base - 1] : 0));
                if (own_end - s >= 128 && hi - s >= 128) {
                    const int32_t h0 = __ldg(L + lane), h1 = __ldg(L + 32 + lane), h2 = __ldg(L + 64 + lane),
                                  h3 = __ldg(L + 96 + lane);
                    fn(h0);
                    fn(h1);
                    fn(h2);
                    fn(h3);
                    s += 128;
                } else {
                    const int32_t h0 = __ldg(L + lane), h1 = __ldg(L + 32 + lane);
                    fn(h0);
                    fn(h1);
                    s += 64;
                }
                if (s >= own_end) base = s < hi ? walk_owner_search(W.pre, s) : base;
                continue;
            }
            const int cand = base + lane < 1024 ? W.pre[base + lane] : 0x7fffffff;
            const int last = __shfl_sync(0xffffffffu, cand, 31);
            const int iA = s + lane, iB = s + 32 + lane;
            const bool vA = iA < hi, vB = iB < hi;
            // owners beyond base + 31 (a run of empty lists): full search
            int ownA = base + owner_of(cand, iA), ownB = base + owner_of(cand, iB);
            if (vA && iA >= last) ownA = walk_owner_search(W.pre, iA);
            if (vB && iB >= last) ownB = walk_owner_search(W.pre, iB);
            int32_t hA = 0, hB = 0;
            if (vA) hA = __ldg(W.ptr[ownA] + (iA - (ownA ? W.pre[ownA - 1] : 0)));
            if (vB) hB = __ldg(W.ptr[ownB] + (iB - (ownB ? W.pre[ownB - 1] : 0)));
            if (vA) fn(hA);
            if (vB) fn(hB);
            // the next step's first entry (s + 64) belongs to lane 31's second
            // owner or a later list; the loop ends when that entry is invalid
            base = __shfl_sync(0xffffffffu, ownB, 31);
            s += 64;
        }
        __syncthreads();
    }
    return visited;
}

__global__ void __launch_bounds__(kHubWarps * 32, 1) k_hub(HubArgs A) {
    extern __shared__ __align__(16) uint32_t s_dyn[];
    __shared__ unsigned long long s_red[kHubWarps][PGD_NSUMS];
    __shared__ __align__(16) uint32_t s_R[kHubWarps][kRankBits / 32];
    __shared__ long long s_item;
    __shared__ int s_enext;
    __shared__ unsigned long long s_hcount;
    const DevGraph &G = A.G;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t *Rw = s_R[wid];
    for (int i = lane; i < kRankBits / 32; i += 32) Rw[i] = 0;
    static_assert(kWalkScratchWords <= kHubWarps * (kRankBits / 32), "walk scratch exceeds the T bitmaps");
    WalkScratch walk;
    uint32_t *const s_flat = &s_R[0][0];
    walk.pre = (int *)s_flat;
    walk.ptr = (const int32_t **)(s_flat + 1024);
    walk.wtot = (int *)(s_flat + 3072);
    const bool smem_hist = A.smem_hist != 0;
    // dynamic shared memory: [histogram (when shared)][rank bitmap, ranks < split]
    uint32_t *sh_hist = s_dyn;
    uint32_t *gl_hist = A.ghist + (int64_t)blockIdx.x * A.hstride;
    RankBits bm;
    bm.s = s_dyn + (smem_hist ? A.hstride : 0);
    bm.g = A.gbitmap ? A.gbitmap + (int64_t)blockIdx.x * A.nwords : nullptr;
    bm.split = A.split;
    const bool h16 = A.hist16 != 0;
    // this warp's partial sums live in shared memory (lane 0 updates them),
    // which keeps 30 registers free for the gathers
    unsigned long long *acc = s_red[wid];
    if (lane < PGD_NSUMS) acc[lane] = 0;
    const int nh4 = (int)(A.hstride >> 2);
    // counter h: word and increment.  Wide tier (h < nwide): 16-bit halves
    // (never carry: W < 65536) or whole words; 8-bit tier: bytes (never carry:
    // W(w,p) <= deg(w) < 256)
    const int32_t nwide = A.nwide;
    const int32_t wwords = (int32_t)A.wide_words;
    auto hw = [=](int32_t h) { return h < nwide ? (h16 ? (h >> 1) : h) : wwords + ((h - nwide) >> 2); };
    auto hinc = [=](int32_t h) {
        return h < nwide ? (h16 ? (1u << ((h & 1) << 4)) : 1u) : (1u << (((h - nwide) & 3) << 3));
    };
    auto hval = [=](uint32_t word, int32_t h) {
        return h < nwide ? (h16 ? ((word >> ((h & 1) << 4)) & 0xffffu) : word) : ((word >> (((h - nwide) & 3) << 3)) & 0xffu);
    };
    int cur_g = -1;
    for (int i = threadIdx.x; i < (A.split >> 5); i += blockDim.x) bm.s[i] = 0;
    {
        uint4 *h4 = (uint4 *)(smem_hist ? sh_hist : gl_hist);
        for (int i = threadIdx.x; i < nh4; i += blockDim.x) h4[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();

    while (true) {
        if (threadIdx.x == 0) {
            s_item = (long long)atomicAdd(A.next, 1ull);
            s_enext = 0;
            s_hcount = 0;
        }
        __syncthreads();
        const long long item = s_item;
        if (item >= A.nitems) break;
        const int64_t start = A.items[item], end = A.items[item + 1];
        const int nedge = (int)(end - start);
        int32_t p;
        {
            const int32_t id = G.order[A.hpos[start]];
            const int32_t v = G.ev[id], u = G.eu[id];
            p = ranks_above(v, u, G.deg) ? v : u;
        }
        const int dp = G.deg[p];
        const int32_t *Np = G.adj + G.off[p];
        const int32_t *Rp = G.adj_rank + G.off[p];

        // ---- (1) N(p) bitmap and the W histogram --------------------------
        // (the walk borrows the T bitmaps as scratch and they are zeroed again
        // before the edges, which need them clear)
        {
            long long visited;
            if (smem_hist)
                visited = walk_lists(G, Np, Rp, dp, &bm, walk, [&](int32_t h) { atomicAdd(sh_hist + hw(h), hinc(h)); });
            else
                visited = walk_lists(G, Np, Rp, dp, &bm, walk, [&](int32_t h) { atomicAdd(gl_hist + hw(h), hinc(h)); });
            if (threadIdx.x == 0) s_hcount = (unsigned long long)visited;
            for (int i = threadIdx.x; i < kWalkScratchWords; i += blockDim.x) s_flat[i] = 0;
        }
        __syncthreads();

        // ---- (2) the chunk's edges ---------------------------------------
        // fetched one ahead: the next edge's record is in flight while the
        // current edge is decomposed
        int kc = 0;
        if (lane == 0) kc = atomicAdd(&s_enext, 1);
        kc = __shfl_sync(0xffffffffu, kc, 0);
        int2 rc = kc < nedge ? __ldg(A.hrec + start + kc) : make_int2(0, 0);
        while (kc < nedge) {
            int kn = 0;
            if (lane == 0) kn = atomicAdd(&s_enext, 1);
            kn = __shfl_sync(0xffffffffu, kn, 0);
            const int2 rn = kn < nedge ? __ldg(A.hrec + start + kn) : make_int2(0, 0);
            const int64_t e = rc.x;
            const int32_t q = rc.y;
            const int4 qa = __ldg(G.vrec + 2 * (int64_t)q), qb = __ldg(G.vrec + 2 * (int64_t)q + 1);
            const int dq = qb.x;
            const int64_t offq = rec_off(qa);
            const int32_t *Nq = G.adj + offq;
            // pass 1: T (rank bitmap), t, sum of t(x,q) over T, W's of hubs;
            // for q of degree <= 32 also what pass 2 scans, kept in registers
            unsigned t = 0;
            unsigned long long sumtq = 0, sumW = 0, k4 = 0;
            int len0 = 0, kind0 = 0;
            const int32_t *list0 = nullptr, *rlist0 = nullptr;
            int nhigh = A.thigh ? 0 : -1;   // T members of rank >= kRankBits listed so far (warp-uniform)
            for (int base = 0; base < dq; base += 64) {
                const int j0 = base + lane, j1 = base + 32 + lane;
                const int4 none = make_int4(p, 0, -1, 0);
                const int4 s0 = j0 < dq ? __ldg(G.slot + offq + j0) : none;
                const int4 s1 = j1 < dq ? __ldg(G.slot + offq + j1) : none;
#pragma unroll
                for (int h2 = 0; h2 < 2; h2++) {
                    const int4 sr = h2 ? s1 : s0;
                    bool inT = false, hi = false;
                    if (sr.x != p) {
                        inT = bm.test(sr.y & 0x7fffffff);
                        if (inT) {
                            sumtq += (uint32_t)sr.w;
                            const int32_t r = sr.y & 0x7fffffff;
                            if (r < kRankBits) atomicOr(Rw + (r >> 5), 1u << (r & 31));
                            else if (r < kRankBits + 32 * A.twin_words)
                                atomicOr(twin_of(A) + ((r - kRankBits) >> 5), 1u << (r & 31));
                            hi = r >= kRankBits;
                        } else {
                            const int32_t h = sr.z;
                            if (h >= 0) sumW += hval(smem_hist ? sh_hist[hw(h)] : __ldcg(gl_hist + hw(h)), h);
                        }
                        if (dq <= 32 && h2 == 0) plan_entry(G, inT, sr, len0, kind0, list0, rlist0);
                    }
                    t += __popc(__ballot_sync(0xffffffffu, inT));
                    // list T's high-rank members in N(q)'s (id) order
                    const unsigned hm = __ballot_sync(0xffffffffu, hi);
                    if (hm && nhigh >= 0) {
                        const int at = nhigh + __popc(hm & ((1u << lane) - 1));
                        if (nhigh + __popc(hm) > kTHigh) nhigh = -1;
                        else {
                            if (hi) A.thigh[(int64_t)(blockIdx.x * kHubWarps + wid) * kTHigh + at] = sr.x;
                            nhigh += __popc(hm);
                        }
                    }
                }
            }
            __syncwarp();
            THigh th;
            th.ids = A.thigh ? A.thigh + (int64_t)(blockIdx.x * kHubWarps + wid) * kTHigh : nullptr;
            th.count = nhigh;
            // pass 2: N(w) of non-hub w in S_q (kind 0), N+(x) of x in T as a
            // list (kind 1) or as a rank-bitmap row (kind 2)
            for (int base = 0; base < dq; base += 32) {
                int len = len0, kind = kind0;
                const int32_t *list = list0;
                const int32_t *rlist = rlist0;
                if (dq > 32) {
                    const int j = base + lane;
                    len = 0;
                    kind = 0;
                    list = rlist = nullptr;
                    if (j < dq) {
                        const int4 sr = __ldg(G.slot + offq + j);
                        if (sr.x != p) plan_entry(G, bm.test(sr.y & 0x7fffffff), sr, len, kind, list, rlist);
                    }
                }
                // long lists (>= 64 entries): one at a time, warp-cooperative
                unsigned longm = __ballot_sync(0xffffffffu, len >= 64);
                while (longm) {
                    const int src = __ffs(longm) - 1;
                    longm &= longm - 1;
                    const int32_t *L = (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)list, src);
                    const int32_t *LR = (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)rlist, src);
                    const int ln = __shfl_sync(0xffffffffu, len, src);
                    const int lk = __shfl_sync(0xffffffffu, kind, src);
                    if (lk == 0) {
                        sumW += count_bits(bm, L, ln, lane);
                    } else if (lk == 2) {
                        k4 += row_and_count((const uint32_t *)L, Rw, ln, lane);
                    } else {
                        int i = lane;
                        for (; i + 32 < ln; i += 64) {
                            const int32_t r0 = __ldg(L + i), r1 = __ldg(L + i + 32);
                            k4 += (in_t(Rw, A, bm, Nq, dq, LR + i, r0, th) ? 1 : 0) +
                                  (in_t(Rw, A, bm, Nq, dq, LR + i + 32, r1, th) ? 1 : 0);
                        }
                        for (; i < ln; i += 32) k4 += in_t(Rw, A, bm, Nq, dq, LR + i, __ldg(L + i), th) ? 1 : 0;
                    }
                }
                // short lists: flattened over the warp (a short row counts its
                // 64-bit words)
                if (len >= 64) len = 0;
                if (kind == 2) len >>= 1;
                const int incl = pgd_warp_incl_scan(len);
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                const int excl = incl - len;
                for (int b2 = 0; b2 < total; b2 += 64) {
                    const int itA = b2 + lane, itB = b2 + 32 + lane;
                    const int ownA = owner_of(incl, itA), ownB = owner_of(incl, itB);
                    const int32_t *olA = (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)list, ownA);
                    const int32_t *orA = (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)rlist, ownA);
                    const int okA = __shfl_sync(0xffffffffu, kind, ownA);
                    const int idxA = itA - __shfl_sync(0xffffffffu, excl, ownA);
                    const int32_t *olB = (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)list, ownB);
                    const int32_t *orB = (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)rlist, ownB);
                    const int okB = __shfl_sync(0xffffffffu, kind, ownB);
                    const int idxB = itB - __shfl_sync(0xffffffffu, excl, ownB);
                    const bool vA = itA < total, vB = itB < total;
                    const unsigned long long *t64 = (const unsigned long long *)Rw;
                    unsigned long long xA = 0, xB = 0;
                    if (vA) xA = okA == 2 ? __ldg((const unsigned long long *)olA + idxA) : (uint32_t)__ldg(olA + idxA);
                    if (vB) xB = okB == 2 ? __ldg((const unsigned long long *)olB + idxB) : (uint32_t)__ldg(olB + idxB);
                    if (vA) {
                        if (okA == 0) sumW += bm.test((int32_t)xA);
                        else if (okA == 2) k4 += __popcll(xA & t64[idxA]);
                        else k4 += in_t(Rw, A, bm, Nq, dq, orA + idxA, (int32_t)xA, th) ? 1 : 0;
                    }
                    if (vB) {
                        if (okB == 0) sumW += bm.test((int32_t)xB);
                        else if (okB == 2) k4 += __popcll(xB & t64[idxB]);
                        else k4 += in_t(Rw, A, bm, Nq, dq, orB + idxB, (int32_t)xB, th) ? 1 : 0;
                    }
                }
            }
            sumtq = pgd_warp_sum(sumtq);
            sumW = pgd_warp_sum(sumW);
            k4 = pgd_warp_sum(k4);
            const long long c4 = (long long)sumW - ((long long)dq - (long long)t - 1) - (long long)sumtq +
                                 2 * (long long)k4 + (long long)t;
            edge_epilogue_d(G, acc, cur_g, e, dp, dq, t, k4, (unsigned long long)c4, lane);
            __syncwarp();
            for (int i = lane; i < kRankBits / 32; i += 32) Rw[i] = 0;
            if (A.twin_words) {
                // clear the window words of T's listed high-rank members, or all of
                // it when the list overflowed
                uint32_t *twp = twin_of(A);
                if (nhigh >= 0) {
                    for (int i = lane; i < nhigh; i += 32) {
                        const int32_t r = G.vrank[th.ids[i]];
                        if (r < kRankBits + 32 * A.twin_words) twp[(r - kRankBits) >> 5] = 0;
                    }
                } else {
                    for (int i = lane; i < A.twin_words; i += 32) twp[i] = 0;
                }
            }
            __syncwarp();
            kc = kn;
            rc = rn;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < dp; i += blockDim.x) bm.clear_word(__ldg(Rp + i));
        if (smem_hist || s_hcount * 4 >= (unsigned long long)A.nhubs) {
            // a shared histogram is cleared whole: a few 16-byte stores per thread
            uint4 *h4 = (uint4 *)(smem_hist ? sh_hist : gl_hist);
            for (int i = threadIdx.x; i < nh4; i += blockDim.x) h4[i] = make_uint4(0, 0, 0, 0);
        } else {
            // few entries of a global histogram touched (large graphs, small
            // anchors): clear just those (a 16-bit word's other counter is zero
            // or cleared too); the walk's scratch is zeroed by the next item's
            // phase 1 before any edge reads the T bitmaps
            __syncthreads();
            walk_lists(G, Np, Rp, dp, nullptr, walk, [&](int32_t h) { gl_hist[hw(h)] = 0; });
        }
        __syncthreads();
    }
    block_flush(G, acc, cur_g, s_red, kHubWarps);
}

// ---------------------------------------------------------------------------
// t of the hub-anchored edges, grouped like k_hub's work items: per item the
// anchor's neighbours go into the rank bitmap once, then each edge (p, q)
// counts the entries of N(q) whose rank is set -- one coalesced pass over
// q's ranks and shared-memory bit tests, instead of a binary search in N(p)
// per entry.  Both CSR slots of the edge get t.

__global__ void __launch_bounds__(kHubWarps * 32, 1) k_tslot_hub(HubArgs A) {
    extern __shared__ __align__(16) uint32_t s_dyn[];
    __shared__ long long s_item;
    __shared__ int s_enext;
    const DevGraph &G = A.G;
    const int lane = threadIdx.x & 31;
    RankBits bm;
    bm.s = s_dyn;
    bm.g = A.gbitmap ? A.gbitmap + (int64_t)blockIdx.x * A.nwords : nullptr;
    bm.split = A.split;
    for (int i = threadIdx.x; i < (A.split >> 5); i += blockDim.x) bm.s[i] = 0;
    __syncthreads();
    while (true) {
        if (threadIdx.x == 0) {
            s_item = (long long)atomicAdd(A.next, 1ull);
            s_enext = 0;
        }
        __syncthreads();
        const long long item = s_item;
        if (item >= A.nitems) break;
        const int64_t start = A.items[item], end = A.items[item + 1];
        const int nedge = (int)(end - start);
        int32_t p;
        {
            const int2 r0 = A.hrec[start];
            const int32_t id = G.order[r0.x];
            p = G.ev[id] == r0.y ? G.eu[id] : G.ev[id];
        }
        const int64_t offp = G.off[p];
        const int dp = G.deg[p];
        const int32_t *Rp = G.adj_rank + offp;
        for (int i = threadIdx.x; i < dp; i += blockDim.x) bm.set(__ldg(Rp + i));
        __syncthreads();
        while (true) {
            int k = 0;
            if (lane == 0) k = atomicAdd(&s_enext, 1);
            k = __shfl_sync(0xffffffffu, k, 0);
            if (k >= nedge) break;
            const int32_t q = __ldg(&A.hrec[start + k].y);
            const int64_t offq = G.off[q];
            const int dq = G.deg[q];
            const int32_t *Rq = G.adj_rank + offq;
            unsigned c = 0;
            int i = lane;
            for (; i + 96 < dq; i += 128) {
                const int32_t r0 = __ldg(Rq + i), r1 = __ldg(Rq + i + 32), r2 = __ldg(Rq + i + 64), r3 = __ldg(Rq + i + 96);
                c += bm.test(r0) + bm.test(r1) + bm.test(r2) + bm.test(r3);
            }
            for (; i < dq; i += 32) c += bm.test(__ldg(Rq + i));
            c = __reduce_add_sync(0xffffffffu, c);
            if (lane == 0) A.slot_out[offp + pgd_lower_bound(G.adj + offp, dp, q)].w = (int)c;
            if (lane == 1) A.slot_out[offq + pgd_lower_bound(G.adj + offq, dq, p)].w = (int)c;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < dp; i += blockDim.x) bm.clear_word(__ldg(Rp + i));
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Light anchors (degree < kAnchorHub): one warp per edge, N(p) staged and
// labelled (T / S_p / q) in shared memory.

struct LightArgs {
    DevGraph G;
    const int32_t *lpos;   // E_ordered positions of light-anchored edges
    int64_t nlight;
    unsigned long long *next;
};

__global__ void __launch_bounds__(kLightWarps * 32) k_light(LightArgs A) {
    __shared__ int32_t s_np[kLightWarps][kLightStageMax];
    __shared__ uint8_t s_lab[kLightWarps][kLightStageMax];
    __shared__ unsigned long long s_red[kLightWarps][PGD_NSUMS];
    const DevGraph &G = A.G;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t *np_s = s_np[wid];
    uint8_t *lab_s = s_lab[wid];
    int cur_g = -1;
    unsigned long long acc[PGD_NSUMS];
#pragma unroll
    for (int i = 0; i < PGD_NSUMS; i++) acc[i] = 0;

    // edges are fetched four at a time: neighbouring positions mostly belong
    // to the same graph when a batch is decomposed
    unsigned long long idx = 0, idx_end = 0;
    while (true) {
        if (idx == idx_end) {
            if (lane == 0) idx = atomicAdd(A.next, 4ull);
            idx = __shfl_sync(0xffffffffu, idx, 0);
            idx_end = min(idx + 4, (unsigned long long)A.nlight);
        }
        if (idx >= (unsigned long long)A.nlight) break;
        const int64_t e = A.lpos[idx++];
        const int32_t id = G.order[e];
        const int32_t v = G.ev[id], u = G.eu[id];
        const int32_t p = ranks_above(v, u, G.deg) ? v : u;
        const int32_t q = (p == v) ? u : v;
        const int dp = G.deg[p], dq = G.deg[q];
        const int32_t *Np = G.adj + G.off[p];
        const int64_t offq = G.off[q];
        const int32_t *Nq = G.adj + offq;
        for (int i = lane; i < dp; i += 32) {
            const int32_t y = __ldg(Np + i);
            np_s[i] = y;
            lab_s[i] = (y == q) ? 0 : (pgd_contains(Nq, dq, y) ? 3 : 1);
        }
        __syncwarp();
        const int logp = 32 - __clz(dp | 1);
        unsigned long long t = 0, sumtq = 0, sumW = 0, k4 = 0;
        for (int base = 0; base < dq; base += 32) {
            const int j = base + lane;
            int len = 0, kind = 0, dw = 0;
            bool rev = false;
            const int32_t *list = nullptr;
            if (j < dq) {
                const int32_t w = __ldg(Nq + j);
                if (w != p) {
                    const int pos = pgd_lower_bound(np_s, dp, w);
                    if (pos < dp && np_s[pos] == w) {     // w in T
                        t++;
                        sumtq += (uint32_t)G.slot[offq + j].w;
                        kind = 1;
                        const int64_t o = G.offp[w];
                        len = (int)(G.offp[w + 1] - o);
                        list = G.adjp + o;
                    } else {
                        dw = G.deg[w];
                        list = G.adj + G.off[w];
                        const int logw = 32 - __clz(dw | 1);
                        rev = (long long)dw * logp > 2LL * dp * logw;
                        len = rev ? 0 : dw;
                    }
                }
            }
            const int incl = pgd_warp_incl_scan(len);
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            const int excl = incl - len;
            for (int b2 = 0; b2 < total; b2 += 32) {
                const int it = b2 + lane;
                const int own = owner_of(incl, it);
                const int32_t *olist = (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)list, own);
                const int okind = __shfl_sync(0xffffffffu, kind, own);
                const int oexcl = __shfl_sync(0xffffffffu, excl, own);
                if (it < total) {
                    const int32_t x = __ldg(olist + (it - oexcl));
                    const int pos = pgd_lower_bound(np_s, dp, x);
                    const bool in_p = pos < dp && np_s[pos] == x;
                    if (okind == 0) sumW += in_p;
                    else k4 += (in_p && lab_s[pos] == 3) ? 1 : 0;
                }
            }
            // long lists: search N(p)'s entries in N(w) instead
            unsigned revmask = __ballot_sync(0xffffffffu, rev);
            while (revmask) {
                const int src = __ffs(revmask) - 1;
                revmask &= revmask - 1;
                const int32_t *Nw = (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)list, src);
                const int wdeg = __shfl_sync(0xffffffffu, dw, src);
                for (int i = lane; i < dp; i += 32) sumW += pgd_contains(Nw, wdeg, np_s[i]) ? 1 : 0;
            }
        }
        t = pgd_warp_sum(t);
        sumtq = pgd_warp_sum(sumtq);
        sumW = pgd_warp_sum(sumW);
        k4 = pgd_warp_sum(k4);
        const long long c4 = (long long)sumW - ((long long)dq - (long long)t - 1) - (long long)sumtq +
                             2 * (long long)k4 + (long long)t;
        edge_epilogue(G, acc, cur_g, e, v, u, t, k4, (unsigned long long)c4, lane);
        __syncwarp();
    }
    block_flush(G, acc, cur_g, s_red, kLightWarps);
}

// ---------------------------------------------------------------------------
// Small graphs (batches): one warp per edge with whole adjacency rows as
// bitsets.  A row of up to 2048 vertices is 32 words of 64 bits, one per
// lane, so with A_x the row of x, T = A_p & A_q,
// S_p = A_p & ~A_q & ~{q}, S_q = A_q & ~A_p & ~{p}:
//   t = popc(T),  c4 = sum_{w in S_q} popc(A_w & S_p),
//   k4 = 1/2 sum_{x in T} popc(A_x & T),
// each row read once, coalesced, from L2.

struct DenseArgs {
    DevGraph G;
    const uint64_t *bits;     // rows of every dense graph, concatenated
    const int64_t *wbase;     // per graph: first word of its rows
    const int64_t *vbase;     // per graph: first union vertex id
    const int32_t *dpos;      // E_ordered positions of dense-graph edges
    int64_t ndense;
    unsigned long long *next;
};

__global__ void k_dense_bits(const int64_t *off, const int32_t *adj, const int32_t *vgraph, const uint8_t *gdense,
                             const int64_t *wbase, const int64_t *vbase, const long long *gnm, int64_t N,
                             unsigned long long *bits) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t x = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; x < N; x += nw) {
        const int g = vgraph[x];
        if (!gdense[g]) continue;
        const int64_t W = (gnm[2 * g] + 63) >> 6, vb = vbase[g];
        unsigned long long *row = bits + wbase[g] + (x - vb) * W;
        for (int64_t j = off[x] + lane; j < off[x + 1]; j += 32) {
            const int64_t c = adj[j] - vb;
            atomicOr(row + (c >> 6), 1ull << (c & 63));
        }
    }
}

// q of a dense-graph edge: the endpoint of smaller degree (ties: v)
__device__ __forceinline__ int32_t dense_q(const DevGraph &G, int64_t e) {
    const int32_t id = G.order[e];
    const int32_t v = G.ev[id], u = G.eu[id];
    return G.deg[v] <= G.deg[u] ? v : u;
}

// Sort keys grouping the dense-graph edges by q (then by position), so that
// k_dense can serve several edges with one pass over A_q's rows:
// (plain << (qb + eb)) | (q << eb) | position, q below 2^qb and positions
// below 2^eb.  Edges of graphs with a common-neighbour matrix (cbase[g] >= 0,
// plain = 0) sort first.
__global__ void k_dense_keys(DevGraph G, const int32_t *dpos, int64_t nd, const int64_t *cbase, uint64_t *keys,
                             int32_t *vals, unsigned long long *ncn, int qb, int eb) {
    unsigned long long cnt = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t e = dpos[i];
        const uint64_t plain = (cbase && cbase[G.egraph[e]] >= 0) ? 0ull : 1ull;
        keys[i] = (plain << (qb + eb)) | ((uint64_t)(uint32_t)dense_q(G, e) << eb) | (uint32_t)e;
        vals[i] = e;
        cnt += 1ull - plain;
    }
    cnt = pgd_warp_sum(cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(ncn, cnt);
}

constexpr int kDenseGroup = 6;   // edges sharing q decomposed together

// Up to kDenseGroup edges (p_j, q) with the same q: one pass over the rows of
// A_q's neighbours w serves all of them -- row w is ANDed with S_p_j when
// w is in S_q_j and with T_j when w is in T_j.
__global__ void __launch_bounds__(256, 3) k_dense(DenseArgs A) {
    __shared__ unsigned long long s_red[8][PGD_NSUMS];
    const DevGraph &G = A.G;
    const int lane = threadIdx.x & 31;
    int cur_g = -1;
    unsigned long long acc[PGD_NSUMS];
#pragma unroll
    for (int i = 0; i < PGD_NSUMS; i++) acc[i] = 0;
    while (true) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(A.next, (unsigned long long)kDenseGroup);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= (unsigned long long)A.ndense) break;
        const int64_t iend = min(idx + (unsigned long long)kDenseGroup, (unsigned long long)A.ndense);
        int64_t i0 = (int64_t)idx;
        while (i0 < iend) {
            // the run of edges with the same q (dpos is grouped by q)
            const int32_t qg = dense_q(G, A.dpos[i0]);
            int64_t i1 = i0 + 1;
            while (i1 < iend && dense_q(G, A.dpos[i1]) == qg) i1++;
            const int R = (int)(i1 - i0);
            const int g = G.egraph[A.dpos[i0]];
            const int64_t vb = A.vbase[g];
            const int W = (int)((G.gnm[2 * g] + 63) >> 6);
            const uint64_t *rows = A.bits + A.wbase[g];
            const int64_t q = qg - vb;
            const uint64_t Aq = lane < W ? __ldg(rows + q * W + lane) : 0ull;
            const uint64_t bq = (lane == (int)(q >> 6)) ? (1ull << (q & 63)) : 0ull;
            uint64_t T[kDenseGroup], Sp[kDenseGroup], Sq[kDenseGroup];
            unsigned c4[kDenseGroup], k4x2[kDenseGroup];
#pragma unroll
            for (int j = 0; j < kDenseGroup; j++) {
                T[j] = Sp[j] = Sq[j] = 0;
                c4[j] = k4x2[j] = 0;
                if (j < R) {
                    const int32_t id = G.order[A.dpos[i0 + j]];
                    const int32_t v = G.ev[id], u = G.eu[id];
                    const int64_t p = (v == qg ? u : v) - vb;
                    const uint64_t Ap = lane < W ? __ldg(rows + p * W + lane) : 0ull;
                    const uint64_t bp = (lane == (int)(p >> 6)) ? (1ull << (p & 63)) : 0ull;
                    T[j] = Ap & Aq;
                    Sp[j] = Ap & ~Aq & ~bq;
                    Sq[j] = Aq & ~Ap & ~bp;
                }
            }
            for (int L = 0; L < W; L++) {
                uint64_t wq = __shfl_sync(0xffffffffu, Aq, L);
                uint64_t ws[kDenseGroup], wt[kDenseGroup];
#pragma unroll
                for (int j = 0; j < kDenseGroup; j++) {
                    ws[j] = __shfl_sync(0xffffffffu, Sq[j], L);
                    wt[j] = __shfl_sync(0xffffffffu, T[j], L);
                }
                while (wq) {
                    const int b0 = __ffsll(wq) - 1;
                    wq &= wq - 1;
                    int b1 = -1;
                    if (wq) {
                        b1 = __ffsll(wq) - 1;
                        wq &= wq - 1;
                    }
                    const uint64_t r0 = lane < W ? __ldg(rows + ((int64_t)L * 64 + b0) * W + lane) : 0ull;
                    const uint64_t r1 = (b1 >= 0 && lane < W) ? __ldg(rows + ((int64_t)L * 64 + b1) * W + lane) : 0ull;
#pragma unroll
                    for (int j = 0; j < kDenseGroup; j++) {
                        if ((ws[j] >> b0) & 1ull) c4[j] += __popcll(r0 & Sp[j]);
                        else if ((wt[j] >> b0) & 1ull) k4x2[j] += __popcll(r0 & T[j]);
                        if (b1 >= 0) {
                            if ((ws[j] >> b1) & 1ull) c4[j] += __popcll(r1 & Sp[j]);
                            else if ((wt[j] >> b1) & 1ull) k4x2[j] += __popcll(r1 & T[j]);
                        }
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < kDenseGroup; j++) {
                if (j >= R) break;
                const unsigned long long t = pgd_warp_sum(__popcll(T[j]));
                const unsigned long long c = pgd_warp_sum(c4[j]);
                const unsigned long long k2 = pgd_warp_sum(k4x2[j]);
                const int64_t e = A.dpos[i0 + j];
                const int32_t id = G.order[e];
                edge_epilogue(G, acc, cur_g, e, G.ev[id], G.eu[id], t, k2 >> 1, c, lane);
            }
            i0 = i1;
        }
    }
    block_flush(G, acc, cur_g, s_red, 8);
}

// ---------------------------------------------------------------------------
// Dense graphs with a common-neighbour matrix.  For a graph of n vertices
// (W = ceil(n/64) row words) CN[a][b] = |N(a) ∩ N(b)| = popc(A_a & A_b), in
// 16-bit entries (n <= 2048), rows padded to 64·W entries so that a warp
// reads 64 entries per row word.  With it, c4 of an edge (p, q) follows from
//   c4 = sum_{w in S_q} CN[p][w] - |S_q| - sum_{x in T} CN[q][x] + 2·k4 + t
// (for w in S_q, N(w) ∩ N(p) holds q, |N(w) ∩ T| members of T and the rest
// of S_p; the edges between S_q and T number sum_{x in T} t(x, q) - 2·k4 - t,
// t(x, q) = CN[q][x]), so only the rows of T's members are scanned (for k4),
// not those of all of N(q).  Building CN costs n·64W·W word operations, which
// pays off for graphs of average degree >= n/16.

constexpr int kCnRows = 32;   // rows a of CN computed by one block

// One block per tile of 32 rows a of one graph: the tile's bit rows in shared
// memory, one column b per thread, 32 counters in registers.  ctile[g] is
// the first tile of graph g (k + 1 entries, non-decreasing).
__global__ void __launch_bounds__(256) k_dense_common(const uint64_t *bits, const int64_t *wbase,
                                                      const long long *gnm, const int64_t *cbase,
                                                      const int64_t *ctile, int k, int64_t ntiles, uint16_t *cn) {
    __shared__ uint64_t sa[kCnRows][32];
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int g = batch_find(ctile, k, tile);
        const int64_t n = gnm[2 * g];
        const int W = (int)((n + 63) >> 6);
        const int64_t stride = (int64_t)W * 64;
        const int64_t a0 = (tile - ctile[g]) * kCnRows;
        const uint64_t *rows = bits + wbase[g];
        __syncthreads();   // the previous tile's rows are no longer read
        for (int i = threadIdx.x; i < kCnRows * 32; i += blockDim.x) {
            const int r = i >> 5, w = i & 31;
            sa[r][w] = (a0 + r < n && w < W) ? rows[(a0 + r) * W + w] : 0ull;
        }
        __syncthreads();
        uint16_t *out = cn + cbase[g];
        for (int64_t b = threadIdx.x; b < stride; b += blockDim.x) {
            uint32_t acc[kCnRows];
#pragma unroll
            for (int i = 0; i < kCnRows; i++) acc[i] = 0;
            if (b < n) {
                const uint64_t *rb = rows + b * W;
                for (int w = 0; w < W; w++) {
                    const uint64_t x = __ldg(rb + w);
#pragma unroll
                    for (int i = 0; i < kCnRows; i++) acc[i] += __popcll(x & sa[i][w]);
                }
            }
#pragma unroll
            for (int i = 0; i < kCnRows; i++)
                if (a0 + i < n) out[(a0 + i) * stride + b] = (uint16_t)acc[i];
        }
    }
}

struct DenseCnArgs {
    DevGraph G;
    const uint64_t *bits;
    const int64_t *wbase;
    const int64_t *vbase;
    const uint16_t *cn;       // CN matrices of the graphs that have one
    const int64_t *cbase;     // per graph: first entry of its CN matrix
    const int32_t *dpos;      // E_ordered positions of those graphs' edges, grouped by q
    const uint32_t *k4pre;    // per position of dpos: 0xffffffff where k_dense_tc did not take the run (or null)
    int64_t ndense;
    unsigned long long *next;
};

// Up to kDenseGroup edges (p_j, q) with the same q, as in k_dense; per row
// word L of A_q the warp reads 64 entries of CN[q] and of each CN[p_j] (two
// per lane) for the two sums, and the rows of the word's members of T_j.
// Groups of the runs k_dense_tc took are left to k_dense_close.
__global__ void __launch_bounds__(256, 3) k_dense_cn(DenseCnArgs A) {
    __shared__ unsigned long long s_red[8][PGD_NSUMS];
    const DevGraph &G = A.G;
    const int lane = threadIdx.x & 31;
    int cur_g = -1;
    unsigned long long acc[PGD_NSUMS];
#pragma unroll
    for (int i = 0; i < PGD_NSUMS; i++) acc[i] = 0;
    while (true) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(A.next, (unsigned long long)kDenseGroup);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= (unsigned long long)A.ndense) break;
        const int64_t iend = min(idx + (unsigned long long)kDenseGroup, (unsigned long long)A.ndense);
        int64_t i0 = (int64_t)idx;
        while (i0 < iend) {
            const int32_t qg = dense_q(G, A.dpos[i0]);
            int64_t i1 = i0 + 1;
            while (i1 < iend && dense_q(G, A.dpos[i1]) == qg) i1++;
            const int R = (int)(i1 - i0);
            const int g = G.egraph[A.dpos[i0]];
            const int64_t vb = A.vbase[g];
            const int W = (int)((G.gnm[2 * g] + 63) >> 6);
            const int64_t stride = (int64_t)W * 64;
            const uint64_t *rows = A.bits + A.wbase[g];
            const uint16_t *cnb = A.cn + A.cbase[g];
            // a run taken by the tensor cores (all edges of a group share q, so
            // all or none of them are) is closed by k_dense_close
            if (A.k4pre && A.k4pre[i0] != 0xffffffffu) {
                i0 = i1;
                continue;
            }
            const int64_t q = qg - vb;
            const uint16_t *cq = cnb + q * stride;
            const uint64_t Aq = lane < W ? __ldg(rows + q * W + lane) : 0ull;
            uint64_t T[kDenseGroup], Sq[kDenseGroup];
            int32_t pl[kDenseGroup];
            unsigned k4x2[kDenseGroup];
            int dsum[kDenseGroup];   // this lane's share of sum_{S_q} CN[p][w] - sum_T CN[q][x]
#pragma unroll
            for (int j = 0; j < kDenseGroup; j++) {
                T[j] = Sq[j] = 0;
                pl[j] = 0;
                k4x2[j] = 0;
                dsum[j] = 0;
                if (j < R) {
                    const int32_t id = G.order[A.dpos[i0 + j]];
                    const int32_t v = G.ev[id], u = G.eu[id];
                    const int64_t p = (v == qg ? u : v) - vb;
                    const uint64_t Ap = lane < W ? __ldg(rows + p * W + lane) : 0ull;
                    const uint64_t bp = (lane == (int)(p >> 6)) ? (1ull << (p & 63)) : 0ull;
                    T[j] = Ap & Aq;
                    Sq[j] = Aq & ~Ap & ~bp;
                    pl[j] = (int32_t)p;
                }
            }
            for (int L = 0; L < W; L++) {
                // word L of every T_j as 32-bit halves
                uint32_t tlo[kDenseGroup], thi[kDenseGroup];
                uint32_t ulo = 0, uhi = 0;
#pragma unroll
                for (int j = 0; j < kDenseGroup; j++) {
                    tlo[j] = __shfl_sync(0xffffffffu, (uint32_t)T[j], L);
                    thi[j] = __shfl_sync(0xffffffffu, (uint32_t)(T[j] >> 32), L);
                    ulo |= tlo[j];
                    uhi |= thi[j];
                }
                // entries 64L + 2·lane and the next of CN[q] and CN[p_j]; their
                // bits are bits 2·lane, 2·lane + 1 of the word: of its low half
                // for lanes 0-15, of its high half for lanes 16-31
                const int64_t col = (int64_t)L * 64 + 2 * lane;
                const uint32_t cq2 = __ldg((const uint32_t *)(cq + col));
                const int sh = (2 * lane) & 31;
#pragma unroll
                for (int j = 0; j < kDenseGroup; j++) {
                    const uint32_t slo = __shfl_sync(0xffffffffu, (uint32_t)Sq[j], L);
                    const uint32_t shi = __shfl_sync(0xffffffffu, (uint32_t)(Sq[j] >> 32), L);
                    if (j < R) {
                        const uint32_t cp2 = __ldg((const uint32_t *)(cnb + (int64_t)pl[j] * stride + col));
                        const unsigned sb = (lane < 16 ? slo : shi) >> sh, tb = (lane < 16 ? tlo[j] : thi[j]) >> sh;
                        dsum[j] += (int)(((sb & 1u) ? (cp2 & 0xffffu) : 0u) + ((sb & 2u) ? (cp2 >> 16) : 0u)) -
                                   (int)(((tb & 1u) ? (cq2 & 0xffffu) : 0u) + ((tb & 2u) ? (cq2 >> 16) : 0u));
                    }
                }
                // rows of this word's members of the T_j (k4), one half at a
                // time, two rows in flight, each row tested against every T_j
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    uint32_t u = h ? uhi : ulo;
                    const uint64_t *rb = rows + ((int64_t)L * 64 + 32 * h) * W + lane;
                    while (u) {
                        const int b0 = __ffs(u) - 1;
                        u &= u - 1;
                        int b1 = -1;
                        if (u) {
                            b1 = __ffs(u) - 1;
                            u &= u - 1;
                        }
                        const uint32_t m0 = 1u << b0, m1 = b1 >= 0 ? (1u << b1) : 0u;
                        const uint64_t r0 = lane < W ? __ldg(rb + (int64_t)b0 * W) : 0ull;
                        const uint64_t r1 = (b1 >= 0 && lane < W) ? __ldg(rb + (int64_t)b1 * W) : 0ull;
#pragma unroll
                        for (int j = 0; j < kDenseGroup; j++) {
                            const uint32_t tj = h ? thi[j] : tlo[j];
                            if (tj & m0) k4x2[j] += __popcll(r0 & T[j]);
                            if (tj & m1) k4x2[j] += __popcll(r1 & T[j]);
                        }
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < kDenseGroup; j++) {
                if (j >= R) break;
                const unsigned long long t = pgd_warp_sum(__popcll(T[j]));
                const unsigned long long nsq = pgd_warp_sum(__popcll(Sq[j]));
                const unsigned long long k4 = pgd_warp_sum(k4x2[j]) >> 1;
                // sum_{S_q} CN[p][w] - sum_T CN[q][x]: lane shares are signed, the
                // warp's total modulo 2^64 is exact (|total| < 2^23)
                const unsigned long long dtot = pgd_warp_sum((unsigned long long)(long long)dsum[j]);
                const unsigned long long c = dtot + 2 * k4 + t - nsq;
                const int64_t e = A.dpos[i0 + j];
                const int32_t id = G.order[e];
                edge_epilogue(G, acc, cur_g, e, G.ev[id], G.eu[id], t, k4, c, lane);
            }
            i0 = i1;
        }
    }
    block_flush(G, acc, cur_g, s_red, 8);
}

// ---------------------------------------------------------------------------
// k4 of dense graphs on the tensor cores.  For an edge (p, q) with
// T = N(p) ∩ N(q),
//   2·k4(p, q) = sum_{y in T} |N(y) ∩ T| = sum_{y in N(q)} A_py · D[p][y],
//   D[p][y]    = sum_{x in N(q)} A_px · A_yx = |N(p) ∩ N(y) ∩ N(q)|,
// so for all edges (p_i, q) of one run (same q) D is a product of rows of the
// ego network of q, compacted to the columns N(q): the rows p_i (M side, one
// TMEM lane each) times every row y of N(q) (N side, one TMEM column each),
// over K = N(q).  0/1 entries are exact in e4m3 and every fp32 sum stays below
// 2^24 (d_q <= kTcMaxDeg), so the counts are exact.
//
// One CTA of 16 warps per SM takes runs from a counter.  Per run: the rows of
// N(q), compacted to N(q)'s columns (a software bit-compress per 64-bit word,
// the "compress" of Hacker's Delight §7-4 with its masks computed once per word
// of A_q), go to shared memory.  Then for each pair of 128-edge tiles and each
// 256-row tile of N(q), every 64-column chunk is expanded to e4m3 tiles (one B
// tile shared by both edge tiles) by 15 builder warps into one of two
// alternating stages while the tensor cores run the previous chunk's MMAs,
// which one thread of the last warp issues into two TMEM accumulators.  The
// builders and the issuing thread meet at per-stage mbarriers only: "full"
// (every builder warp arrived) and "empty" (tcgen05.commit of the MMAs that
// read the stage); at the end of a row tile every warp reads back one
// accumulator quarter (a row per thread) and dots it with the rows' own
// compact bits.  A one is encoded as 2^-6 (0x08), so that a nibble spreads to
// four bytes in two instructions; all sums are multiples of 2^-12 below 2^9,
// exact in fp32.

constexpr int kTcThreads = 512;
constexpr int kTcBuilders = 15;            // warps that expand operand tiles; the last warp issues the MMAs
constexpr int kTcM = 128;                  // edges per tile (TMEM lanes); two tiles per pass
constexpr int kTcN = 256;                  // ego rows per tile (TMEM columns per accumulator)
constexpr int kTcK = 64;                   // ego columns per stage: one compact word
constexpr int kTcMaxDeg = 1088;            // largest d_q whose compacted ego network fits shared memory
constexpr int kTcMaxWords = kTcMaxDeg / 64;
constexpr int kTcStageBytes = (2 * kTcM + kTcN) * kTcK;   // A tiles of both edge tiles, then B
constexpr int kTcSmem = 2 * kTcStageBytes + kTcMaxDeg * kTcMaxWords * 8 + 1024;
constexpr long long kTcWaitCycles = 1ll << 30;   // about half a second: a wait that long has failed
static_assert(kTcStageBytes % 1024 == 0, "stage tiles stay 1024-byte aligned");
static_assert(kTcMaxDeg % 64 == 0, "whole compact words");

struct DenseTcArgs {
    DevGraph G;
    const uint64_t *bits;
    const int64_t *wbase;
    const int64_t *vbase;
    const int32_t *dpos;                // positions of the CN-graph edges, grouped by q
    const int64_t *runs;                // per run taken: {first, one past last} position
    const unsigned long long *nruns;
    uint32_t *k4;                       // per position: k4 (left at 0xffffffff outside the runs)
    unsigned long long *next;
    unsigned long long *err;            // waits that ran out
};

// run starts of the CN-graph edges (sorted dense keys: q above the eb
// position bits) whose q has degree in [min_deg, kTcMaxDeg]
__global__ void k_tc_run_flags(const uint64_t *keys, int64_t ncn, const int32_t *deg, int min_deg, uint32_t *flag,
                               int eb) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncn; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t q = (uint32_t)(keys[i] >> eb);
        const bool start = i == 0 || (uint32_t)(keys[i - 1] >> eb) != q;
        const int d = deg[q];
        flag[i] = (start && d >= min_deg && d <= kTcMaxDeg) ? 1u : 0u;
    }
}

// positions of the CN-graph edges whose q's degree is outside [min_deg,
// kTcMaxDeg]: the ones k_dense_cn decomposes, kept in their order
__global__ void k_tc_rest_flags(const uint64_t *keys, int64_t ncn, const int32_t *deg, int min_deg, uint32_t *flag,
                                int eb) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncn; i += (int64_t)gridDim.x * blockDim.x) {
        const int d = deg[(uint32_t)(keys[i] >> eb)];
        flag[i] = (d < min_deg || d > kTcMaxDeg) ? 1u : 0u;
    }
}

__global__ void k_tc_rest_fill(const int32_t *dpos, const uint32_t *flag, const uint32_t *pos, int64_t ncn,
                               int32_t *rest, unsigned long long *nrest) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncn; i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) rest[pos[i]] = dpos[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) *nrest = pos[ncn];
}

__global__ void k_tc_run_fill(const uint64_t *keys, const uint32_t *flag, const uint32_t *pos, int64_t ncn,
                              int64_t *runs, unsigned long long *nruns, int eb) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncn; i += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        const uint32_t q = (uint32_t)(keys[i] >> eb);
        int64_t lo = i + 1, hi = ncn;   // one past the run's last position
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if ((uint32_t)(keys[mid] >> eb) == q) lo = mid + 1; else hi = mid;
        }
        runs[2 * pos[i]] = i;
        runs[2 * pos[i] + 1] = lo;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *nruns = pos[ncn];
}

// masks of the compress of Hacker's Delight §7-4 (bits of x at the set bits of
// m, packed to the low end), for repeated use with one m
__device__ __forceinline__ void tc_compress_masks(uint64_t m, uint64_t mv[6]) {
    uint64_t mk = ~m << 1;
#pragma unroll
    for (int i = 0; i < 6; i++) {
        uint64_t mp = mk ^ (mk << 1);
        mp ^= mp << 2;
        mp ^= mp << 4;
        mp ^= mp << 8;
        mp ^= mp << 16;
        mp ^= mp << 32;
        const uint64_t v = mp & m;
        mv[i] = v;
        m = (m ^ v) | (v >> (1 << i));
        mk &= ~mp;
    }
}

__device__ __forceinline__ uint64_t tc_compress(uint64_t x, uint64_t m, const uint64_t mv[6]) {
    x &= m;
#pragma unroll
    for (int i = 0; i < 6; i++) {
        const uint64_t t = x & mv[i];
        x = (x ^ t) | (t >> (1 << i));
    }
    return x;
}

// four bits -> four e4m3 bytes, 2^-6 (0x08) where the bit is set: the
// product places bit i of nib at bit 8i + 3, and no two shifted copies overlap
__device__ __forceinline__ uint32_t tc_spread4(uint32_t nib) { return (nib * 0x01020408u) & 0x08080808u; }

__global__ void __launch_bounds__(kTcThreads, 1) k_dense_tc(DenseTcArgs A) {
    extern __shared__ uint8_t tc_smem[];
    __shared__ uint64_t s_m[32];          // A_q, per word
    __shared__ uint64_t s_mv[32][6];      // compress masks per word of A_q
    __shared__ int32_t s_o[33];           // compact offset of each word (prefix of popcounts)
    __shared__ uint16_t s_col[kTcMaxDeg]; // N(q), ascending
    __shared__ int16_t s_jrow[2][kTcM];   // compact row of each edge's p in the pass, -1 past the run
    __shared__ float s_part[2][2][kTcM];  // per edge tile and column half
    __shared__ uint32_t s_taddr;
    __shared__ __align__(8) uint64_t s_full[2];
    __shared__ __align__(8) uint64_t s_empty[2];
    __shared__ long long s_run;
    __shared__ int s_abort;
    using namespace pgd_tc;
    const DevGraph &G = A.G;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // 1024-aligned stages, then the compacted ego rows
    uint8_t *base = tc_smem + ((1024u - (smem_addr(tc_smem) & 1023u)) & 1023u);
    uint64_t *C = (uint64_t *)(base + 2 * kTcStageBytes);
    if (warp == 0) tmem_alloc(&s_taddr, 2 * kTcN);
    if (tid == 0) {
        for (int i = 0; i < 2; i++) {
            mbar_init(&s_full[i], kTcBuilders);
            mbar_init(&s_empty[i], 1);
        }
        s_abort = 0;
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = s_taddr;
    // read-back role: edge tile et, column half eh, TMEM lanes 32·(warp & 3)
    const int et = warp >> 3, eh = (warp >> 2) & 1, erow = 32 * (warp & 3) + lane;
    const uint32_t etaddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(et * kTcN);
    const bool issuer = warp == kTcBuilders && lane == 0;
    int chunk = 0;      // chunks so far: chunk c uses stage c & 1 for the (c >> 1)-th time
    int last = -1;      // issuer: the last chunk committed
    bool bad = false;
    const int64_t nruns = (int64_t)*A.nruns;
    while (true) {
        if (tid == 0) s_run = (long long)atomicAdd(A.next, 1ull);
        __syncthreads();
        const int64_t r = s_run;
        __syncthreads();
        if (r >= nruns) break;
        const int64_t i0 = A.runs[2 * r], i1 = A.runs[2 * r + 1];
        const int32_t qg = dense_q(G, A.dpos[i0]);
        const int g = G.egraph[A.dpos[i0]];
        const int64_t vb = A.vbase[g];
        const int W = (int)((G.gnm[2 * g] + 63) >> 6);
        const uint64_t *rows = A.bits + A.wbase[g];
        const int64_t q = qg - vb;
        // the first pass's edges: their other endpoints p, loaded by the upper
        // half of the CTA now, so that the latency of the chain hides under the
        // set-up (warp 0) and the compaction
        const int ptid = tid - (kTcThreads - 2 * kTcM);   // this thread's edge of the first pass, if >= 0
        int pfirst = 0;
        if (ptid >= 0 && ptid < (int)(i1 - i0)) {
            const int32_t id = G.order[A.dpos[i0 + ptid]];
            const int32_t v = G.ev[id], u = G.eu[id];
            pfirst = (int)((v == qg ? u : v) - vb);
        }
        if (warp == 0) {
            const uint64_t mq = lane < W ? __ldg(rows + q * W + lane) : 0ull;
            const int c = __popcll(mq);
            int o = c;
#pragma unroll
            for (int sft = 1; sft < 32; sft <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, o, sft);
                if (lane >= sft) o += y;
            }
            o -= c;
            s_m[lane] = mq;
            s_o[lane] = o;
            if (lane == 31) s_o[32] = o + c;
            uint64_t mv[6];
            tc_compress_masks(mq, mv);
#pragma unroll
            for (int i = 0; i < 6; i++) s_mv[lane][i] = mv[i];
        }
        __syncthreads();
        const int d = s_o[32];   // = deg(q), which the run flags bound; a run beyond the
        if (d > kTcMaxDeg) continue;   // shared-memory limit is left to k_dense_cn
        // compact words per ego row, and the row stride: odd, so that the
        // rows a warp reads together fall in different banks
        const int KW = (d + 63) >> 6, KS = KW | 1;
        // N(q) in ascending order (four bits of A_q per thread) and the compact rows cleared
        for (int t = tid; t < 32 * 16; t += kTcThreads) {
            const int w = t >> 4, b0 = 4 * (t & 15);
            const uint64_t mw = s_m[w];
            uint32_t nib = (uint32_t)(mw >> b0) & 15u;
            int j = s_o[w] + __popcll(mw & ((1ull << b0) - 1));
            while (nib) {
                s_col[j++] = (uint16_t)(64 * w + b0 + __ffs(nib) - 1);
                nib &= nib - 1;
            }
        }
        for (int i = tid; i < d * KS; i += kTcThreads) C[i] = 0ull;
        __syncthreads();
        {   // C[j] = compact(A_{col[j]}), lane = word of the uncompacted row; eight rows in
            // flight.  Lane w's compressed bits start at bit ow of the compact row, in word
            // w0; the lanes starting in one word form a contiguous segment, and only the
            // segment's last lane can spill into the next word.  A segmented OR-scan over
            // the lanes assembles each word in its segment's last lane: no atomics.
            uint64_t mv[6];
#pragma unroll
            for (int i = 0; i < 6; i++) mv[i] = s_mv[lane][i];
            const uint64_t mw = s_m[lane];
            const int ow = s_o[lane], cw = __popcll(mw), sh = ow & 63, w0 = ow >> 6;
            const bool spills = sh && sh + cw > 64;
            const int w0prev = __shfl_up_sync(0xffffffffu, w0, 1), w0next = __shfl_down_sync(0xffffffffu, w0, 1);
            const bool first = lane == 0 || w0prev != w0, lastl = lane == 31 || w0next != w0;
            unsigned same = 0;   // bit i: lane - 2^i is in this lane's segment
#pragma unroll
            for (int i = 0; i < 5; i++) {
                const int o2 = __shfl_up_sync(0xffffffffu, w0, 1 << i);
                if (lane >= (1 << i) && o2 == w0) same |= 1u << i;
            }
            constexpr int kWarps = kTcThreads / 32, kFly = 8;
            for (int jb = warp; jb < d; jb += kFly * kWarps) {
                uint64_t w[kFly];
#pragma unroll
                for (int k = 0; k < kFly; k++) {
                    const int j = jb + k * kWarps;
                    w[k] = (cw && j < d) ? __ldg(rows + (int64_t)s_col[j] * W + lane) : 0ull;
                }
#pragma unroll
                for (int k = 0; k < kFly; k++) {
                    const int j = jb + k * kWarps;   // uniform over the warp
                    if (j >= d) break;
                    const uint64_t v = cw ? tc_compress(w[k], mw, mv) : 0ull;
                    const uint64_t hi = spills ? v >> (64 - sh) : 0ull;
                    const uint64_t hprev = __shfl_up_sync(0xffffffffu, hi, 1);
                    uint64_t val = (v << sh) | (first && lane > 0 ? hprev : 0ull);
#pragma unroll
                    for (int i = 0; i < 5; i++) {
                        const uint64_t t = __shfl_up_sync(0xffffffffu, val, 1 << i);
                        if ((same >> i) & 1u) val |= t;
                    }
                    if (lastl && w0 < KW) C[j * KS + w0] = val;
                    if (lane == 31 && hi) C[j * KS + w0 + 1] = hi;
                }
            }
        }
        const int rr = (int)(i1 - i0);
        for (int m0 = 0; m0 < rr && !bad; m0 += 2 * kTcM) {
            const int ntiles = rr - m0 > kTcM ? 2 : 1;   // edge tiles of this pass
            __syncthreads();   // C complete; the previous pass's s_jrow and s_part read
            if (ptid >= 0) {
                int jr = -1;
                if (m0 + ptid < rr) {
                    int p = pfirst;
                    if (m0 > 0) {
                        const int32_t id = G.order[A.dpos[i0 + m0 + ptid]];
                        const int32_t v = G.ev[id], u = G.eu[id];
                        p = (int)((v == qg ? u : v) - vb);
                    }
                    jr = s_o[p >> 6] + __popcll(s_m[p >> 6] & ((1ull << (p & 63)) - 1));
                }
                s_jrow[ptid >> 7][ptid & (kTcM - 1)] = (int16_t)jr;
            }
            __syncthreads();
            float acc = 0.f;   // row erow of edge tile et, column half eh
            for (int n0 = 0; n0 < d && !bad; n0 += kTcN) {
                const int nt = min(kTcN, ((d - n0 + 15) >> 4) << 4);
                const uint32_t idesc = idesc_e4m3_f32(kTcM, nt);
                // this builder thread's items (16 columns of one row each) of
                // every chunk of this tile: compact source word, shift,
                // destination.  In the core-matrix layout (LBO 128, SBO 512)
                // item i of a tile lives at byte 16·i; a stage holds A of tile
                // 0, A of tile 1, B.
                const int nA = ntiles * kTcM * 4, nItems = nA + nt * 4;
                constexpr int kPer = (2 * kTcM * 4 + kTcN * 4 + 32 * kTcBuilders - 1) / (32 * kTcBuilders);
                if (warp < kTcBuilders) {
                    // per item: its 16 bits of chunk 0 as a halfword of C (chunk kc
                    // is 4·kc halfwords further), and its destination.  Rows past
                    // the run's edges and past d_q are not built: they only feed
                    // accumulator rows and columns that are never read (stale
                    // stage bytes there are harmless: the read-back selects by the
                    // row's bits, which are zero past d_q).
                    const uint16_t *C16 = (const uint16_t *)C;
                    int src[kPer];
                    uint32_t dst[kPer];
#pragma unroll
                    for (int k = 0; k < kPer; k++) {
                        const int it = tid + k * 32 * kTcBuilders;
                        const bool isA = it < nA;
                        const int i2 = isA ? (it & (kTcM * 4 - 1)) : it - nA;
                        const int row = ((i2 >> 5) << 3) | (i2 & 7);
                        int cr = -1;
                        if (it < nItems) cr = isA ? s_jrow[it >> 9][row] : (n0 + row < d ? n0 + row : -1);
                        src[k] = 4 * cr * KS + ((i2 >> 3) & 3);
                        dst[k] = cr < 0 ? 0xffffffffu
                                 : isA ? (uint32_t)((it >> 9) * kTcM * kTcK + 16 * i2)
                                       : (uint32_t)(2 * kTcM * kTcK + 16 * i2);
                    }
                    for (int kc = 0; kc < KW; kc++) {
                        const int c = chunk + kc, st = c & 1, u = c >> 1;
                        // the MMAs that read this stage last (chunk c - 2) are done
                        int ok = 1;
                        if (lane == 0 && u > 0)
                            ok = mbar_wait_or_abort(&s_empty[st], (u - 1) & 1, kTcWaitCycles, &s_abort);
                        bad |= !__shfl_sync(0xffffffffu, ok, 0);
                        uint8_t *stg = base + st * kTcStageBytes;
                        uint32_t b16[kPer];
#pragma unroll
                        for (int k = 0; k < kPer; k++) b16[k] = dst[k] != 0xffffffffu ? C16[src[k] + 4 * kc] : 0u;
#pragma unroll
                        for (int k = 0; k < kPer; k++) {
                            if (dst[k] != 0xffffffffu)
                                *(uint4 *)(stg + dst[k]) =
                                    make_uint4(tc_spread4(b16[k] & 15u), tc_spread4((b16[k] >> 4) & 15u),
                                               tc_spread4((b16[k] >> 8) & 15u), tc_spread4(b16[k] >> 12));
                        }
                        fence_async_smem();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&s_full[st]);
                    }
                } else if (issuer) {
                    for (int kc = 0; kc < KW; kc++) {
                        const int c = chunk + kc, st = c & 1, u = c >> 1;
                        bad |= !mbar_wait_or_abort(&s_full[st], u & 1, kTcWaitCycles, &s_abort);
                        fence_after_sync();
                        const uint32_t sa = smem_addr(base + st * kTcStageBytes), sb = sa + 2 * kTcM * kTcK;
                        for (int t = 0; t < ntiles; t++)
#pragma unroll
                            for (int ks = 0; ks < 2; ks++)
                                mma_e4m3(tmem + (uint32_t)(t * kTcN),
                                         smem_desc(sa + t * kTcM * kTcK + 256 * ks, 128, 512),
                                         smem_desc(sb + 256 * ks, 128, 512), idesc, (kc | ks) != 0);
                        mma_commit(&s_empty[st]);
                        last = c;
                    }
                    // the accumulators are complete once the last commit lands
                    bad |= !mbar_wait_or_abort(&s_empty[last & 1], (last >> 1) & 1, kTcWaitCycles, &s_abort);
                }
                chunk += KW;
                if (__syncthreads_or(bad)) {
                    bad = true;
                    break;
                }
                fence_after_sync();
                if (et < ntiles) {
                    const int jr = s_jrow[et][erow];
                    const int cend = min(nt, eh * 128 + 128);
                    // 32 columns per step: two loads in flight, one wait
                    for (int c0 = eh * 128; c0 < cend; c0 += 32) {
                        uint32_t v[32];
                        const bool two = c0 + 16 < cend;   // nt is a multiple of 16
                        tmem_ld16_async(etaddr + (uint32_t)c0, v);
                        if (two) tmem_ld16_async(etaddr + (uint32_t)(c0 + 16), v + 16);
                        const int y0 = n0 + c0;   // a multiple of 32, below d
                        const uint32_t b32 = jr >= 0 ? (uint32_t)(C[jr * KS + (y0 >> 6)] >> (y0 & 63)) : 0u;
                        tmem_wait_ld();
#pragma unroll
                        for (int i = 0; i < 16; i++) acc += ((b32 >> i) & 1u) ? __uint_as_float(v[i]) : 0.f;
                        if (two) {
#pragma unroll
                            for (int i = 16; i < 32; i++) acc += ((b32 >> i) & 1u) ? __uint_as_float(v[i]) : 0.f;
                        }
                    }
                }
                fence_before_sync();
                __syncthreads();   // accumulators read before the next tile's MMAs
            }
            if (bad) break;
            if (et < ntiles) s_part[et][eh][erow] = acc;
            __syncthreads();
            if (tid < ntiles * kTcM && m0 + tid < rr) {
                const int t = tid >> 7, row = tid & (kTcM - 1);
                // (sum of D·A_py) · 2^12 = 2·k4
                const float k2 = (s_part[t][0][row] + s_part[t][1][row]) * 4096.f;
                A.k4[i0 + m0 + tid] = (uint32_t)k2 >> 1;
            }
        }
        if (bad) break;
    }
    if (bad && issuer) {
        atomicAdd(A.err, 1ull);
        // MMAs still in flight: one more bounded wait for the last commit
        if (last >= 0) mbar_wait(&s_empty[last & 1], (last >> 1) & 1, kTcWaitCycles);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 2 * kTcN);
}

// ---------------------------------------------------------------------------
// The two c4 sums of a dense graph's edges on the tensor cores.  With A the
// adjacency, CN = A² and TA = A ∘ CN (t of each edge, 0 off the edges), an
// edge (p, q) with S_q = N(q) \ N(p) \ {p} and T = N(p) ∩ N(q) has
//   sum_{w in S_q} CN[p][w] = (A·CN)[q][p] - (TA·A)[p][q] - d_p,
//   sum_{x in T}   CN[q][x] = (TA·A)[q][p],
// so their difference is E[q][p] - d_p with the symmetric integer matrix
//   E = A·(CN - TA) - TA·A.
// One CTA per SM takes (graph, 128-row tile, 256-column tile) items; each
// item runs the chain over K = n of A × (CN - TA), then of TA × A with the
// product negated, in tf32 (entries below 2^11 are exact, |sums| < 2^23 stay
// exact in fp32), 16 columns per stage from four stages.  The tile is read
// back one row per thread and E[x][y] written for the edges only, at the
// adjacency slot x -> y.

constexpr int kGramThreads = 512;
constexpr int kGramM = 128, kGramN = 256;
constexpr int kGramStages = 4;
constexpr int kGramStageBytes = (kGramM + kGramN) * 64;   // 16 tf32 columns per row
constexpr int kGramSmem = kGramStages * kGramStageBytes + 1024;
static_assert(kGramStageBytes % 1024 == 0, "stage tiles stay 1024-byte aligned");

struct GramArgs {
    const uint64_t *bits;
    const int64_t *wbase;
    const int64_t *vbase;
    const uint16_t *cn;
    const int64_t *cbase;
    const long long *gnm;
    const int64_t *off;        // union adjacency offsets
    const int64_t *etile;      // first item of each graph (k + 1 entries)
    int k;
    int32_t *eslot;            // E[x][y] per adjacency slot x -> y of the graphs with a CN matrix
    unsigned long long *next;
    unsigned long long *err;
};

__global__ void k_gram_tiles(const long long *gnm, const int64_t *cbase, int k, int64_t *tiles) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g <= k; g += gridDim.x * blockDim.x) {
        int64_t t = 0;
        if (g < k && cbase[g] >= 0) {
            const int64_t n = gnm[2 * g];
            t = ((n + kGramM - 1) / kGramM) * ((n + kGramN - 1) / kGramN);
        }
        tiles[g] = t;
    }
}

__global__ void __launch_bounds__(kGramThreads, 1) k_dense_gram(GramArgs A) {
    extern __shared__ uint8_t gram_smem[];
    __shared__ uint32_t s_taddr;
    __shared__ __align__(8) uint64_t s_bar[kGramStages];
    __shared__ long long s_item;
    using namespace pgd_tc;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *base = gram_smem + ((1024u - (smem_addr(gram_smem) & 1023u)) & 1023u);
    if (warp == 0) tmem_alloc(&s_taddr, kGramN);
    if (tid == 0)
        for (int i = 0; i < kGramStages; i++) mbar_init(&s_bar[i], 1);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = s_taddr;
    // read-back role: TMEM lanes 32·(warp & 3), columns 64·(warp >> 2) ...
    const int lg = warp & 3, cq = warp >> 2;
    const int64_t total = A.etile[A.k];
    uint32_t phase = 0, pend = 0;   // thread 0, per stage
    int chunk = 0;
    bool bad = false;
    while (true) {
        if (tid == 0) s_item = (long long)atomicAdd(A.next, 1ull);
        __syncthreads();
        const int64_t item = s_item;
        __syncthreads();
        if (item >= total) break;
        const int g = batch_find(A.etile, A.k, item);
        const int n = (int)A.gnm[2 * g];
        const int W = (n + 63) >> 6;
        const int64_t stride = (int64_t)W * 64;
        const int tcols = (n + kGramN - 1) / kGramN;
        const int local = (int)(item - A.etile[g]);
        const int i0 = (local / tcols) * kGramM, j0 = (local % tcols) * kGramN;
        const int nt = min(kGramN, ((n - j0 + 15) >> 4) << 4);
        const uint64_t *rows = A.bits + A.wbase[g];
        const uint16_t *cng = A.cn + A.cbase[g];
        const int nK = (n + 15) >> 4;
        const uint32_t id_pos = idesc_tf32_f32(kGramM, nt, false), id_neg = idesc_tf32_f32(kGramM, nt, true);
        // this thread's items (4 columns of one row each, 16 bytes): A tile
        // items 0..511, B tile items after them; in the core-matrix layout
        // (LBO 128, SBO 512) item i of a tile lives at byte 16·i
        const int nItems = kGramM * 4 + nt * 4;
        int grow[3], gblk[3];
        uint32_t dst[3];
        bool isA[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int it = tid + k * kGramThreads;
            isA[k] = it < kGramM * 4;
            const int i2 = isA[k] ? it : it - kGramM * 4;
            const int row = ((i2 >> 5) << 3) | (i2 & 7);
            const int r = isA[k] ? i0 + row : j0 + row;
            grow[k] = (it < nItems && r < n) ? r : -1;
            gblk[k] = (i2 >> 3) & 3;
            dst[k] = isA[k] ? (uint32_t)(16 * i2) : (uint32_t)(kGramM * 64 + 16 * i2);
        }
        // the global words of one chunk's items: the bit-row word and, where the
        // item takes CN, its four entries; loaded one chunk ahead
        auto fetch = [&](int ch, uint64_t *bw, uint64_t *cw) {
            const bool second = ch >= nK;
            const int kc = second ? ch - nK : ch;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                bw[k] = cw[k] = 0ull;
                if (tid + k * kGramThreads < nItems && grow[k] >= 0) {
                    const int k0 = kc * 16 + gblk[k] * 4;   // first column, below 64·W
                    bw[k] = rows[(int64_t)grow[k] * W + (k0 >> 6)];
                    if (isA[k] == second) cw[k] = *(const uint64_t *)(cng + (int64_t)grow[k] * stride + k0);
                }
            }
        };
        uint64_t pbw[3], pcw[3];
        fetch(0, pbw, pcw);
        for (int ch = 0; ch < 2 * nK; ch++) {
            const bool second = ch >= nK;   // TA x A, negated
            const int kc = second ? ch - nK : ch;
            const int st = chunk % kGramStages;
            uint8_t *stg = base + st * kGramStageBytes;
            uint64_t nbw[3] = {0ull, 0ull, 0ull}, ncw[3] = {0ull, 0ull, 0ull};
            if (ch + 1 < 2 * nK) fetch(ch + 1, nbw, ncw);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                if (tid + k * kGramThreads >= nItems) continue;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (grow[k] >= 0) {
                    const int k0 = kc * 16 + gblk[k] * 4;
                    const uint32_t b4 = (uint32_t)(pbw[k] >> (k0 & 63)) & 15u;
                    // A x (CN - TA): A side bits, B side CN off the edges;
                    // TA x A: A side CN on the edges, B side bits
                    if (isA[k] == second) {
                        const uint64_t c4 = pcw[k];
                        const uint32_t keep = second ? b4 : ~b4;
                        v.x = (keep & 1u) ? __float_as_uint((float)(uint32_t)(c4 & 0xffffu)) : 0u;
                        v.y = (keep & 2u) ? __float_as_uint((float)(uint32_t)((c4 >> 16) & 0xffffu)) : 0u;
                        v.z = (keep & 4u) ? __float_as_uint((float)(uint32_t)((c4 >> 32) & 0xffffu)) : 0u;
                        v.w = (keep & 8u) ? __float_as_uint((float)(uint32_t)(c4 >> 48)) : 0u;
                    } else {
                        v.x = (b4 & 1u) ? 0x3f800000u : 0u;
                        v.y = (b4 & 2u) ? 0x3f800000u : 0u;
                        v.z = (b4 & 4u) ? 0x3f800000u : 0u;
                        v.w = (b4 & 8u) ? 0x3f800000u : 0u;
                    }
                }
                *(uint4 *)(stg + dst[k]) = v;
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                pbw[k] = nbw[k];
                pcw[k] = ncw[k];
            }
            fence_async_smem();
            __syncthreads();   // stage st written
            if (tid == 0) {
                fence_after_sync();
                const uint32_t sa = smem_addr(stg), sb = sa + kGramM * 64;
#pragma unroll
                for (int ks = 0; ks < 2; ks++)
                    mma_tf32(tmem, smem_desc(sa + 256 * ks, 128, 512), smem_desc(sb + 256 * ks, 128, 512),
                             second ? id_neg : id_pos, (ch | ks) != 0);
                mma_commit(&s_bar[st]);
                pend |= 1u << st;
                // the next chunk's stage must be free: its MMAs (kGramStages - 1 chunks ago) done
                const int nx = (chunk + 1) % kGramStages;
                if ((pend >> nx) & 1u) {
                    bad |= !mbar_wait(&s_bar[nx], (phase >> nx) & 1u, kTcWaitCycles);
                    phase ^= 1u << nx;
                    pend &= ~(1u << nx);
                }
            }
            chunk++;
            if (__syncthreads_or(bad)) {
                bad = true;
                break;
            }
        }
        if (bad) break;
        if (tid == 0)
            for (int st = 0; st < kGramStages; st++)
                if ((pend >> st) & 1u) {
                    bad |= !mbar_wait(&s_bar[st], (phase >> st) & 1u, kTcWaitCycles);
                    phase ^= 1u << st;
                    pend &= ~(1u << st);
                }
        if (__syncthreads_or(bad)) {
            bad = true;
            break;
        }
        fence_after_sync();
        if (cq * 64 < nt) {
            const int i = i0 + 32 * lg + lane;
            const int jw = (j0 + cq * 64) >> 6;   // the columns' word of row i
            uint64_t word = 0;
            int64_t slot = 0;
            if (i < n) {
                const uint64_t *ri = rows + (int64_t)i * W;
                word = ri[jw];
                int before = 0;
                for (int w = 0; w < jw; w++) before += __popcll(ri[w]);
                slot = A.off[A.vbase[g] + i] + before;
            }
            for (int c0 = 0; c0 < 64 && cq * 64 + c0 < nt; c0 += 16) {
                uint32_t v[16];
                tmem_ld16(tmem + ((uint32_t)(32 * lg) << 16) + (uint32_t)(cq * 64 + c0), v);
#pragma unroll
                for (int e = 0; e < 16; e++)
                    if ((word >> (c0 + e)) & 1ull) A.eslot[slot++] = (int32_t)__uint_as_float(v[e]);
            }
        }
        fence_before_sync();
        __syncthreads();   // accumulator read before the next item's MMAs
    }
    if (bad && tid == 0) {
        atomicAdd(A.err, 1ull);
        for (int st = 0; st < kGramStages; st++)
            if ((pend >> st) & 1u) mbar_wait(&s_bar[st], (phase >> st) & 1u, kTcWaitCycles);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kGramN);
}

// The edges of the runs k_dense_tc took, one per lane: t = CN[p][q],
// |S_q| = d_q - t - 1, k4 from k_dense_tc, the two c4 sums from E as
// E[q][p] - d_p (the slot q -> p: p's rank in N(q) from A_q's popcounts),
// then the closed forms and the per-edge row.  A warp takes a run at a time.
struct DenseCloseArgs {
    DevGraph G;
    const uint64_t *bits;
    const int64_t *wbase;
    const int64_t *vbase;
    const uint16_t *cn;
    const int64_t *cbase;
    const int32_t *dpos;
    const int64_t *runs;
    const unsigned long long *nruns;
    const uint32_t *k4;
    const int32_t *eslot;
    unsigned long long *next;
};

// a warp's per-lane sums of graph g, reduced and added to the graph's sums
__device__ __forceinline__ void warp_flush_graph(const DevGraph &G, unsigned long long *acc, int g, int lane) {
#pragma unroll
    for (int i = 0; i < PGD_NSUMS; i++) {
        const unsigned long long v = pgd_warp_sum(acc[i]);
        if (lane == 0 && v) atomicAdd(G.sums + (int64_t)g * PGD_NSUMS + i, v);
        acc[i] = 0;
    }
}

__global__ void __launch_bounds__(256) k_dense_close(DenseCloseArgs A) {
    const DevGraph &G = A.G;
    const int lane = threadIdx.x & 31;
    int cur_g = -1;
    unsigned long long acc[PGD_NSUMS];
#pragma unroll
    for (int i = 0; i < PGD_NSUMS; i++) acc[i] = 0;
    const unsigned long long nruns = *A.nruns;
    while (true) {
        unsigned long long r = 0;
        if (lane == 0) r = atomicAdd(A.next, 1ull);
        r = __shfl_sync(0xffffffffu, r, 0);
        if (r >= nruns) break;
        const int64_t i0 = A.runs[2 * r], i1 = A.runs[2 * r + 1];
        const int32_t qg = dense_q(G, A.dpos[i0]);
        const int g = G.egraph[A.dpos[i0]];
        if (g != cur_g) {
            if (cur_g >= 0) warp_flush_graph(G, acc, cur_g, lane);
            cur_g = g;
        }
        const int64_t vb = A.vbase[g];
        const long long n = G.gnm[2 * g], m = G.gnm[2 * g + 1];
        const int W = (int)((n + 63) >> 6);
        const int64_t stride = (int64_t)W * 64;
        const uint64_t *rows = A.bits + A.wbase[g];
        const uint16_t *cnb = A.cn + A.cbase[g];
        const int64_t q = qg - vb;
        const uint64_t Aq = lane < W ? __ldg(rows + q * W + lane) : 0ull;
        const int c = __popcll(Aq);
        int o = c;
#pragma unroll
        for (int sft = 1; sft < 32; sft <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, o, sft);
            if (lane >= sft) o += y;
        }
        o -= c;
        const int64_t qoff = G.off[qg];
        const long long dq = G.deg[qg];
        for (int64_t b = i0; b < i1; b += 32) {
            const int64_t i = b + lane;
            const bool act = i < i1;
            int64_t e = 0;
            int32_t v = 0, u = 0, pl = 0;
            if (act) {
                e = A.dpos[i];
                const int32_t id = G.order[e];
                v = G.ev[id];
                u = G.eu[id];
                pl = (int32_t)((v == qg ? u : v) - vb);
            }
            const int pw = pl >> 6;
            const uint64_t aw = __shfl_sync(0xffffffffu, Aq, pw);
            const int ow = __shfl_sync(0xffffffffu, o, pw);
            if (act) {
                const int rank = ow + __popcll(aw & ((1ull << (pl & 63)) - 1));
                const unsigned long long t = cnb[(int64_t)pl * stride + q];
                const unsigned long long k4 = A.k4[i];
                const unsigned long long dsum =
                    (unsigned long long)(long long)(A.eslot[qoff + rank] - G.deg[vb + pl]);
                const unsigned long long nsq = (unsigned long long)(dq - (long long)t - 1);
                const unsigned long long c4 = dsum + 2 * k4 + t - nsq;
                const long long dv = G.deg[v], du = G.deg[u];
                pgd_edge_sums(acc, dv, du, t, m, n);
                acc[3] += k4;
                acc[4] += c4;
                if (G.micro) {
#pragma unroll
                    for (int col = 0; col < PGD_NMICRO; col++)
                        G.micro[e * PGD_NMICRO + col] = pgd_micro_col(col, dv, du, t, k4, c4);
                }
            }
        }
    }
    if (cur_g >= 0) warp_flush_graph(G, acc, cur_g, lane);
}

}  // namespace

// ---------------------------------------------------------------------------

// Stream-ordered temporaries released on every return path (also when an
// allocation or a CUDA call fails half-way).
struct TmpGuard {
    pgd_ctx *ctx;
    std::vector<void *> held;
    explicit TmpGuard(pgd_ctx *c) : ctx(c) {}
    TmpGuard(const TmpGuard &) = delete;
    TmpGuard &operator=(const TmpGuard &) = delete;
    ~TmpGuard() {
        for (void *p : held) pgd_tmp_free(ctx, p);
    }
    template <typename T>
    pgd_status alloc(T **out, size_t bytes) {
        void *p = nullptr;
        const pgd_status st = pgd_tmp_alloc(ctx, &p, bytes);
        if (st == PGD_OK) {
            held.push_back(p);
            *out = (T *)p;
        }
        return st;
    }
};

static pgd_status build_aux(pgd_graph *g) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    const int64_t n = g->n, nnz = 2 * g->m;
    if (!g->offp) {
        if ((st = pgd_graph_alloc(g, (void **)&g->offp, (n + 1) * sizeof(int64_t)))) return st;
        if ((st = pgd_graph_alloc(g, (void **)&g->adjp, (g->m + 1) * sizeof(int32_t)))) return st;
        if ((st = pgd_graph_alloc(g, (void **)&g->vrank, (n + 1) * sizeof(int32_t)))) return st;
        if ((st = pgd_graph_alloc(g, (void **)&g->adjp_rank, (g->m + 1) * sizeof(int32_t)))) return st;
        if ((st = pgd_graph_alloc(g, (void **)&g->hubid, (n + 1) * sizeof(int32_t)))) return st;
        if ((st = pgd_graph_alloc(g, (void **)&g->slot, (nnz + 1) * sizeof(int4)))) return st;
        if ((st = pgd_graph_alloc(g, (void **)&g->adj_rank, (nnz + 1) * sizeof(int32_t)))) return st;
        if ((st = pgd_graph_alloc(g, (void **)&g->offh, (n + 1) * sizeof(int64_t)))) return st;
        if ((st = pgd_graph_alloc(g, (void **)&g->vrec, (n + 1) * 32))) return st;
        g->top_r = (int32_t)std::min<int64_t>(n, kRankBits);
        g->top_words = top_row_base(g->top_r);
        if ((st = pgd_graph_alloc(g, (void **)&g->toprows, (g->top_words + 1) * sizeof(uint32_t)))) return st;
    }
    TmpGuard tg(ctx);
    int32_t *row = nullptr;
    uint32_t *flag = nullptr, *pos = nullptr;
    const int64_t len = std::max(nnz, n) + 1;
    if ((st = tg.alloc(&row, (nnz + 1) * sizeof(int32_t)))) return st;
    if ((st = tg.alloc(&flag, len * sizeof(uint32_t)))) return st;
    if ((st = tg.alloc(&pos, len * sizeof(uint32_t)))) return st;
    void *tmp = nullptr;
    size_t tb = 0;
    // oriented lists
    PGD_LAUNCH(ctx, k_rows, grid_for(nnz), kThreads, 0, g->off, n, nnz, row);
    PGD_LAUNCH(ctx, k_oriented_flags, grid_for(nnz), kThreads, 0, row, g->adj, g->deg, nnz, flag);
    PGD_CUDA(ctx, cudaMemsetAsync(flag + nnz, 0, sizeof(uint32_t), s));
    cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, pos, nnz + 1, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, nnz + 1, s);
    pgd_tmp_free(ctx, tmp);
    PGD_LAUNCH(ctx, k_oriented_fill, grid_for(std::max(nnz, n + 1)), kThreads, 0, g->off, g->adj, flag, pos, n, nnz,
               g->offp, g->adjp);
    // hub ids, wide tier first
    uint32_t *flag_b = nullptr, *pos_b = nullptr;
    if ((st = tg.alloc(&flag_b, (n + 1) * sizeof(uint32_t)))) return st;
    if ((st = tg.alloc(&pos_b, (n + 1) * sizeof(uint32_t)))) return st;
    PGD_LAUNCH(ctx, k_hub_tier_flags, grid_for(n), kThreads, 0, g->deg, n, ctx->cache_hub, kWideHub, flag, flag_b);
    PGD_CUDA(ctx, cudaMemsetAsync(flag + n, 0, sizeof(uint32_t), s));
    PGD_CUDA(ctx, cudaMemsetAsync(flag_b + n, 0, sizeof(uint32_t), s));
    tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, pos, n + 1, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, n + 1, s);
    cub::DeviceScan::ExclusiveSum(tmp, tb, flag_b, pos_b, n + 1, s);
    pgd_tmp_free(ctx, tmp);
    PGD_LAUNCH(ctx, k_hub_tier_ids, grid_for(n), kThreads, 0, flag, pos, flag_b, pos_b, n, g->hubid);
    uint32_t nh_a = 0, nh_b = 0;
    PGD_CUDA(ctx, cudaMemcpyAsync(&nh_a, pos + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaMemcpyAsync(&nh_b, pos_b + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    // hub-neighbour lists (their length depends on the hub threshold)
    PGD_LAUNCH(ctx, k_hubnb_flags, grid_for(nnz), kThreads, 0, g->adj, g->hubid, nnz, flag);
    PGD_CUDA(ctx, cudaMemsetAsync(flag + nnz, 0, sizeof(uint32_t), s));
    tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, pos, nnz + 1, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, nnz + 1, s);
    pgd_tmp_free(ctx, tmp);
    {
        uint32_t nadjh = 0;
        PGD_CUDA(ctx, cudaMemcpyAsync(&nadjh, pos + nnz, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        PGD_CUDA(ctx, cudaStreamSynchronize(s));
        pgd_graph_free(g, g->adjh, (g->nadjh + 1) * sizeof(int32_t));
        g->adjh = nullptr;
        g->nadjh = nadjh;
        if ((st = pgd_graph_alloc(g, (void **)&g->adjh, (g->nadjh + 1) * sizeof(int32_t)))) return st;
    }
    PGD_LAUNCH(ctx, k_hubnb_fill, grid_for(std::max(nnz, n + 1)), kThreads, 0, g->off, g->adj, g->hubid, flag, pos, n,
               nnz, g->offh, g->adjh);
    // degree ranks of the vertices and of the oriented list entries
    {
        uint64_t *rk = nullptr, *rk2 = nullptr;
        if ((st = tg.alloc(&rk, (n + 1) * sizeof(uint64_t)))) return st;
        if ((st = tg.alloc(&rk2, (n + 1) * sizeof(uint64_t)))) return st;
        if (n > 0) {
            PGD_LAUNCH(ctx, k_rank_keys, grid_for(n), kThreads, 0, g->deg, n, rk);
            tb = 0;
            cub::DeviceRadixSort::SortKeys(nullptr, tb, rk, rk2, n, 0, 64, s);
            if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
            cub::DeviceRadixSort::SortKeys(tmp, tb, rk, rk2, n, 0, 64, s);
            pgd_tmp_free(ctx, tmp);
            PGD_LAUNCH(ctx, k_rank_scatter, grid_for(n), kThreads, 0, rk2, n, g->vrank);
        }
        if (g->m > 0) {
            PGD_LAUNCH(ctx, k_gather_rank, grid_for(g->m), kThreads, 0, g->adjp, g->vrank, g->m, g->adjp_rank);
            PGD_LAUNCH(ctx, k_gather_rank, grid_for(nnz), kThreads, 0, g->adj, g->vrank, nnz, g->adj_rank);
        }
    }
    if (n > 0)
        PGD_LAUNCH(ctx, k_vrec, grid_for(n), kThreads, 0, g->off, g->offp, g->deg, g->vrank, g->hubid, n,
                   (int4 *)g->vrec);
    if (nnz > 0)
        PGD_LAUNCH(ctx, k_slot_fill, grid_for(nnz), kThreads, 0, g->adj, g->vrank, g->hubid, g->offp, nnz, g->top_r,
                   (int4 *)g->slot);
    // rank-bitmap rows of the highest-ranked vertices (ranks do not depend on
    // the thresholds, so a rebuild for new thresholds recomputes the same rows)
    PGD_CUDA(ctx, cudaMemsetAsync(g->toprows, 0, (g->top_words + 1) * sizeof(uint32_t), s));
    if (g->top_r > 0 && g->m > 0)
        PGD_LAUNCH(ctx, k_top_rows, grid_for(32 * n), kThreads, 0, g->offp, g->adjp_rank, g->vrank, n, g->top_r,
                   g->toprows);
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    g->nhubs = (int32_t)(nh_a + nh_b);
    g->nhubs_wide = (int32_t)nh_a;
    PGD_CUDA(ctx, cudaGetLastError());
    g->aux_cache_hub = ctx->cache_hub;
    g->has_aux = true;
    return PGD_OK;
}

static DevGraph dev_view(pgd_graph *g, bool micro) {
    DevGraph G;
    G.off = g->off;
    G.adj = g->adj;
    G.deg = g->deg;
    G.offp = g->offp;
    G.adjp = g->adjp;
    G.hubid = g->hubid;
    G.slot = (const int4 *)g->slot;
    G.ev = g->ev;
    G.eu = g->eu;
    G.order = g->order;
    G.n = g->n;
    G.m = g->m;
    G.npos = g->norder;
    G.micro = micro ? g->micro : nullptr;
    G.sums = g->ctx->d_sums;
    G.egraph = nullptr;
    G.gnm = nullptr;
    G.gdense = nullptr;
    G.vrank = g->vrank;
    G.adjp_rank = g->adjp_rank;
    G.adj_rank = g->adj_rank;
    G.offh = g->offh;
    G.adjh = g->adjh;
    G.toprows = g->toprows;
    G.vrec = (const int4 *)g->vrec;
    G.top_r = g->top_r;
    G.anchor_hub = g->ctx->anchor_hub;
    return G;
}

// Triangle pass, work plan and both decomposition kernels for the graph view
// G (one graph, or the union of a batch); *ms gets their device time.
struct DenseView {
    const uint64_t *bits;
    const int64_t *wbase;
    const int64_t *vbase;
    const uint16_t *cn;       // common-neighbour matrices (null: none)
    const int64_t *cbase;     // per graph: first CN entry, or -1
    int ngraphs;
};

// The tensor-core part of the CN-graph edges: k4 of the runs whose q has
// degree in [ctx->tc_min_deg, kTcMaxDeg] (k_dense_tc: runs of equal q from
// the sorted dense keys, one CTA per SM) and E of every CN graph
// (k_dense_gram).  out->k4 gets k4 per position of dpos (0xffffffff outside
// those runs), out->eslot E per adjacency slot, out->runs the runs.  ctr[8..10]: run counter, run
// count and failed-wait count; ctr[11]: the run counter of k_dense_close;
// ctr[12]: the item counter of k_dense_gram; ctr[13]: the count of positions
// left to k_dense_cn (out->rest, out->nrest).
struct TcOut {
    uint32_t *k4 = nullptr;
    int32_t *eslot = nullptr;
    int64_t *runs = nullptr;
    const unsigned long long *nruns = nullptr;
    int32_t *rest = nullptr;    // positions left to k_dense_cn, in dpos order
    int64_t nrest = 0;
};

static pgd_status dense_tc(pgd_ctx *ctx, const DevGraph &G, TmpGuard &tg, const DenseView *dense,
                           const int32_t *dpos, const uint64_t *keys, int64_t ncn, int eb, TcOut *out) {
    cudaStream_t s = ctx->stream;
    pgd_status st;
    uint32_t *flag = nullptr, *pos = nullptr, *k4 = nullptr;
    int64_t *runs = nullptr;
    const int64_t maxruns = std::min<int64_t>(ncn, G.n);
    if ((st = tg.alloc(&flag, (ncn + 1) * sizeof(uint32_t)))) return st;
    if ((st = tg.alloc(&pos, (ncn + 1) * sizeof(uint32_t)))) return st;
    if ((st = tg.alloc(&k4, ncn * sizeof(uint32_t)))) return st;
    if ((st = tg.alloc(&runs, (2 * maxruns + 2) * sizeof(int64_t)))) return st;
    unsigned long long *ctr = ctx->d_ctr;
    PGD_CUDA(ctx, cudaMemsetAsync(ctr + 8, 0, 6 * sizeof(unsigned long long), s));
    PGD_LAUNCH(ctx, k_tc_run_flags, grid_for(ncn), kThreads, 0, keys, ncn, G.deg, ctx->tc_min_deg, flag, eb);
    PGD_CUDA(ctx, cudaMemsetAsync(flag + ncn, 0, sizeof(uint32_t), s));
    size_t tb = 0;
    void *tmp = nullptr;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, pos, ncn + 1, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, ncn + 1, s);
    pgd_tmp_free(ctx, tmp);
    PGD_LAUNCH(ctx, k_tc_run_fill, grid_for(ncn), kThreads, 0, keys, flag, pos, ncn, runs, ctr + 9, eb);
    PGD_CUDA(ctx, cudaMemsetAsync(k4, 0xff, ncn * sizeof(uint32_t), s));
    PGD_CUDA(ctx, cudaFuncSetAttribute(k_dense_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    DenseTcArgs T;
    T.G = G;
    T.bits = dense->bits;
    T.wbase = dense->wbase;
    T.vbase = dense->vbase;
    T.dpos = dpos;
    T.runs = runs;
    T.nruns = ctr + 9;
    T.k4 = k4;
    T.next = ctr + 8;
    T.err = ctr + 10;
    PGD_LAUNCH(ctx, k_dense_tc, ctx->num_sms, kTcThreads, kTcSmem, T);
    // E of every CN graph: (graph, row tile, column tile) items
    const int k = dense->ngraphs;
    int64_t *tiles = nullptr, *etile = nullptr;
    int32_t *eslot = nullptr;
    if ((st = tg.alloc(&tiles, ((size_t)k + 1) * sizeof(int64_t)))) return st;
    if ((st = tg.alloc(&etile, ((size_t)k + 1) * sizeof(int64_t)))) return st;
    if ((st = tg.alloc(&eslot, ((size_t)2 * G.m + 1) * sizeof(int32_t)))) return st;
    PGD_LAUNCH(ctx, k_gram_tiles, grid_for(k + 1), kThreads, 0, G.gnm, dense->cbase, k, tiles);
    tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, tiles, etile, k + 1, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    cub::DeviceScan::ExclusiveSum(tmp, tb, tiles, etile, k + 1, s);
    pgd_tmp_free(ctx, tmp);
    PGD_CUDA(ctx, cudaFuncSetAttribute(k_dense_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, kGramSmem));
    GramArgs E;
    E.bits = dense->bits;
    E.wbase = dense->wbase;
    E.vbase = dense->vbase;
    E.cn = dense->cn;
    E.cbase = dense->cbase;
    E.gnm = G.gnm;
    E.off = G.off;
    E.etile = etile;
    E.k = k;
    E.eslot = eslot;
    E.next = ctr + 12;
    E.err = ctr + 10;
    PGD_LAUNCH(ctx, k_dense_gram, ctx->num_sms, kGramThreads, kGramSmem, E);
    // the positions left to k_dense_cn (flag and pos arrays reused)
    int32_t *rest = nullptr;
    if ((st = tg.alloc(&rest, (ncn + 1) * sizeof(int32_t)))) return st;
    PGD_LAUNCH(ctx, k_tc_rest_flags, grid_for(ncn), kThreads, 0, keys, ncn, G.deg, ctx->tc_min_deg, flag, eb);
    PGD_CUDA(ctx, cudaMemsetAsync(flag + ncn, 0, sizeof(uint32_t), s));
    tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, pos, ncn + 1, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, ncn + 1, s);
    pgd_tmp_free(ctx, tmp);
    PGD_LAUNCH(ctx, k_tc_rest_fill, grid_for(ncn), kThreads, 0, dpos, flag, pos, ncn, rest, ctr + 13);
    unsigned long long nrest = 0;
    PGD_CUDA(ctx, cudaMemcpyAsync(&nrest, ctr + 13, sizeof(nrest), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    out->k4 = k4;
    out->eslot = eslot;
    out->runs = runs;
    out->nruns = ctr + 9;
    out->rest = rest;
    out->nrest = (int64_t)nrest;
    return PGD_OK;
}

// Where k_hub keeps the W histogram and the N(p) rank bitmap: the histogram
// (atomics) in shared memory when it fits, then as many bitmap ranks as the
// remaining shared memory holds; per-CTA global slices for the rest.  Fills
// the layout fields of H and returns the dynamic shared memory size.
static size_t hub_layout(int64_t n, int32_t nhubs, int32_t nwide, int32_t max_degree, HubArgs *H) {
    H->thigh = nullptr;
    H->twin = nullptr;
    H->twin_words = 0;
    H->nwords = (n + 31) / 32;
    H->nhubs = nhubs;
    H->nwide = nwide;
    H->hist16 = max_degree < 65536 ? 1 : 0;
    H->wide_words = H->hist16 ? ((int64_t)nwide + 1) / 2 : (int64_t)nwide;
    const int64_t hwords = H->wide_words + ((int64_t)(nhubs - nwide) + 3) / 4;
    H->hstride = std::max<int64_t>(4, (hwords + 3) & ~(int64_t)3);
    H->smem_hist = H->hstride * 4 <= kMaxDynSmem ? 1 : 0;
    const int64_t rem_words = kMaxDynSmem / 4 - (H->smem_hist ? H->hstride : 0);
    const int64_t bm_words = std::min<int64_t>(H->nwords, rem_words);
    H->split = (int32_t)std::min<int64_t>(bm_words * 32, 0x7fffffe0);
    return (size_t)((H->smem_hist ? H->hstride : 0) + bm_words) * 4;
}

// Device times of one decomposition: all kernels, the triangle pass, k_hub.
struct StageMs {
    float total = 0, tri = 0, hub = 0;
};

// The work plan of the positions G.order[0..G.npos): hub-anchored positions
// grouped by anchor into work items (with their {position, q} records), then
// dense-graph positions, then light ones (posv).
struct Plan {
    int32_t *posv = nullptr;
    unsigned long long nh = 0, nd = 0;
    int64_t nlight = 0, nitems = 0;
    int64_t *items = nullptr;
    int2 *hrec = nullptr;
};

// bits that hold every value below x (at least one)
static int bits_for(int64_t x) {
    int b = 1;
    while (b < 63 && (int64_t(1) << b) < x) b++;
    return b;
}

static pgd_status build_plan(pgd_ctx *ctx, const DevGraph &G, TmpGuard &tg, Plan *P, uint64_t **keys_out = nullptr,
                             int32_t **vals_out = nullptr, uint64_t **keys2_out = nullptr) {
    cudaStream_t s = ctx->stream;
    pgd_status st;
    const int64_t m = G.npos;
    uint64_t *keys = nullptr, *keys2 = nullptr;
    int32_t *vals = nullptr;
    uint32_t *flag = nullptr, *fpos = nullptr;
    if ((st = tg.alloc(&keys, m * sizeof(uint64_t)))) return st;
    if ((st = tg.alloc(&keys2, m * sizeof(uint64_t)))) return st;
    if ((st = tg.alloc(&P->posv, m * sizeof(int32_t)))) return st;
    if ((st = tg.alloc(&vals, m * sizeof(int32_t)))) return st;
    // [0] hub edges, [1] hub item counter, [2] light counter, [3] dense edges, [4] dense counter,
    // [5] triangle-pass item counter
    unsigned long long *ctr = ctx->d_ctr;
    PGD_CUDA(ctx, cudaMemsetAsync(ctr, 0, 8 * sizeof(unsigned long long), s));
    const int eb = bits_for(m), end_bit = eb + bits_for(G.n + 2);
    PGD_LAUNCH(ctx, k_plan_keys, grid_for(m), kThreads, 0, G, keys, vals, ctr, eb);
    unsigned long long cnt[4] = {0, 0, 0, 0};
    PGD_CUDA(ctx, cudaMemcpyAsync(cnt, ctr, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    P->nh = cnt[0];
    P->nd = cnt[3];
    P->nlight = m - (int64_t)P->nh - (int64_t)P->nd;
    size_t tb = 0;
    void *tmp = nullptr;
    if (P->nd == (unsigned long long)m) {
        // every position is a dense-graph edge: the sorted order is the identity
        PGD_CUDA(ctx, cudaMemcpyAsync(P->posv, vals, m * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    } else {
        cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, keys2, vals, P->posv, m, 0, end_bit, s);
        if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
        cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, P->posv, m, 0, end_bit, s);
        pgd_tmp_free(ctx, tmp);
    }
    const unsigned long long nh = P->nh;
    if (nh > 0) {
        if ((st = tg.alloc(&flag, (nh + 1) * sizeof(uint32_t)))) return st;
        if ((st = tg.alloc(&fpos, (nh + 1) * sizeof(uint32_t)))) return st;
        PGD_LAUNCH(ctx, k_item_flags, grid_for(nh), kThreads, 0, keys2, (int64_t)nh, flag, eb);
        PGD_CUDA(ctx, cudaMemsetAsync(flag + nh, 0, sizeof(uint32_t), s));
        tb = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, fpos, (int64_t)nh + 1, s);
        if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
        cub::DeviceScan::ExclusiveSum(tmp, tb, flag, fpos, (int64_t)nh + 1, s);
        pgd_tmp_free(ctx, tmp);
        uint32_t ni = 0;
        PGD_CUDA(ctx, cudaMemcpyAsync(&ni, fpos + nh, sizeof(ni), cudaMemcpyDeviceToHost, s));
        PGD_CUDA(ctx, cudaStreamSynchronize(s));
        P->nitems = ni;
        if ((st = tg.alloc(&P->items, (P->nitems + 1) * sizeof(int64_t)))) return st;
        PGD_LAUNCH(ctx, k_item_fill, grid_for(nh), kThreads, 0, flag, fpos, (int64_t)nh, P->items);
        if ((st = tg.alloc(&P->hrec, (nh + 1) * sizeof(int2)))) return st;
        PGD_LAUNCH(ctx, k_hub_recs, grid_for(nh), kThreads, 0, G, P->posv, (int64_t)nh, P->hrec);
    }
    if (keys_out) *keys_out = keys;
    if (vals_out) *vals_out = vals;
    if (keys2_out) *keys2_out = keys2;
    return PGD_OK;
}

// t of the edges of a plan, written to both slots of each: hub-anchored
// edges grouped by anchor (k_tslot_hub), the rest one warp each.
static pgd_status triangle_pass(pgd_ctx *ctx, const DevGraph &G, int4 *slot, const Plan &P, const HubArgs &H,
                                uint32_t *gbm) {
    const int nsm = ctx->num_sms;
    if (P.nitems > 0) {
        HubArgs T = H;
        T.G = G;
        T.hrec = P.hrec;
        T.items = P.items;
        T.nitems = P.nitems;
        T.gbitmap = gbm;
        T.next = ctx->d_ctr + 5;
        T.slot_out = slot;
        // the whole dynamic shared memory holds bitmap ranks (no histogram here)
        const int64_t tw = std::min<int64_t>(H.nwords, kMaxTslotSmem / 4);
        T.split = (int32_t)std::min<int64_t>(tw * 32, 0x7fffffe0);
        PGD_CUDA(ctx, cudaFuncSetAttribute(k_tslot_hub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(tw * 4)));
        PGD_LAUNCH(ctx, k_tslot_hub, nsm, kHubWarps * 32, (size_t)(tw * 4), T);
    }
    if (P.nlight > 0)
        PGD_LAUNCH(ctx, k_tslot, grid_for(32 * P.nlight), kThreads, 0, G, slot, P.posv + P.nh + P.nd, P.nlight);
    return PGD_OK;
}

__global__ void k_iota(int32_t *a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = (int32_t)i;
}

static pgd_status run_decompose(pgd_ctx *ctx, const DevGraph &G, int4 *slot, int32_t nhubs, int32_t nwide,
                                int32_t max_degree,
                                StageMs *ms, const DenseView *dense = nullptr) {
    cudaStream_t s = ctx->stream;
    pgd_status st;
    const int64_t m = G.npos;   // positions to decompose (E_ordered length)
    *ms = StageMs();
    if (m == 0) return PGD_OK;
    // a sampled order decomposes some edges but reads t(x, q) of any edge
    const bool sampled = G.npos < G.m;
    uint32_t *ghist = nullptr;
    uint32_t *gbm = nullptr;
    int32_t *thigh = nullptr;
    TmpGuard tg(ctx);
    const int nsm = ctx->num_sms;
    bool tc_ran = false;
    HubArgs H;
    const size_t smem = hub_layout(G.n, nhubs, nwide, max_degree, &H);
    if ((int64_t)H.split < G.n) {
        if ((st = tg.alloc(&gbm, (size_t)nsm * H.nwords * 4))) return st;
        PGD_CUDA(ctx, cudaMemsetAsync(gbm, 0, (size_t)nsm * H.nwords * 4, s));
    }
    PGD_CUDA(ctx, cudaEventRecord(ctx->ev0, s));
    // triangle counts of every edge first: k_hub and k_light read t(x, q) of
    // other edges.  A sampled order still needs t of all edges: the same
    // grouped pass runs over a plan of every edge (positions = edge ids).
    if (sampled) {
        int32_t *iota = nullptr;
        if ((st = tg.alloc(&iota, (size_t)G.m * sizeof(int32_t)))) return st;
        PGD_LAUNCH(ctx, k_iota, grid_for(G.m), kThreads, 0, iota, G.m);
        DevGraph GA = G;
        GA.order = iota;
        GA.npos = G.m;
        GA.micro = nullptr;
        Plan PA;
        if ((st = build_plan(ctx, GA, tg, &PA))) return st;
        PGD_CUDA(ctx, cudaEventRecord(ctx->evt0, s));
        if ((st = triangle_pass(ctx, GA, slot, PA, H, gbm))) return st;
        PGD_CUDA(ctx, cudaEventRecord(ctx->evt1, s));
    }
    Plan P;
    uint64_t *keys = nullptr, *keys2 = nullptr;
    int32_t *vals = nullptr;
    if ((st = build_plan(ctx, G, tg, &P, &keys, &vals, &keys2))) return st;
    int32_t *posv = P.posv;
    const unsigned long long nh = P.nh, nd = P.nd;
    const int64_t nlight = P.nlight, nitems = P.nitems;
    int64_t *items = P.items;
    int2 *hrec = P.hrec;
    unsigned long long *ctr = ctx->d_ctr;
    if (!sampled) {
        PGD_CUDA(ctx, cudaEventRecord(ctx->evt0, s));
        if ((st = triangle_pass(ctx, G, slot, P, H, gbm))) return st;
        PGD_CUDA(ctx, cudaEventRecord(ctx->evt1, s));
    }
    if (nitems > 0) {
        if (!H.smem_hist) {
            if ((st = tg.alloc(&ghist, (size_t)nsm * H.hstride * 4))) return st;
        }
        if ((st = tg.alloc(&thigh, (size_t)nsm * kHubWarps * kTHigh * sizeof(int32_t)))) return st;
        if (G.n > kRankBits) {
            // per-warp window bitmaps over ranks [kRankBits, min(n, kTWin)), zero at the start
            const int64_t lim = std::min<int64_t>(G.n, kTWin);
            H.twin_words = (int32_t)((lim - kRankBits + 31) / 32);
            const size_t bytes = (size_t)nsm * kHubWarps * H.twin_words * sizeof(uint32_t);
            if ((st = tg.alloc(&H.twin, bytes))) return st;
            PGD_CUDA(ctx, cudaMemsetAsync(H.twin, 0, bytes, s));
        }
        PGD_CUDA(ctx, cudaFuncSetAttribute(k_hub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        H.G = G;
        H.hpos = posv;
        H.hrec = hrec;
        H.items = items;
        H.nitems = nitems;
        H.ghist = ghist;
        H.gbitmap = gbm;
        H.next = ctr + 1;
        H.thigh = thigh;
        PGD_CUDA(ctx, cudaEventRecord(ctx->evh0, s));
        PGD_LAUNCH(ctx, k_hub, nsm, kHubWarps * 32, smem, H);
        PGD_CUDA(ctx, cudaEventRecord(ctx->evh1, s));
    }
    if (nd > 0 && dense) {
        // dense edges grouped by q, so that k_dense serves several per row pass
        // (edges of graphs with a CN matrix first, counted in ctr[7])
        const int qb = bits_for(G.n), ebd = bits_for(G.npos);
        PGD_LAUNCH(ctx, k_dense_keys, grid_for(nd), kThreads, 0, G, posv + nh, (int64_t)nd,
                   dense->cn ? dense->cbase : nullptr, keys, vals, ctr + 7, qb, ebd);
        size_t tbd = 0;
        void *tmpd = nullptr;
        cub::DeviceRadixSort::SortPairs(nullptr, tbd, keys, keys2, vals, posv + nh, (int64_t)nd, 0, 1 + qb + ebd, s);
        if ((st = pgd_tmp_alloc(ctx, &tmpd, tbd))) return st;
        cub::DeviceRadixSort::SortPairs(tmpd, tbd, keys, keys2, vals, posv + nh, (int64_t)nd, 0, 1 + qb + ebd, s);
        pgd_tmp_free(ctx, tmpd);
        int64_t ncn = 0;
        if (dense->cn) {
            unsigned long long h = 0;
            PGD_CUDA(ctx, cudaMemcpyAsync(&h, ctr + 7, sizeof(h), cudaMemcpyDeviceToHost, s));
            PGD_CUDA(ctx, cudaStreamSynchronize(s));
            ncn = (int64_t)h;
        }
        TcOut tc;
        if (ncn > 0 && ctx->tc_min_deg > 0) {
            if ((st = dense_tc(ctx, G, tg, dense, posv + nh, keys2, ncn, ebd, &tc))) return st;
            tc_ran = true;
        }
        if (ncn > 0 && (!tc.k4 || tc.nrest > 0)) {
            DenseCnArgs C;
            C.G = G;
            C.bits = dense->bits;
            C.wbase = dense->wbase;
            C.vbase = dense->vbase;
            C.cn = dense->cn;
            C.cbase = dense->cbase;
            // with the tensor-core path, only the positions outside its runs
            C.dpos = tc.k4 ? tc.rest : posv + nh;
            C.k4pre = nullptr;
            C.ndense = tc.k4 ? tc.nrest : ncn;
            C.next = ctr + 6;
            PGD_LAUNCH(ctx, k_dense_cn, nsm * 8, 256, 0, C);
        }
        if (ncn > 0) {
            if (tc.k4) {
                DenseCloseArgs Z;
                Z.G = G;
                Z.bits = dense->bits;
                Z.wbase = dense->wbase;
                Z.vbase = dense->vbase;
                Z.cn = dense->cn;
                Z.cbase = dense->cbase;
                Z.dpos = posv + nh;
                Z.runs = tc.runs;
                Z.nruns = tc.nruns;
                Z.k4 = tc.k4;
                Z.eslot = tc.eslot;
                Z.next = ctr + 11;
                PGD_LAUNCH(ctx, k_dense_close, nsm * 8, 256, 0, Z);
            }
        }
        if ((int64_t)nd > ncn) {
            DenseArgs D;
            D.G = G;
            D.bits = dense->bits;
            D.wbase = dense->wbase;
            D.vbase = dense->vbase;
            D.dpos = posv + nh + ncn;
            D.ndense = (int64_t)nd - ncn;
            D.next = ctr + 4;
            PGD_LAUNCH(ctx, k_dense, nsm * 8, 256, 0, D);
        }
    }
    if (nlight > 0) {
        LightArgs L;
        L.G = G;
        L.lpos = posv + nh + nd;
        L.nlight = nlight;
        L.next = ctr + 2;
        PGD_LAUNCH(ctx, k_light, nsm * 8, kLightWarps * 32, 0, L);
    }
    PGD_CUDA(ctx, cudaEventRecord(ctx->ev1, s));
    PGD_CUDA(ctx, cudaGetLastError());
    PGD_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    PGD_CUDA(ctx, cudaEventElapsedTime(&ms->total, ctx->ev0, ctx->ev1));
    PGD_CUDA(ctx, cudaEventElapsedTime(&ms->tri, ctx->evt0, ctx->evt1));
    if (nitems > 0) PGD_CUDA(ctx, cudaEventElapsedTime(&ms->hub, ctx->evh0, ctx->evh1));
    if (tc_ran) {
        unsigned long long failed = 0;
        PGD_CUDA(ctx, cudaMemcpy(&failed, ctr + 10, sizeof(failed), cudaMemcpyDeviceToHost));
        if (failed) return pgd_fail(ctx, PGD_ETIMEOUT, "a tensor-core wait in k_dense_tc or k_dense_gram ran out");
    }
    return PGD_OK;
}

pgd_status pgd_dev_decompose(pgd_graph *g, bool micro, pgd_counts *out) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    if (micro && !g->micro) {
        if ((st = pgd_graph_alloc(g, (void **)&g->micro, (g->m + 1) * PGD_NMICRO * sizeof(uint64_t)))) return st;
    }
    if ((!g->has_aux || g->aux_cache_hub != ctx->cache_hub) && (st = build_aux(g))) return st;
    PGD_CUDA(ctx, cudaMemsetAsync(ctx->d_sums, 0, PGD_NSUMS * sizeof(unsigned long long), s));
    StageMs ms;
    if ((st = run_decompose(ctx, dev_view(g, micro), (int4 *)g->slot, g->nhubs, g->nhubs_wide, g->max_degree, &ms))) return st;
    unsigned long long h[PGD_NSUMS];
    PGD_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_sums, sizeof(h), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    for (int i = 0; i < PGD_NSUMS; i++) out->sums[i] = h[i];
    out->n = g->n;
    out->m = g->m;
    out->kernel_ms = ms.total;
    out->hub_ms = ms.hub;
    out->tri_ms = ms.tri;
    pgd_close_counts(out->sums, g->n, g->m, out->totals);
    g->has_micro = micro;
    return PGD_OK;
}

// ---------------------------------------------------------------------------
// Batched decomposition: the graphs become one disjoint union on the device
// (vertex, slot and edge ids offset per graph), decomposed by the same
// persistent kernels; t, k4 and c4 never cross graphs, the closed forms use
// each edge's own graph's n and m, and the sums are kept per graph.

struct BatchDesc {
    const int64_t *off;
    const int32_t *adj;
    const int32_t *deg;
    const int32_t *ev;
    const int32_t *eu;
    const int32_t *order;
    int64_t n, m, vbase, ebase, sbase;   // vertex, edge and slot offsets in the union
};

__global__ void k_union_vertices(const BatchDesc *D, const int64_t *vbase, int k, int64_t N, int64_t *off,
                                 int32_t *deg, int32_t *vgraph) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < N; x += (int64_t)gridDim.x * blockDim.x) {
        const int g = batch_find(vbase, k, x);
        const int64_t v = x - D[g].vbase;
        off[x] = D[g].sbase + D[g].off[v];
        deg[x] = D[g].deg[v];
        vgraph[x] = g;
    }
}

__global__ void k_union_slots(const BatchDesc *D, const int64_t *sbase, int k, int64_t S, int32_t *adj) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < S; j += (int64_t)gridDim.x * blockDim.x) {
        const int g = batch_find(sbase, k, j);
        adj[j] = (int32_t)(D[g].adj[j - D[g].sbase] + D[g].vbase);
    }
}

__global__ void k_union_edges(const BatchDesc *D, const int64_t *ebase, int k, int64_t M, int32_t *ev, int32_t *eu,
                              int32_t *order, int32_t *egraph) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M; e += (int64_t)gridDim.x * blockDim.x) {
        const int g = batch_find(ebase, k, e);
        const int64_t l = e - D[g].ebase;
        ev[e] = (int32_t)(D[g].ev[l] + D[g].vbase);
        eu[e] = (int32_t)(D[g].eu[l] + D[g].vbase);
        order[e] = (int32_t)(D[g].order[l] + D[g].ebase);
        egraph[e] = g;
    }
}

// Graphs of a batch that also get a common-neighbour matrix (k_dense_cn):
// graphs on the row-bitset path whose average degree is at least n/16
// (32·m >= n²), as long as the matrices stay within kCnMaxEntries.  Fills
// cbase (first entry per graph, -1 for none) and ctile (first 32-row tile
// per graph; k + 1 entries) and returns the number of 16-bit entries.
constexpr int64_t kCnMaxEntries = 4ll << 30;   // 8 GiB

static int64_t plan_common(int k, const std::vector<long long> &gnm, const std::vector<uint8_t> &gdense,
                           std::vector<int64_t> &cbase, std::vector<int64_t> &ctile) {
    cbase.assign((size_t)k, -1);
    ctile.assign((size_t)k + 1, 0);
    int64_t entries = 0, tiles = 0;
    for (int g = 0; g < k; g++) {
        ctile[(size_t)g] = tiles;
        const int64_t n = gnm[(size_t)2 * g], m = gnm[(size_t)2 * g + 1];
        if (!gdense[(size_t)g] || 32 * m < n * n) continue;
        const int64_t e = n * (((n + 63) / 64) * 64);   // a multiple of 64: every matrix is 128-byte aligned
        if (entries + e > kCnMaxEntries) continue;
        cbase[(size_t)g] = entries;
        entries += e;
        tiles += (n + kCnRows - 1) / kCnRows;
    }
    ctile[(size_t)k] = tiles;
    return entries;
}

pgd_status pgd_dev_decompose_batch(pgd_ctx *ctx, pgd_graph *const *graphs, int k, bool micro, pgd_counts *out) {
    cudaStream_t s = ctx->stream;
    pgd_status st;
    std::vector<BatchDesc> desc((size_t)k);
    std::vector<int64_t> bases((size_t)3 * k + 3, 0);
    std::vector<long long> gnm((size_t)2 * k);
    int64_t N = 0, M = 0, S = 0;
    int32_t max_degree = 0;
    for (int i = 0; i < k; i++)
        if (graphs[i]->norder != graphs[i]->m)
            return pgd_fail(ctx, PGD_EINVAL, "a graph of the batch has a sampled edge order (decompose it alone)");
    for (int i = 0; i < k; i++) {
        pgd_graph *g = graphs[i];
        if (micro && !g->micro) {
            if ((st = pgd_graph_alloc(g, (void **)&g->micro, (g->m + 1) * PGD_NMICRO * sizeof(uint64_t)))) return st;
        }
        BatchDesc &d = desc[(size_t)i];
        d.off = g->off;
        d.adj = g->adj;
        d.deg = g->deg;
        d.ev = g->ev;
        d.eu = g->eu;
        d.order = g->order;
        d.n = g->n;
        d.m = g->m;
        d.vbase = N;
        d.ebase = M;
        d.sbase = S;
        bases[(size_t)i] = N;
        bases[(size_t)k + 1 + i] = M;
        bases[(size_t)2 * k + 2 + i] = S;
        gnm[(size_t)2 * i] = g->n;
        gnm[(size_t)2 * i + 1] = g->m;
        max_degree = std::max(max_degree, g->max_degree);
        N += g->n;
        M += g->m;
        S += 2 * g->m;
    }
    if (N > 0x7ffffffe || S > 0x7fffffff)
        return pgd_fail(ctx, PGD_EINVAL, "batch too large for 32-bit vertex and slot ids");
    // the union, as a transient graph of this context
    pgd_graph U;
    U.ctx = ctx;
    U.n = N;
    U.m = M;
    U.norder = M;
    U.max_degree = max_degree;
    BatchDesc *d_desc = nullptr;
    int64_t *d_bases = nullptr;
    long long *d_gnm = nullptr;
    int32_t *egraph = nullptr, *vgraph = nullptr;
    unsigned long long *gsums = nullptr, *bits = nullptr;
    uint64_t *umicro = nullptr;
    uint8_t *d_gdense = nullptr;
    int64_t *d_wbase = nullptr, *d_cbase = nullptr, *d_ctile = nullptr;
    uint16_t *cn = nullptr;
    // graphs of at most dense_max vertices use the row-bitset kernel
    std::vector<uint8_t> gdense((size_t)k, 0);
    std::vector<int64_t> wbase((size_t)k, 0);
    int64_t words = 0;
    int ndense_graphs = 0;
    for (int i = 0; i < k; i++) {
        const int64_t n = graphs[i]->n;
        if (n > 0 && n <= ctx->dense_max && graphs[i]->m > 0) {
            gdense[(size_t)i] = 1;
            wbase[(size_t)i] = words;
            words += n * ((n + 63) / 64);
            ndense_graphs++;
        }
    }
    std::vector<int64_t> cbase, ctile;
    const int64_t cn_entries = plan_common(k, gnm, gdense, cbase, ctile);
    auto cleanup = [&]() {
        pgd_tmp_free(ctx, cn);
        pgd_tmp_free(ctx, d_cbase);
        pgd_tmp_free(ctx, d_ctile);
        pgd_tmp_free(ctx, vgraph);
        pgd_tmp_free(ctx, bits);
        pgd_tmp_free(ctx, d_gdense);
        pgd_tmp_free(ctx, d_wbase);
        pgd_tmp_free(ctx, d_desc);
        pgd_tmp_free(ctx, d_bases);
        pgd_tmp_free(ctx, d_gnm);
        pgd_tmp_free(ctx, egraph);
        pgd_tmp_free(ctx, gsums);
        pgd_tmp_free(ctx, umicro);
        pgd_graph_free(&U, U.off, (N + 1) * sizeof(int64_t));
        pgd_graph_free(&U, U.adj, (S + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.deg, (N + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.ev, (M + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.eu, (M + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.order, (M + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.offp, (N + 1) * sizeof(int64_t));
        pgd_graph_free(&U, U.adjp, (M + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.hubid, (N + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.vrank, (N + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.adjp_rank, (M + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.slot, (S + 1) * sizeof(int4));
        pgd_graph_free(&U, U.offh, (N + 1) * sizeof(int64_t));
        pgd_graph_free(&U, U.adjh, (U.nadjh + 1) * sizeof(int32_t));
        pgd_graph_free(&U, U.toprows, (U.top_words + 1) * sizeof(uint32_t));
        pgd_graph_free(&U, U.vrec, (N + 1) * 32);
        pgd_graph_free(&U, U.adj_rank, (S + 1) * sizeof(int32_t));
    };
#define BATCH_TRY(expr)                      \
    do {                                     \
        if ((st = (expr)) != PGD_OK) {       \
            cleanup();                       \
            return st;                       \
        }                                    \
    } while (0)
    BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&d_desc, (size_t)k * sizeof(BatchDesc)));
    BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&d_bases, bases.size() * sizeof(int64_t)));
    BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&d_gnm, gnm.size() * sizeof(long long)));
    BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&egraph, (M + 1) * sizeof(int32_t)));
    BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&vgraph, (N + 1) * sizeof(int32_t)));
    BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&d_gdense, (size_t)k));
    BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&d_wbase, (size_t)k * sizeof(int64_t)));
    if (words > 0) BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&bits, (size_t)words * sizeof(unsigned long long)));
    if (cn_entries > 0) {
        BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&cn, (size_t)cn_entries * sizeof(uint16_t)));
        BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&d_cbase, (size_t)k * sizeof(int64_t)));
        BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&d_ctile, ((size_t)k + 1) * sizeof(int64_t)));
    }
    BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&gsums, (size_t)k * PGD_NSUMS * sizeof(unsigned long long)));
    if (micro) BATCH_TRY(pgd_tmp_alloc(ctx, (void **)&umicro, (M + 1) * PGD_NMICRO * sizeof(uint64_t)));
    BATCH_TRY(pgd_graph_alloc(&U, (void **)&U.off, (N + 1) * sizeof(int64_t)));
    BATCH_TRY(pgd_graph_alloc(&U, (void **)&U.adj, (S + 1) * sizeof(int32_t)));
    BATCH_TRY(pgd_graph_alloc(&U, (void **)&U.deg, (N + 1) * sizeof(int32_t)));
    BATCH_TRY(pgd_graph_alloc(&U, (void **)&U.ev, (M + 1) * sizeof(int32_t)));
    BATCH_TRY(pgd_graph_alloc(&U, (void **)&U.eu, (M + 1) * sizeof(int32_t)));
    BATCH_TRY(pgd_graph_alloc(&U, (void **)&U.order, (M + 1) * sizeof(int32_t)));
    if (cudaMemcpyAsync(d_desc, desc.data(), (size_t)k * sizeof(BatchDesc), cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(d_bases, bases.data(), bases.size() * sizeof(int64_t), cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(d_gnm, gnm.data(), gnm.size() * sizeof(long long), cudaMemcpyHostToDevice, s) ||
        cudaMemsetAsync(gsums, 0, (size_t)k * PGD_NSUMS * sizeof(unsigned long long), s) ||
        cudaMemcpyAsync(d_gdense, gdense.data(), (size_t)k, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(d_wbase, wbase.data(), (size_t)k * sizeof(int64_t), cudaMemcpyHostToDevice, s) ||
        (words > 0 && cudaMemsetAsync(bits, 0, (size_t)words * sizeof(unsigned long long), s)) ||
        (cn_entries > 0 &&
         (cudaMemcpyAsync(d_cbase, cbase.data(), (size_t)k * sizeof(int64_t), cudaMemcpyHostToDevice, s) ||
          cudaMemcpyAsync(d_ctile, ctile.data(), ((size_t)k + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s)))) {
        cleanup();
        return pgd_fail(ctx, PGD_ECUDA, "batch set-up copy failed");
    }
    PGD_LAUNCH(ctx, k_union_vertices, grid_for(N), kThreads, 0, d_desc, d_bases, k, N, U.off, U.deg, vgraph);
    PGD_CUDA(ctx, cudaMemcpyAsync(U.off + N, &S, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    PGD_LAUNCH(ctx, k_union_slots, grid_for(S), kThreads, 0, d_desc, d_bases + 2 * k + 2, k, S, U.adj);
    PGD_LAUNCH(ctx, k_union_edges, grid_for(M), kThreads, 0, d_desc, d_bases + k + 1, k, M, U.ev, U.eu, U.order,
               egraph);
    BATCH_TRY(build_aux(&U));
    if (words > 0)
        PGD_LAUNCH(ctx, k_dense_bits, grid_for(32 * N), kThreads, 0, U.off, U.adj, vgraph, d_gdense, d_wbase, d_bases,
                   d_gnm, N, bits);
    if (cn_entries > 0)
        PGD_LAUNCH(ctx, k_dense_common, (int)std::min<int64_t>(ctile[(size_t)k], (int64_t)ctx->num_sms * 8), 256, 0,
                   (const uint64_t *)bits, d_wbase, d_gnm, d_cbase, d_ctile, k, ctile[(size_t)k], cn);
    DevGraph G = dev_view(&U, micro);
    G.micro = micro ? umicro : nullptr;
    G.sums = gsums;
    G.egraph = egraph;
    G.gnm = d_gnm;
    G.gdense = ndense_graphs ? d_gdense : nullptr;
    DenseView dv{(const uint64_t *)bits, d_wbase, d_bases, cn, d_cbase, k};
    StageMs ms;
    BATCH_TRY(run_decompose(ctx, G, (int4 *)U.slot, U.nhubs, U.nhubs_wide, U.max_degree, &ms, ndense_graphs ? &dv : nullptr));
    std::vector<unsigned long long> h((size_t)k * PGD_NSUMS);
    if (cudaMemcpyAsync(h.data(), gsums, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s)) {
        cleanup();
        return pgd_fail(ctx, PGD_ECUDA, "batch result copy failed");
    }
    for (int i = 0; micro && i < k; i++) {
        pgd_graph *g = graphs[i];
        if (g->m && cudaMemcpyAsync(g->micro, umicro + desc[(size_t)i].ebase * PGD_NMICRO,
                                    g->m * PGD_NMICRO * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s)) {
            cleanup();
            return pgd_fail(ctx, PGD_ECUDA, "batch micro copy failed");
        }
    }
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    for (int i = 0; i < k; i++) {
        pgd_counts &o = out[i];
        memset(&o, 0, sizeof(o));
        for (int j = 0; j < PGD_NSUMS; j++) o.sums[j] = h[(size_t)i * PGD_NSUMS + j];
        o.n = gnm[(size_t)2 * i];
        o.m = gnm[(size_t)2 * i + 1];
        o.kernel_ms = ms.total;
        o.hub_ms = ms.hub;
        o.tri_ms = ms.tri;
        pgd_close_counts(o.sums, o.n, o.m, o.totals);
        graphs[i]->has_micro = micro;
    }
    cleanup();
#undef BATCH_TRY
    return PGD_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free decomposition (no counterpart in the reference).
//
// Some callers cannot allocate device memory at the moment they need counts:
// code inside a framework that hands out a fixed workspace and forbids
// allocation (inference plugins, custom ops), and latency-critical loops
// where cudaMalloc/cudaFree would synchronise the device.  For them
// pgd_decompose_csr_noalloc runs the same kernels on a caller's device CSR
// with every intermediate carved out of one file-scope device array of
// kNoAllocScratchBytes, and it never calls cudaMalloc, cudaFree or an
// allocating library routine.
//
// The array is a __device__ object: every GPU that loads this library holds
// kNoAllocScratchBytes for it until the process exits.  All calls share it,
// and each call clears what must start at zero; calls that overlap on the
// GPU (two streams, two threads) race on it and must be serialised by the
// caller.  Host code must not use the array's name as an address: its
// device address is looked up with cudaGetSymbolAddress once per device, by
// the first call on that device.

namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_addr[kNoAllocMaxDevices] = {};

// Offsets must start at 0, end at nnz and never decrease; checked before
// anything indexes the adjacency through them.
__global__ void k_na_offsets(const int64_t *off, int64_t n, int64_t nnz, unsigned long long *bad) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = off[v], b = off[v + 1];
        bool ok = a <= b && a >= 0 && b <= nnz;
        if (v == 0) ok = ok && a == 0;
        if (v == n - 1) ok = ok && b == nnz;
        if (!ok) atomicAdd(bad, 1ull);
    }
}

// Rows must be sorted, in range, free of self loops, and symmetric.
__global__ void k_na_check(const int64_t *off, const int32_t *adj, const int32_t *row, int64_t n, int64_t nnz,
                           unsigned long long *bad) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = row[j], c = adj[j];
        bool ok = c >= 0 && c < n && c != r && (j == off[r] || adj[j - 1] < c);
        if (ok) ok = pgd_contains(adj + off[c], (int)(off[c + 1] - off[c]), r);
        if (!ok) atomicAdd(bad, 1ull);
    }
}

__global__ void k_na_degrees(const int64_t *off, int64_t n, int32_t *deg) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        deg[v] = (int32_t)(off[v + 1] - off[v]);
}

__global__ void k_na_edge_flags(const int32_t *row, const int32_t *adj, int64_t nnz, uint32_t *flag) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        flag[j] = row[j] < adj[j] ? 1u : 0u;
}

__global__ void k_na_edges(const int32_t *row, const int32_t *adj, const uint32_t *flag, const uint32_t *pos,
                           int64_t nnz, int32_t *ev, int32_t *eu, int32_t *order) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[j]) continue;
        const uint32_t id = pos[j];
        ev[id] = row[j];
        eu[id] = adj[j];
        order[id] = (int32_t)id;
    }
}

// Bump allocator over the scratch array (host-side bookkeeping only).
struct Carve {
    unsigned char *base;
    size_t used = 0, limit;
    bool ok = true;
    template <typename T>
    T *take(size_t count) {
        size_t bytes = ((count * sizeof(T)) + 255) & ~(size_t)255;
        if (used + bytes > limit) { ok = false; return nullptr; }
        T *p = (T *)(base + used);
        used += bytes;
        return p;
    }
};

// Restores the calling thread's current device on every return path.
struct DeviceRestore {
    int prev = -1;
    DeviceRestore() {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            prev = -1;
            cudaGetLastError();
        }
    }
    ~DeviceRestore() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

void na_msg(char *err, size_t errlen, const std::string &m) {
    if (err && errlen) {
        size_t k = std::min(errlen - 1, m.size());
        memcpy(err, m.data(), k);
        err[k] = 0;
    }
}

}  // namespace

#define NA_CUDA(call)                                                                         \
    do {                                                                                      \
        cudaError_t e__ = (call);                                                             \
        if (e__ != cudaSuccess) {                                                             \
            na_msg(err, errlen, std::string("CUDA error ") + cudaGetErrorString(e__) + " in " #call); \
            return e__ == cudaErrorMemoryAllocation ? PGD_ENOMEM : PGD_ECUDA;                  \
        }                                                                                     \
    } while (0)

extern "C" uint64_t pgd_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

extern "C" pgd_status pgd_decompose_csr_noalloc(const int64_t *d_off, const int32_t *d_adj, int64_t n, int64_t nnz,
                                                int device, void *stream_, pgd_counts *out, char *err,
                                                size_t errlen) {
    if (!d_off || (nnz > 0 && !d_adj) || n < 0 || nnz < 0 || (nnz & 1) || !out) {
        na_msg(err, errlen, "bad arguments (device CSR pointers, n >= 0, even nnz, out)");
        return PGD_EINVAL;
    }
    if (device < 0 || device >= kNoAllocMaxDevices || n > 0x7ffffffe || nnz > 0x7fffffff) {
        na_msg(err, errlen, "device ordinal or graph size out of range");
        return PGD_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream_;
    DeviceRestore restore_device;
    NA_CUDA(cudaSetDevice(device));
    unsigned char *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[device]) {
            void *ptr = nullptr;
            NA_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
            g_noalloc_addr[device] = (unsigned char *)ptr;
        }
        base = g_noalloc_addr[device];
    }
    int nsm = 0;
    NA_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    const int64_t m = nnz / 2;
    const int64_t nwords = (n + 31) / 32;
    const int64_t hub_bound = std::max<int64_t>(1, std::min<int64_t>(n, nnz / kCacheHub + 1));

    // CUB temporary storage sizes (queries only)
    size_t tb_scan = 0, tb_sort = 0, tb_pairs = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb_scan, (uint32_t *)nullptr, (uint32_t *)nullptr, std::max(nnz, n) + 1, s);
    cub::DeviceRadixSort::SortKeys(nullptr, tb_sort, (uint64_t *)nullptr, (uint64_t *)nullptr,
                                   std::max<int64_t>(std::max(m, n), 1), 0, 64, s);
    cub::DeviceRadixSort::SortPairs(nullptr, tb_pairs, (uint64_t *)nullptr, (uint64_t *)nullptr, (int32_t *)nullptr,
                                    (int32_t *)nullptr, std::max<int64_t>(m, 1), 0, 64, s);
    tb_sort = std::max(tb_sort, tb_pairs);

    // carve every buffer up front, with upper bounds, so an oversized graph
    // is refused before anything runs
    Carve C{base, 0, kNoAllocScratchBytes};
    unsigned long long *sums = C.take<unsigned long long>(PGD_NSUMS + 1);
    unsigned long long *ctr = C.take<unsigned long long>(8);
    int32_t *deg = C.take<int32_t>(n + 1);
    int32_t *row = C.take<int32_t>(nnz + 1);
    uint32_t *flag = C.take<uint32_t>(std::max(nnz, n) + 2);
    uint32_t *pos = C.take<uint32_t>(std::max(nnz, n) + 2);
    int32_t *ev = C.take<int32_t>(m + 1);
    int32_t *eu = C.take<int32_t>(m + 1);
    int32_t *order = C.take<int32_t>(m + 1);
    int64_t *offp = C.take<int64_t>(n + 1);
    int32_t *adjp = C.take<int32_t>(m + 1);
    int32_t *hubid = C.take<int32_t>(n + 1);
    int32_t *vrank = C.take<int32_t>(n + 1);
    int32_t *adjp_rank = C.take<int32_t>(m + 1);
    uint64_t *rk = C.take<uint64_t>(n + 1);
    uint64_t *rk2 = C.take<uint64_t>(n + 1);
    int4 *slot = C.take<int4>(nnz + 1);
    uint64_t *keys = C.take<uint64_t>(m + 1);
    uint64_t *keys2 = C.take<uint64_t>(m + 1);
    int32_t *posv = C.take<int32_t>(m + 1);
    int32_t *vals = C.take<int32_t>(m + 1);
    uint32_t *iflag = C.take<uint32_t>(m + 2);
    uint32_t *ipos = C.take<uint32_t>(m + 2);
    int64_t *items = C.take<int64_t>(m + 2);
    int2 *hrec = C.take<int2>(m + 1);
    int64_t *offh = C.take<int64_t>(n + 1);
    int4 *vrec = C.take<int4>(2 * (n + 1));
    int32_t *adjh = C.take<int32_t>(nnz + 1);
    // k_hub's layout depends on the hub count, known only later: carve for
    // the largest possible count (the maximum degree is not known here
    // either: 32-bit counters)
    HubArgs H;
    hub_layout(n, (int32_t)hub_bound, (int32_t)hub_bound, 1 << 30, &H);
    // fewer hubs never need more global memory: a histogram that fits in
    // shared memory for hub_bound hubs fits for fewer, and the bitmap's
    // shared part only grows
    uint32_t *ghist = H.smem_hist ? nullptr : C.take<uint32_t>((size_t)nsm * H.hstride);
    uint32_t *gbm = (int64_t)H.split >= n ? nullptr : C.take<uint32_t>((size_t)nsm * nwords);
    int32_t *adj_rank = C.take<int32_t>(nnz + 1);
    void *tmp = C.take<unsigned char>(std::max(tb_scan, tb_sort) + 16);
    if (!C.ok) {
        na_msg(err, errlen, "graph too large for the allocation-free path: needs more than the " +
                                std::to_string(kNoAllocScratchBytes >> 20) + " MiB scratch array (n=" +
                                std::to_string(n) + ", nnz=" + std::to_string(nnz) + ")");
        return PGD_ENOMEM;
    }
    size_t tb = std::max(tb_scan, tb_sort) + 16;

    NA_CUDA(cudaMemsetAsync(sums, 0, (PGD_NSUMS + 1) * sizeof(unsigned long long), s));
    NA_CUDA(cudaMemsetAsync(ctr, 0, 8 * sizeof(unsigned long long), s));
    memset(out, 0, sizeof(*out));
    out->n = n;
    out->m = m;
    if (m == 0) {
        pgd_close_counts(out->sums, n, m, out->totals);
        return PGD_OK;
    }
    // validate the offsets, then the rows, then derive the per-graph structures
    unsigned long long bad = 0;
    k_na_offsets<<<grid_for(n), kThreads, 0, s>>>(d_off, n, nnz, ctr + 4);
    NA_CUDA(cudaMemcpyAsync(&bad, ctr + 4, sizeof(bad), cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    if (bad) {
        na_msg(err, errlen, "device CSR rejected: offsets must start at 0, end at nnz and never decrease");
        return PGD_EINVAL;
    }
    k_rows<<<grid_for(nnz), kThreads, 0, s>>>(d_off, n, nnz, row);
    k_na_check<<<grid_for(nnz), kThreads, 0, s>>>(d_off, d_adj, row, n, nnz, ctr + 3);
    k_na_degrees<<<grid_for(n), kThreads, 0, s>>>(d_off, n, deg);
    NA_CUDA(cudaMemcpyAsync(&bad, ctr + 3, sizeof(bad), cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    if (bad) {
        na_msg(err, errlen, "device CSR rejected: rows must be sorted, symmetric, in range and free of self loops");
        return PGD_EINVAL;
    }
    k_na_edge_flags<<<grid_for(nnz), kThreads, 0, s>>>(row, d_adj, nnz, flag);
    NA_CUDA(cudaMemsetAsync(flag + nnz, 0, sizeof(uint32_t), s));
    NA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, nnz + 1, s));
    k_na_edges<<<grid_for(nnz), kThreads, 0, s>>>(row, d_adj, flag, pos, nnz, ev, eu, order);
    k_oriented_flags<<<grid_for(nnz), kThreads, 0, s>>>(row, d_adj, deg, nnz, flag);
    NA_CUDA(cudaMemsetAsync(flag + nnz, 0, sizeof(uint32_t), s));
    NA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, nnz + 1, s));
    k_oriented_fill<<<grid_for(std::max(nnz, n + 1)), kThreads, 0, s>>>(d_off, d_adj, flag, pos, n, nnz, offp, adjp);
    k_hub_flags<<<grid_for(n), kThreads, 0, s>>>(deg, n, kCacheHub, flag);
    NA_CUDA(cudaMemsetAsync(flag + n, 0, sizeof(uint32_t), s));
    NA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, n + 1, s));
    k_hub_ids<<<grid_for(n), kThreads, 0, s>>>(flag, pos, n, hubid);
    uint32_t nhubs = 0;
    NA_CUDA(cudaMemcpyAsync(&nhubs, pos + n, sizeof(nhubs), cudaMemcpyDeviceToHost, s));
    k_hubnb_flags<<<grid_for(nnz), kThreads, 0, s>>>(d_adj, hubid, nnz, flag);
    NA_CUDA(cudaMemsetAsync(flag + nnz, 0, sizeof(uint32_t), s));
    NA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, nnz + 1, s));
    k_hubnb_fill<<<grid_for(std::max(nnz, n + 1)), kThreads, 0, s>>>(d_off, d_adj, hubid, flag, pos, n, nnz, offh,
                                                                      adjh);
    k_rank_keys<<<grid_for(n), kThreads, 0, s>>>(deg, n, rk);
    NA_CUDA(cub::DeviceRadixSort::SortKeys(tmp, tb, rk, rk2, n, 0, 64, s));
    k_rank_scatter<<<grid_for(n), kThreads, 0, s>>>(rk2, n, vrank);
    k_gather_rank<<<grid_for(m), kThreads, 0, s>>>(adjp, vrank, m, adjp_rank);
    k_gather_rank<<<grid_for(nnz), kThreads, 0, s>>>(d_adj, vrank, nnz, adj_rank);
    k_vrec<<<grid_for(n), kThreads, 0, s>>>(d_off, offp, deg, vrank, hubid, n, vrec);
    k_slot_fill<<<grid_for(nnz), kThreads, 0, s>>>(d_adj, vrank, hubid, offp, nnz, 0, slot);

    DevGraph G;
    G.off = d_off;
    G.adj = d_adj;
    G.deg = deg;
    G.offp = offp;
    G.adjp = adjp;
    G.hubid = hubid;
    G.slot = slot;
    G.ev = ev;
    G.eu = eu;
    G.order = order;
    G.n = n;
    G.m = m;
    G.npos = m;
    G.micro = nullptr;
    G.sums = sums;
    G.egraph = nullptr;
    G.gnm = nullptr;
    G.gdense = nullptr;
    G.vrank = vrank;
    G.adjp_rank = adjp_rank;
    G.adj_rank = adj_rank;
    G.offh = offh;
    G.adjh = adjh;
    G.toprows = nullptr;   // no rank-bitmap rows here: k4 always scans N+(x)
    G.vrec = vrec;
    G.top_r = 0;
    G.anchor_hub = kAnchorHub;
    k_tslot<<<grid_for(32 * m), kThreads, 0, s>>>(G, slot, nullptr, 0);
    k_plan_keys<<<grid_for(m), kThreads, 0, s>>>(G, keys, vals, ctr, 32);
    NA_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, posv, m, 0, 64, s));
    unsigned long long nh = 0;
    NA_CUDA(cudaMemcpyAsync(&nh, ctr, sizeof(nh), cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    int64_t nitems = 0;
    if (nh > 0) {
        k_item_flags<<<grid_for(nh), kThreads, 0, s>>>(keys2, (int64_t)nh, iflag, 32);
        NA_CUDA(cudaMemsetAsync(iflag + nh, 0, sizeof(uint32_t), s));
        NA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, iflag, ipos, (int64_t)nh + 1, s));
        uint32_t ni = 0;
        NA_CUDA(cudaMemcpyAsync(&ni, ipos + nh, sizeof(ni), cudaMemcpyDeviceToHost, s));
        NA_CUDA(cudaStreamSynchronize(s));
        nitems = ni;
        k_item_fill<<<grid_for(nh), kThreads, 0, s>>>(iflag, ipos, (int64_t)nh, items);
        k_hub_recs<<<grid_for(nh), kThreads, 0, s>>>(G, posv, (int64_t)nh, hrec);
    }
    if (nitems > 0) {
        // the layout for the actual hub count (the carve above covers it)
        const size_t smem = hub_layout(n, (int32_t)nhubs, (int32_t)nhubs, 1 << 30, &H);
        if ((!H.smem_hist && !ghist) || ((int64_t)H.split < n && !gbm)) {
            na_msg(err, errlen, "internal: k_hub layout needs a global slice that was not carved");
            return PGD_ECUDA;
        }
        if ((int64_t)H.split < n) NA_CUDA(cudaMemsetAsync(gbm, 0, (size_t)nsm * nwords * 4, s));
        NA_CUDA(cudaFuncSetAttribute(k_hub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        H.G = G;
        H.hpos = posv;
        H.hrec = hrec;
        H.items = items;
        H.nitems = nitems;
        H.ghist = ghist;
        H.gbitmap = gbm;
        H.next = ctr + 1;
        H.thigh = nullptr;   // membership beyond the rank bitmap by searching N(q)
        k_hub<<<nsm, kHubWarps * 32, smem, s>>>(H);
    }
    const int64_t nlight = m - (int64_t)nh;
    if (nlight > 0) {
        LightArgs L;
        L.G = G;
        L.lpos = posv + nh;
        L.nlight = nlight;
        L.next = ctr + 2;
        k_light<<<nsm * 8, kLightWarps * 32, 0, s>>>(L);
    }
    NA_CUDA(cudaGetLastError());
    unsigned long long h[PGD_NSUMS];
    NA_CUDA(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < PGD_NSUMS; i++) out->sums[i] = h[i];
    pgd_close_counts(out->sums, n, m, out->totals);
    return PGD_OK;
}

// ---------------------------------------------------------------------------
// Batched decomposition straight from host pair lists: every graph's pairs
// are offset into its own vertex range on the device and the whole batch is
// built as one CSR (one sort), then decomposed with per-graph sums.  Used by
// the request server, where per-graph set-up would otherwise dominate.

namespace {

// Largest vertex id of each graph's pairs (self loops excluded).  The warp
// walks 32 consecutive pairs at a time; when they belong to one graph (the
// usual case) it reduces them first and issues one atomic.
__global__ void k_pairs_graph_max(const int64_t *pair_off, int k, const int32_t *src, const int32_t *dst, int64_t P,
                                  int *gmax, unsigned long long *bad) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; base < P; base += stride) {
        const int64_t i = base + lane;
        int g = -1, v = -1;
        if (i < P) {
            g = batch_find(pair_off, k, i);
            const int32_t a = src[i], b = dst[i];
            if (a < 0 || b < 0) atomicAdd(bad, 1ull);
            else if (a != b) v = max(a, b);
        }
        const int g0 = __shfl_sync(0xffffffffu, g, 0);   // lane 0's pair is in range: base < P
        if (__all_sync(0xffffffffu, g == g0 || g < 0)) {
            const int wmax = __reduce_max_sync(0xffffffffu, v);
            if (lane == 0 && wmax >= 0) atomicMax(gmax + g0, wmax);
        } else if (v >= 0) {
            atomicMax(gmax + g, v);
        }
    }
}

__global__ void k_pairs_shift(const int64_t *pair_off, int k, const int64_t *vbase, int64_t P, int32_t *src,
                              int32_t *dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P; i += (int64_t)gridDim.x * blockDim.x) {
        const int g = batch_find(pair_off, k, i);
        src[i] = (int32_t)(src[i] + vbase[g]);
        dst[i] = (int32_t)(dst[i] + vbase[g]);
    }
}

__global__ void k_vertex_graph(const int64_t *vbase, int k, int64_t N, int32_t *vgraph) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < N; x += (int64_t)gridDim.x * blockDim.x)
        vgraph[x] = batch_find(vbase, k, x);
}

__global__ void k_edge_graph(const int32_t *ev, const int32_t *vgraph, int64_t M, int32_t *egraph) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M; e += (int64_t)gridDim.x * blockDim.x)
        egraph[e] = vgraph[ev[e]];
}

__global__ void k_gather_offsets(const int64_t *off, const int64_t *vbase, int k, int64_t *out) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g <= k; g += (int64_t)gridDim.x * blockDim.x)
        out[g] = off[vbase[g]];
}

}  // namespace

pgd_status pgd_dev_decompose_pairs_batch(pgd_ctx *ctx, int k, const int64_t *pair_off, const int32_t *src,
                                         const int32_t *dst, const int64_t *n_min, pgd_counts *out) {
    cudaStream_t s = ctx->stream;
    pgd_status st;
    const int64_t P = pair_off[k];
    if (P < 0 || P > (int64_t)0x7fffffff) return pgd_fail(ctx, PGD_EINVAL, "pair count out of range");
    for (int g = 0; g < k; g++)
        if (pair_off[g + 1] < pair_off[g]) return pgd_fail(ctx, PGD_EINVAL, "pair offsets must not decrease");
    const int64_t P1 = P > 0 ? P : 1;
    int32_t *d_src = nullptr, *d_dst = nullptr, *vgraph = nullptr, *egraph = nullptr, *row = nullptr;
    int64_t *d_poff = nullptr, *d_vbase = nullptr, *d_goff = nullptr, *d_wbase = nullptr;
    int64_t *d_cbase = nullptr, *d_ctile = nullptr;
    uint16_t *cn = nullptr;
    int *gmax = nullptr;
    uint32_t *flag = nullptr, *pos = nullptr;
    unsigned long long *gsums = nullptr, *bits = nullptr;
    long long *d_gnm = nullptr;
    uint8_t *d_gdense = nullptr;
    pgd_graph *U = new pgd_graph();
    U->ctx = ctx;
    auto cleanup = [&]() {
        for (void *p : {(void *)d_src, (void *)d_dst, (void *)vgraph, (void *)egraph, (void *)row, (void *)d_poff,
                        (void *)d_vbase, (void *)d_goff, (void *)d_wbase, (void *)gmax, (void *)flag, (void *)pos,
                        (void *)gsums, (void *)bits, (void *)d_gnm, (void *)d_gdense, (void *)cn, (void *)d_cbase,
                        (void *)d_ctile})
            pgd_tmp_free(ctx, p);
        pgd_graph_destroy(U);
    };
#define PB_TRY(expr)                   \
    do {                               \
        if ((st = (expr)) != PGD_OK) { \
            cleanup();                 \
            return st;                 \
        }                              \
    } while (0)
#define PB_CUDA(call)                                                  \
    do {                                                               \
        cudaError_t e__ = (call);                                      \
        if (e__ != cudaSuccess) {                                      \
            st = pgd_cuda_fail(ctx, e__, #call);                       \
            cleanup();                                                 \
            return st;                                                 \
        }                                                              \
    } while (0)
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_src, P1 * sizeof(int32_t)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_dst, P1 * sizeof(int32_t)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_poff, (k + 1) * sizeof(int64_t)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_vbase, (k + 1) * sizeof(int64_t)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_goff, (k + 1) * sizeof(int64_t)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&gmax, (size_t)k * sizeof(int)));
    if (P > 0) {
        PB_CUDA(pgd_h2d(ctx, d_src, src, P * sizeof(int32_t)));
        PB_CUDA(pgd_h2d(ctx, d_dst, dst, P * sizeof(int32_t)));
    }
    PB_CUDA(cudaMemcpyAsync(d_poff, pair_off, (k + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    PB_CUDA(cudaMemsetAsync(gmax, 0xff, (size_t)k * sizeof(int), s));
    unsigned long long *bad = ctx->d_ctr + 7;
    PB_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s));
    if (P > 0) PGD_LAUNCH(ctx, k_pairs_graph_max, grid_for(P), kThreads, 0, d_poff, k, d_src, d_dst, P, gmax, bad);
    std::vector<int> hmax((size_t)k);
    unsigned long long hbad = 0;
    PB_CUDA(cudaMemcpyAsync(hmax.data(), gmax, (size_t)k * sizeof(int), cudaMemcpyDeviceToHost, s));
    PB_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, s));
    PB_CUDA(cudaStreamSynchronize(s));
    if (hbad) {
        cleanup();
        return pgd_fail(ctx, PGD_EINVAL, "negative vertex id in a batched edge list");
    }
    std::vector<int64_t> vbase((size_t)k + 1, 0);
    for (int g = 0; g < k; g++) {
        int64_t ng = std::max<int64_t>(n_min ? n_min[g] : 0, (int64_t)hmax[(size_t)g] + 1);
        vbase[(size_t)g + 1] = vbase[(size_t)g] + ng;
    }
    const int64_t N = vbase[(size_t)k];
    if (N > 0x7ffffffe) {
        cleanup();
        return pgd_fail(ctx, PGD_EINVAL, "batch too large for 32-bit vertex ids");
    }
    PB_CUDA(cudaMemcpyAsync(d_vbase, vbase.data(), (k + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    if (P > 0) PGD_LAUNCH(ctx, k_pairs_shift, grid_for(P), kThreads, 0, d_poff, k, d_vbase, P, d_src, d_dst);
    // one CSR for the whole batch: symmetrised, deduplicated, self loops dropped
    PB_TRY(pgd_build_from_device_pairs(U, d_src, d_dst, P, N, true));
    pgd_tmp_free(ctx, d_src);
    pgd_tmp_free(ctx, d_dst);
    d_src = d_dst = nullptr;
    const int64_t M = U->m, nnz = 2 * M;
    // per-graph edge counts from the offsets at the range boundaries
    std::vector<int64_t> goff((size_t)k + 1);
    PGD_LAUNCH(ctx, k_gather_offsets, grid_for(k + 1), kThreads, 0, U->off, d_vbase, k, d_goff);
    PB_CUDA(cudaMemcpyAsync(goff.data(), d_goff, (k + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    // edge arrays (edge id = position: the order does not change a global count)
    PB_TRY(pgd_graph_alloc(U, (void **)&U->ev, (M + 1) * sizeof(int32_t)));
    PB_TRY(pgd_graph_alloc(U, (void **)&U->eu, (M + 1) * sizeof(int32_t)));
    PB_TRY(pgd_graph_alloc(U, (void **)&U->order, (M + 1) * sizeof(int32_t)));
    U->norder = M;
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&row, (nnz + 1) * sizeof(int32_t)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&flag, (nnz + 1) * sizeof(uint32_t)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&pos, (nnz + 1) * sizeof(uint32_t)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&vgraph, (N + 1) * sizeof(int32_t)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&egraph, (M + 1) * sizeof(int32_t)));
    if (nnz > 0) {
        PGD_LAUNCH(ctx, k_rows, grid_for(nnz), kThreads, 0, U->off, N, nnz, row);
        PGD_LAUNCH(ctx, k_na_edge_flags, grid_for(nnz), kThreads, 0, row, U->adj, nnz, flag);
        PB_CUDA(cudaMemsetAsync(flag + nnz, 0, sizeof(uint32_t), s));
        size_t tb = 0;
        void *tmp = nullptr;
        cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, pos, nnz + 1, s);
        PB_TRY(pgd_tmp_alloc(ctx, &tmp, tb));
        cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, nnz + 1, s);
        pgd_tmp_free(ctx, tmp);
        PGD_LAUNCH(ctx, k_na_edges, grid_for(nnz), kThreads, 0, row, U->adj, flag, pos, nnz, U->ev, U->eu, U->order);
    }
    if (N > 0) PGD_LAUNCH(ctx, k_vertex_graph, grid_for(N), kThreads, 0, d_vbase, k, N, vgraph);
    if (M > 0) PGD_LAUNCH(ctx, k_edge_graph, grid_for(M), kThreads, 0, U->ev, vgraph, M, egraph);
    PB_CUDA(cudaStreamSynchronize(s));
    // per-graph n, m, dense flags
    std::vector<long long> gnm((size_t)2 * k);
    std::vector<uint8_t> gdense((size_t)k, 0);
    std::vector<int64_t> wbase((size_t)k, 0);
    int64_t words = 0;
    int ndense_graphs = 0;
    for (int g = 0; g < k; g++) {
        const int64_t ng = vbase[(size_t)g + 1] - vbase[(size_t)g];
        const int64_t mg = (goff[(size_t)g + 1] - goff[(size_t)g]) / 2;
        gnm[(size_t)2 * g] = ng;
        gnm[(size_t)2 * g + 1] = mg;
        if (ng > 0 && ng <= ctx->dense_max && mg > 0) {
            gdense[(size_t)g] = 1;
            wbase[(size_t)g] = words;
            words += ng * ((ng + 63) / 64);
            ndense_graphs++;
        }
    }
    std::vector<int64_t> cbase, ctile;
    const int64_t cn_entries = plan_common(k, gnm, gdense, cbase, ctile);
    if (cn_entries > 0) {
        PB_TRY(pgd_tmp_alloc(ctx, (void **)&cn, (size_t)cn_entries * sizeof(uint16_t)));
        PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_cbase, (size_t)k * sizeof(int64_t)));
        PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_ctile, ((size_t)k + 1) * sizeof(int64_t)));
        PB_CUDA(cudaMemcpyAsync(d_cbase, cbase.data(), (size_t)k * sizeof(int64_t), cudaMemcpyHostToDevice, s));
        PB_CUDA(cudaMemcpyAsync(d_ctile, ctile.data(), ((size_t)k + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    }
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&gsums, (size_t)k * PGD_NSUMS * sizeof(unsigned long long)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_gnm, gnm.size() * sizeof(long long)));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_gdense, (size_t)k));
    PB_TRY(pgd_tmp_alloc(ctx, (void **)&d_wbase, (size_t)k * sizeof(int64_t)));
    if (words > 0) PB_TRY(pgd_tmp_alloc(ctx, (void **)&bits, (size_t)words * sizeof(unsigned long long)));
    PB_CUDA(cudaMemsetAsync(gsums, 0, (size_t)k * PGD_NSUMS * sizeof(unsigned long long), s));
    PB_CUDA(cudaMemcpyAsync(d_gnm, gnm.data(), gnm.size() * sizeof(long long), cudaMemcpyHostToDevice, s));
    PB_CUDA(cudaMemcpyAsync(d_gdense, gdense.data(), (size_t)k, cudaMemcpyHostToDevice, s));
    PB_CUDA(cudaMemcpyAsync(d_wbase, wbase.data(), (size_t)k * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    if (words > 0) PB_CUDA(cudaMemsetAsync(bits, 0, (size_t)words * sizeof(unsigned long long), s));
    StageMs ms;
    if (M > 0) {
        PB_TRY(build_aux(U));
        if (words > 0)
            PGD_LAUNCH(ctx, k_dense_bits, grid_for(32 * N), kThreads, 0, U->off, U->adj, vgraph, d_gdense, d_wbase,
                       d_vbase, d_gnm, N, bits);
        if (cn_entries > 0)
            PGD_LAUNCH(ctx, k_dense_common, (int)std::min<int64_t>(ctile[(size_t)k], (int64_t)ctx->num_sms * 8), 256,
                       0, (const uint64_t *)bits, d_wbase, d_gnm, d_cbase, d_ctile, k, ctile[(size_t)k], cn);
        DevGraph G = dev_view(U, false);
        G.sums = gsums;
        G.egraph = egraph;
        G.gnm = d_gnm;
        G.gdense = ndense_graphs ? d_gdense : nullptr;
        DenseView dv{(const uint64_t *)bits, d_wbase, d_vbase, cn, d_cbase, k};
        PB_TRY(run_decompose(ctx, G, (int4 *)U->slot, U->nhubs, U->nhubs_wide, U->max_degree, &ms, ndense_graphs ? &dv : nullptr));
    }
    std::vector<unsigned long long> h((size_t)k * PGD_NSUMS);
    PB_CUDA(cudaMemcpyAsync(h.data(), gsums, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    PB_CUDA(cudaStreamSynchronize(s));
    for (int g = 0; g < k; g++) {
        pgd_counts &o = out[g];
        memset(&o, 0, sizeof(o));
        for (int j = 0; j < PGD_NSUMS; j++) o.sums[j] = h[(size_t)g * PGD_NSUMS + j];
        o.n = gnm[(size_t)2 * g];
        o.m = gnm[(size_t)2 * g + 1];
        o.kernel_ms = ms.total;
        o.hub_ms = ms.hub;
        o.tri_ms = ms.tri;
        pgd_close_counts(o.sums, o.n, o.m, o.totals);
    }
    cleanup();
#undef PB_TRY
#undef PB_CUDA
    return PGD_OK;
}
