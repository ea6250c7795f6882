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
//     W(w,p) of a hub w is computed once per anchor (a cache), not once per
//     edge; t(x,q) is read from a per-slot array filled by a triangle pass.
//   * k4 counts each edge inside T once, from its lower endpoint, by scanning
//     the degree-oriented list N+(x) (neighbours of higher degree, short even
//     for hubs) of every x in T.
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

#include "pgd_internal.h"
#include "pgd_kernels.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kHubWarps = 16;            // hub-anchor CTA: 512 threads
constexpr int kLightWarps = 8;           // light path: 256 threads, one edge per warp
constexpr int kAnchorHub = 128;          // anchors of degree >= this take the bitmap path
constexpr int kCacheHub = 64;            // W(w,p) cached for neighbours of degree >= this
constexpr int kChunk = 2048;             // max edges of one anchor per CTA work item
constexpr uint32_t kPending = 0xffffffffu;
constexpr int kMaxSmemBitmap = 160 * 1024;

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
    const uint32_t *tslot;
    const int32_t *ev;
    const int32_t *eu;
    const int32_t *order;
    long long n, m;
    uint64_t *micro;
    unsigned long long *sums;
};

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

__global__ void k_hub_flags(const int32_t *deg, int64_t n, uint32_t *flag) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        flag[v] = deg[v] >= kCacheHub ? 1u : 0u;
}

__global__ void k_hub_ids(const uint32_t *flag, const uint32_t *pos, int64_t n, int32_t *hubid) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        hubid[v] = flag[v] ? (int32_t)pos[v] : -1;
}

// t of every edge, written to both of its CSR slots.  One warp per edge:
// the shorter list's entries are searched in the longer one.
__global__ void k_tslot(DevGraph G, uint32_t *tslot) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t id = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; id < G.m; id += nw) {
        const int32_t a = G.ev[id], b = G.eu[id];
        const int da = G.deg[a], db = G.deg[b];
        const int32_t s = da <= db ? a : b, l = da <= db ? b : a;
        const int ds = da <= db ? da : db, dl = da <= db ? db : da;
        const int32_t *Ns = G.adj + G.off[s], *Nl = G.adj + G.off[l];
        unsigned long long t = 0;
        for (int i = lane; i < ds; i += 32) t += pgd_contains(Nl, dl, __ldg(Ns + i)) ? 1 : 0;
        t = pgd_warp_sum(t);
        if (lane == 0) tslot[G.off[a] + pgd_lower_bound(G.adj + G.off[a], da, b)] = (uint32_t)t;
        if (lane == 1) tslot[G.off[b] + pgd_lower_bound(G.adj + G.off[b], db, a)] = (uint32_t)t;
    }
}

// ---------------------------------------------------------------------------
// work plan: hub-anchored edges grouped by anchor, light edges listed

// key = (anchor << 32 | position) for hub-anchored edges, (~0 << 32 | position)
// for the rest, so one sort groups the first and lists the second in order.
__global__ void k_plan_keys(DevGraph G, uint64_t *keys, unsigned long long *nhub) {
    unsigned long long local = 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < G.m; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t id = G.order[e];
        const int32_t v = G.ev[id], u = G.eu[id];
        const int32_t p = ranks_above(v, u, G.deg) ? v : u;
        const bool hub = G.deg[p] >= kAnchorHub;
        keys[e] = ((uint64_t)(hub ? (uint32_t)p : 0xffffffffu) << 32) | (uint32_t)e;
        local += hub;
    }
    local = pgd_warp_sum(local);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(nhub, local);
}

// item i starts a chunk: first edge of an anchor, or every kChunk-th of it
__global__ void k_item_flags(const uint64_t *keys, int64_t nh, uint32_t *flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = (uint32_t)(keys[i] >> 32);
        // first index of this anchor's run
        int64_t lo = 0, hi = i;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if ((uint32_t)(keys[mid] >> 32) < p) lo = mid + 1; else hi = mid;
        }
        flag[i] = ((i - lo) % kChunk == 0) ? 1u : 0u;
    }
}

__global__ void k_item_fill(const uint32_t *flag, const uint32_t *pos, int64_t nh, int64_t *items) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh; i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) items[pos[i]] = i;
    if (blockIdx.x == 0 && threadIdx.x == 0) items[pos[nh]] = nh;
}

__global__ void k_keys_pos(const uint64_t *keys, int64_t n, int32_t *posv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        posv[i] = (int32_t)(uint32_t)(keys[i] & 0xffffffffu);
}

// ---------------------------------------------------------------------------
// shared per-edge epilogue

__device__ __forceinline__ void edge_epilogue(const DevGraph &G, unsigned long long *acc, int64_t e, int32_t v,
                                              int32_t u, unsigned long long t, unsigned long long k4,
                                              unsigned long long c4, int lane) {
    const long long dv = G.deg[v], du = G.deg[u];
    if (lane == 0) {
        pgd_edge_sums(acc, dv, du, t, G.m, G.n);
        acc[3] += k4;
        acc[4] += c4;
    }
    if (G.micro && lane < PGD_NMICRO) G.micro[e * PGD_NMICRO + lane] = pgd_micro_col(lane, dv, du, t, k4, c4);
}

__device__ __forceinline__ void block_flush(unsigned long long *acc, unsigned long long (*red)[PGD_NSUMS], int nwarps,
                                            unsigned long long *sums) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < PGD_NSUMS; i++) red[wid][i] = acc[i];
    }
    __syncthreads();
    if (threadIdx.x < PGD_NSUMS) {
        unsigned long long s = 0;
        for (int w = 0; w < nwarps; w++) s += red[w][threadIdx.x];
        atomicAdd(sums + threadIdx.x, s);
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

__device__ __forceinline__ bool bit_of(const uint32_t *bm, int32_t x) { return (bm[x >> 5] >> (x & 31)) & 1u; }

// ---------------------------------------------------------------------------
// Hub anchors: one CTA per (anchor, chunk of its edges).
//
// Per work item: (1) N(p) into the bitmap; (2) every hub w adjacent to a q
// of the chunk but not to p is claimed in this CTA's W cache and queued;
// (3) the queue is drained, one warp per W(w,p); (4) the chunk's edges are
// decomposed, one warp each, fetched dynamically.  Per edge the warp first
// collects T (sorted, in shared memory when it fits), t and the cached W's,
// then scans the remaining lists: N(w) of non-hub w in S_q (W by bit tests)
// and N+(x) of x in T (k4 by bit test and T membership).  Lists of 32 or more
// entries are read warp-cooperatively with four loads in flight per lane;
// shorter ones are flattened across the warp.

constexpr int kTCap = 512;               // T entries kept in shared memory per warp
constexpr int kQueue = 2048;             // queued W computations per CTA

struct HubArgs {
    DevGraph G;
    const int32_t *hpos;      // E_ordered positions of hub-anchored edges, grouped by anchor
    const int64_t *items;     // chunk starts into hpos, nitems+1 entries
    int64_t nitems;
    unsigned long long *cache;  // per CTA: nhubs entries (anchor << 32 | W)
    int32_t nhubs;
    uint32_t *gbitmap;        // per CTA bitmap slices when not in shared memory
    int64_t nwords;
    int smem_bitmap;
    unsigned long long *next;
};

// |{x in L[0..len) : bit(x)}|, warp-cooperative, 4 loads in flight per lane.
__device__ __forceinline__ unsigned count_bits(const uint32_t *bm, const int32_t *L, int len, int lane) {
    unsigned c = 0;
    int i = lane;
    for (; i + 96 < len; i += 128) {
        const int32_t x0 = __ldg(L + i), x1 = __ldg(L + i + 32), x2 = __ldg(L + i + 64), x3 = __ldg(L + i + 96);
        c += bit_of(bm, x0) + bit_of(bm, x1) + bit_of(bm, x2) + bit_of(bm, x3);
    }
    for (; i < len; i += 32) c += bit_of(bm, __ldg(L + i));
    return c;
}

// y in T: T sorted in shared memory (small T) or N(q) searched in global memory.
__device__ __forceinline__ bool in_t(const int32_t *Ts, int t, bool small, const int32_t *Nq, int dq, int32_t y) {
    return small ? pgd_contains(Ts, t, y) : pgd_contains(Nq, dq, y);
}

__global__ void __launch_bounds__(kHubWarps * 32, 1) k_hub(HubArgs A) {
    extern __shared__ uint32_t s_bits[];
    __shared__ unsigned long long s_red[kHubWarps][PGD_NSUMS];
    __shared__ int32_t s_T[kHubWarps][kTCap];
    __shared__ int32_t s_qw[kQueue];
    __shared__ int32_t s_qh[kQueue];
    __shared__ long long s_item;
    __shared__ int s_qlen, s_qnext, s_enext_a, s_enext_c;
    const DevGraph &G = A.G;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t *Ts = s_T[wid];
    uint32_t *bm = A.smem_bitmap ? s_bits : A.gbitmap + (int64_t)blockIdx.x * A.nwords;
    unsigned long long *cache = A.cache + (int64_t)blockIdx.x * A.nhubs;
    unsigned long long acc[PGD_NSUMS];
#pragma unroll
    for (int i = 0; i < PGD_NSUMS; i++) acc[i] = 0;
    if (A.smem_bitmap)
        for (int64_t i = threadIdx.x; i < A.nwords; i += blockDim.x) bm[i] = 0;
    __syncthreads();

    while (true) {
        if (threadIdx.x == 0) {
            s_item = (long long)atomicAdd(A.next, 1ull);
            s_qlen = 0;
            s_qnext = 0;
            s_enext_a = 0;
            s_enext_c = 0;
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
        for (int i = threadIdx.x; i < dp; i += blockDim.x) {
            const int32_t y = __ldg(Np + i);
            atomicOr(bm + (y >> 5), 1u << (y & 31));
        }
        __syncthreads();

        // ---- (2) claim the hub neighbours whose W(w,p) is needed ----------
        while (true) {
            int k = 0;
            if (lane == 0) k = atomicAdd(&s_enext_a, 1);
            k = __shfl_sync(0xffffffffu, k, 0);
            if (k >= nedge) break;
            const int32_t id = G.order[A.hpos[start + k]];
            const int32_t q = (G.ev[id] == p) ? G.eu[id] : G.ev[id];
            const int dq = G.deg[q];
            const int32_t *Nq = G.adj + G.off[q];
            for (int base = 0; base < dq; base += 32) {
                const int j = base + lane;
                bool claim = false;
                int32_t w = -1, h = -1;
                if (j < dq) {
                    w = __ldg(Nq + j);
                    if (w != p && !bit_of(bm, w) && (h = G.hubid[w]) >= 0) {
                        const unsigned long long ent = cache[h];
                        if ((uint32_t)(ent >> 32) != (uint32_t)p) {
                            const unsigned long long mine = ((unsigned long long)(uint32_t)p << 32) | kPending;
                            claim = atomicCAS(cache + h, ent, mine) == ent;
                        }
                    }
                }
                const unsigned mask = __ballot_sync(0xffffffffu, claim);
                if (!mask) continue;
                int slot = 0;
                if (lane == 0) slot = atomicAdd(&s_qlen, __popc(mask));
                slot = __shfl_sync(0xffffffffu, slot, 0) + __popc(mask & ((1u << lane) - 1));
                if (claim && slot < kQueue) {
                    s_qw[slot] = w;
                    s_qh[slot] = h;
                }
                // queue full: compute here
                unsigned over = __ballot_sync(0xffffffffu, claim && slot >= kQueue);
                while (over) {
                    const int src = __ffs(over) - 1;
                    over &= over - 1;
                    const int32_t wc = __shfl_sync(0xffffffffu, w, src);
                    const int32_t hc = __shfl_sync(0xffffffffu, h, src);
                    unsigned long long c = count_bits(bm, G.adj + G.off[wc], G.deg[wc], lane);
                    c = pgd_warp_sum(c);
                    if (lane == 0) cache[hc] = ((unsigned long long)(uint32_t)p << 32) | (uint32_t)c;
                }
            }
        }
        __syncthreads();

        // ---- (3) drain the queue ------------------------------------------
        {
            const int qlen = min(s_qlen, kQueue);
            while (true) {
                int k = 0;
                if (lane == 0) k = atomicAdd(&s_qnext, 1);
                k = __shfl_sync(0xffffffffu, k, 0);
                if (k >= qlen) break;
                const int32_t w = s_qw[k];
                unsigned long long c = count_bits(bm, G.adj + G.off[w], G.deg[w], lane);
                c = pgd_warp_sum(c);
                if (lane == 0) cache[s_qh[k]] = ((unsigned long long)(uint32_t)p << 32) | (uint32_t)c;
            }
        }
        __syncthreads();

        // ---- (4) the chunk's edges ---------------------------------------
        while (true) {
            int k = 0;
            if (lane == 0) k = atomicAdd(&s_enext_c, 1);
            k = __shfl_sync(0xffffffffu, k, 0);
            if (k >= nedge) break;
            const int64_t e = A.hpos[start + k];
            const int32_t id = G.order[e];
            const int32_t v = G.ev[id], u = G.eu[id];
            const int32_t q = (v == p) ? u : v;
            const int dq = G.deg[q];
            const int64_t offq = G.off[q];
            const int32_t *Nq = G.adj + offq;
            // pass 1: T (sorted), t, sum of t(x,q) over T, cached W's
            unsigned t = 0;
            unsigned long long sumtq = 0, sumW = 0, k4 = 0;
            for (int base = 0; base < dq; base += 32) {
                const int j = base + lane;
                bool inT = false;
                int32_t w = -1;
                if (j < dq) {
                    w = __ldg(Nq + j);
                    if (w != p) {
                        if (bit_of(bm, w)) {
                            inT = true;
                            sumtq += G.tslot[offq + j];
                        } else {
                            const int32_t h = G.hubid[w];
                            if (h >= 0) sumW += (uint32_t)cache[h];
                        }
                    }
                }
                const unsigned mask = __ballot_sync(0xffffffffu, inT);
                const unsigned at = t + __popc(mask & ((1u << lane) - 1));
                if (inT && at < (unsigned)kTCap) Ts[at] = w;
                t += __popc(mask);
            }
            __syncwarp();
            const bool tsmall = t <= (unsigned)kTCap;
            // pass 2: scan N(w) of non-hub w in S_q and N+(x) of x in T
            for (int base = 0; base < dq; base += 32) {
                const int j = base + lane;
                int len = 0, kind = 0;
                const int32_t *list = nullptr;
                if (j < dq) {
                    const int32_t w = __ldg(Nq + j);
                    if (w != p) {
                        if (bit_of(bm, w)) {
                            kind = 1;
                            const int64_t o = G.offp[w];
                            len = (int)(G.offp[w + 1] - o);
                            list = G.adjp + o;
                        } else if (G.hubid[w] < 0) {
                            len = G.deg[w];
                            list = G.adj + G.off[w];
                        }
                    }
                }
                // long lists: one at a time, warp-cooperative
                unsigned longm = __ballot_sync(0xffffffffu, len >= 32);
                while (longm) {
                    const int src = __ffs(longm) - 1;
                    longm &= longm - 1;
                    const int32_t *L = (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)list, src);
                    const int ln = __shfl_sync(0xffffffffu, len, src);
                    if (__shfl_sync(0xffffffffu, kind, src) == 0) {
                        sumW += count_bits(bm, L, ln, lane);
                    } else {
                        for (int i = lane; i < ln; i += 32) {
                            const int32_t y = __ldg(L + i);
                            k4 += (bit_of(bm, y) && in_t(Ts, (int)t, tsmall, Nq, dq, y)) ? 1 : 0;
                        }
                    }
                }
                // short lists: flattened over the warp
                if (len >= 32) len = 0;
                const int incl = pgd_warp_incl_scan(len);
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                const int excl = incl - len;
                for (int b2 = 0; b2 < total; b2 += 32) {
                    const int it = b2 + lane;
                    const int own = owner_of(incl, it);
                    const int32_t *olist =
                        (const int32_t *)__shfl_sync(0xffffffffu, (unsigned long long)list, own);
                    const int okind = __shfl_sync(0xffffffffu, kind, own);
                    const int oexcl = __shfl_sync(0xffffffffu, excl, own);
                    if (it < total) {
                        const int32_t x = __ldg(olist + (it - oexcl));
                        if (okind == 0) sumW += bit_of(bm, x);
                        else k4 += (bit_of(bm, x) && in_t(Ts, (int)t, tsmall, Nq, dq, x)) ? 1 : 0;
                    }
                }
            }
            sumtq = pgd_warp_sum(sumtq);
            sumW = pgd_warp_sum(sumW);
            k4 = pgd_warp_sum(k4);
            const long long c4 = (long long)sumW - ((long long)dq - (long long)t - 1) - (long long)sumtq +
                                 2 * (long long)k4 + (long long)t;
            edge_epilogue(G, acc, e, v, u, t, k4, (unsigned long long)c4, lane);
            __syncwarp();
        }
        __syncthreads();
        for (int i = threadIdx.x; i < dp; i += blockDim.x) bm[__ldg(Np + i) >> 5] = 0;
        __syncthreads();
    }
    block_flush(acc, s_red, kHubWarps, G.sums);
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
    __shared__ int32_t s_np[kLightWarps][kAnchorHub];
    __shared__ uint8_t s_lab[kLightWarps][kAnchorHub];
    __shared__ unsigned long long s_red[kLightWarps][PGD_NSUMS];
    const DevGraph &G = A.G;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t *np_s = s_np[wid];
    uint8_t *lab_s = s_lab[wid];
    unsigned long long acc[PGD_NSUMS];
#pragma unroll
    for (int i = 0; i < PGD_NSUMS; i++) acc[i] = 0;

    while (true) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(A.next, 1ull);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= (unsigned long long)A.nlight) break;
        const int64_t e = A.lpos[idx];
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
                        sumtq += G.tslot[offq + j];
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
        edge_epilogue(G, acc, e, v, u, t, k4, (unsigned long long)c4, lane);
        __syncwarp();
    }
    block_flush(acc, s_red, kLightWarps, G.sums);
}

}  // namespace

// ---------------------------------------------------------------------------

static pgd_status build_aux(pgd_graph *g) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    const int64_t n = g->n, nnz = 2 * g->m;
    if ((st = pgd_graph_alloc(g, (void **)&g->offp, (n + 1) * sizeof(int64_t)))) return st;
    if ((st = pgd_graph_alloc(g, (void **)&g->adjp, (g->m + 1) * sizeof(int32_t)))) return st;
    if ((st = pgd_graph_alloc(g, (void **)&g->hubid, (n + 1) * sizeof(int32_t)))) return st;
    if ((st = pgd_graph_alloc(g, (void **)&g->tslot, (nnz + 1) * sizeof(uint32_t)))) return st;
    int32_t *row = nullptr;
    uint32_t *flag = nullptr, *pos = nullptr;
    const int64_t len = std::max(nnz, n) + 1;
    if ((st = pgd_tmp_alloc(ctx, (void **)&row, (nnz + 1) * sizeof(int32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&flag, len * sizeof(uint32_t)))) return st;
    if ((st = pgd_tmp_alloc(ctx, (void **)&pos, len * sizeof(uint32_t)))) return st;
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
    // hub ids
    PGD_LAUNCH(ctx, k_hub_flags, grid_for(n), kThreads, 0, g->deg, n, flag);
    PGD_CUDA(ctx, cudaMemsetAsync(flag + n, 0, sizeof(uint32_t), s));
    tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, pos, n + 1, s);
    if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
    cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, n + 1, s);
    pgd_tmp_free(ctx, tmp);
    PGD_LAUNCH(ctx, k_hub_ids, grid_for(n), kThreads, 0, flag, pos, n, g->hubid);
    uint32_t nh = 0;
    PGD_CUDA(ctx, cudaMemcpyAsync(&nh, pos + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    g->nhubs = (int32_t)nh;
    pgd_tmp_free(ctx, row);
    pgd_tmp_free(ctx, flag);
    pgd_tmp_free(ctx, pos);
    PGD_CUDA(ctx, cudaGetLastError());
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
    G.tslot = g->tslot;
    G.ev = g->ev;
    G.eu = g->eu;
    G.order = g->order;
    G.n = g->n;
    G.m = g->m;
    G.micro = micro ? g->micro : nullptr;
    G.sums = g->ctx->d_sums;
    return G;
}

pgd_status pgd_dev_decompose(pgd_graph *g, bool micro, pgd_counts *out) {
    pgd_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    pgd_status st;
    if (micro && !g->micro) {
        if ((st = pgd_graph_alloc(g, (void **)&g->micro, (g->m + 1) * PGD_NMICRO * sizeof(uint64_t)))) return st;
    }
    if (!g->has_aux && (st = build_aux(g))) return st;
    const int64_t m = g->m;
    PGD_CUDA(ctx, cudaMemsetAsync(ctx->d_sums, 0, PGD_NSUMS * sizeof(unsigned long long), s));
    DevGraph G = dev_view(g, micro);
    float ms = 0;
    if (m > 0) {
        // work plan
        uint64_t *keys = nullptr, *keys2 = nullptr;
        int32_t *posv = nullptr;
        uint32_t *flag = nullptr, *fpos = nullptr;
        int64_t *items = nullptr;
        unsigned long long *cache = nullptr;
        uint32_t *gbm = nullptr;
        if ((st = pgd_tmp_alloc(ctx, (void **)&keys, m * sizeof(uint64_t)))) return st;
        if ((st = pgd_tmp_alloc(ctx, (void **)&keys2, m * sizeof(uint64_t)))) return st;
        if ((st = pgd_tmp_alloc(ctx, (void **)&posv, m * sizeof(int32_t)))) return st;
        unsigned long long *ctr = ctx->d_ctr;  // [0] hub edges, [1] hub item counter, [2] light counter
        PGD_CUDA(ctx, cudaMemsetAsync(ctr, 0, 4 * sizeof(unsigned long long), s));
        PGD_CUDA(ctx, cudaEventRecord(ctx->ev0, s));
        PGD_LAUNCH(ctx, k_tslot, grid_for(32 * m), kThreads, 0, G, g->tslot);
        PGD_LAUNCH(ctx, k_plan_keys, grid_for(m), kThreads, 0, G, keys, ctr);
        size_t tb = 0;
        void *tmp = nullptr;
        cub::DeviceRadixSort::SortKeys(nullptr, tb, keys, keys2, m, 0, 64, s);
        if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
        cub::DeviceRadixSort::SortKeys(tmp, tb, keys, keys2, m, 0, 64, s);
        pgd_tmp_free(ctx, tmp);
        PGD_LAUNCH(ctx, k_keys_pos, grid_for(m), kThreads, 0, keys2, m, posv);
        unsigned long long nh = 0;
        PGD_CUDA(ctx, cudaMemcpyAsync(&nh, ctr, sizeof(nh), cudaMemcpyDeviceToHost, s));
        PGD_CUDA(ctx, cudaStreamSynchronize(s));
        const int64_t nlight = m - (int64_t)nh;
        int64_t nitems = 0;
        if (nh > 0) {
            if ((st = pgd_tmp_alloc(ctx, (void **)&flag, (nh + 1) * sizeof(uint32_t)))) return st;
            if ((st = pgd_tmp_alloc(ctx, (void **)&fpos, (nh + 1) * sizeof(uint32_t)))) return st;
            PGD_LAUNCH(ctx, k_item_flags, grid_for(nh), kThreads, 0, keys2, (int64_t)nh, flag);
            PGD_CUDA(ctx, cudaMemsetAsync(flag + nh, 0, sizeof(uint32_t), s));
            tb = 0;
            cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, fpos, (int64_t)nh + 1, s);
            if ((st = pgd_tmp_alloc(ctx, &tmp, tb))) return st;
            cub::DeviceScan::ExclusiveSum(tmp, tb, flag, fpos, (int64_t)nh + 1, s);
            pgd_tmp_free(ctx, tmp);
            uint32_t ni = 0;
            PGD_CUDA(ctx, cudaMemcpyAsync(&ni, fpos + nh, sizeof(ni), cudaMemcpyDeviceToHost, s));
            PGD_CUDA(ctx, cudaStreamSynchronize(s));
            nitems = ni;
            if ((st = pgd_tmp_alloc(ctx, (void **)&items, (nitems + 1) * sizeof(int64_t)))) return st;
            PGD_LAUNCH(ctx, k_item_fill, grid_for(nh), kThreads, 0, flag, fpos, (int64_t)nh, items);
        }
        const int nsm = ctx->num_sms;
        if (nitems > 0) {
            const int64_t nwords = (g->n + 31) / 32;
            const bool in_smem = nwords * 4 <= kMaxSmemBitmap;
            size_t smem = in_smem ? (size_t)nwords * 4 : 0;
            const int nhubs = std::max(1, (int)g->nhubs);
            if ((st = pgd_tmp_alloc(ctx, (void **)&cache, (size_t)nsm * nhubs * sizeof(unsigned long long)))) return st;
            PGD_CUDA(ctx, cudaMemsetAsync(cache, 0xff, (size_t)nsm * nhubs * sizeof(unsigned long long), s));
            if (!in_smem) {
                if ((st = pgd_tmp_alloc(ctx, (void **)&gbm, (size_t)nsm * nwords * 4))) return st;
                PGD_CUDA(ctx, cudaMemsetAsync(gbm, 0, (size_t)nsm * nwords * 4, s));
            }
            PGD_CUDA(ctx, cudaFuncSetAttribute(k_hub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            HubArgs H;
            H.G = G;
            H.hpos = posv;
            H.items = items;
            H.nitems = nitems;
            H.cache = cache;
            H.nhubs = nhubs;
            H.gbitmap = gbm;
            H.nwords = nwords;
            H.smem_bitmap = in_smem ? 1 : 0;
            H.next = ctr + 1;
            PGD_LAUNCH(ctx, k_hub, nsm, kHubWarps * 32, smem, H);
        }
        if (nlight > 0) {
            LightArgs L;
            L.G = G;
            L.lpos = posv + nh;
            L.nlight = nlight;
            L.next = ctr + 2;
            PGD_LAUNCH(ctx, k_light, nsm * 8, kLightWarps * 32, 0, L);
        }
        PGD_CUDA(ctx, cudaEventRecord(ctx->ev1, s));
        PGD_CUDA(ctx, cudaGetLastError());
        pgd_tmp_free(ctx, keys);
        pgd_tmp_free(ctx, keys2);
        pgd_tmp_free(ctx, posv);
        pgd_tmp_free(ctx, flag);
        pgd_tmp_free(ctx, fpos);
        pgd_tmp_free(ctx, items);
        pgd_tmp_free(ctx, cache);
        pgd_tmp_free(ctx, gbm);
    }
    unsigned long long h[PGD_NSUMS];
    PGD_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_sums, sizeof(h), cudaMemcpyDeviceToHost, s));
    PGD_CUDA(ctx, cudaStreamSynchronize(s));
    if (m > 0) PGD_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    for (int i = 0; i < PGD_NSUMS; i++) out->sums[i] = h[i];
    out->n = g->n;
    out->m = g->m;
    out->kernel_ms = ms;
    pgd_close_counts(out->sums, g->n, g->m, out->totals);
    g->has_micro = micro;
    return PGD_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free decomposition (no counterpart in the reference).
//
// Some callers cannot allocate device memory at the moment they need counts:
// code inside a framework that hands out a fixed workspace and forbids
// allocation (inference plugins, custom ops), code recorded into a CUDA
// stream capture where cudaMalloc is not permitted, and latency-critical
// loops where cudaMalloc/cudaFree would synchronise the device.  For them
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
// the first call on that device, so that first call should come before any
// stream capture.

namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_addr[kNoAllocMaxDevices] = {};

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
    const bool in_smem = nwords * 4 <= kMaxSmemBitmap;
    const int64_t hub_bound = std::max<int64_t>(1, std::min<int64_t>(n, nnz / kCacheHub + 1));

    // CUB temporary storage sizes (queries only)
    size_t tb_scan = 0, tb_sort = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb_scan, (uint32_t *)nullptr, (uint32_t *)nullptr, std::max(nnz, n) + 1, s);
    cub::DeviceRadixSort::SortKeys(nullptr, tb_sort, (uint64_t *)nullptr, (uint64_t *)nullptr, std::max<int64_t>(m, 1),
                                   0, 64, s);

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
    uint32_t *tslot = C.take<uint32_t>(nnz + 1);
    uint64_t *keys = C.take<uint64_t>(m + 1);
    uint64_t *keys2 = C.take<uint64_t>(m + 1);
    int32_t *posv = C.take<int32_t>(m + 1);
    uint32_t *iflag = C.take<uint32_t>(m + 2);
    uint32_t *ipos = C.take<uint32_t>(m + 2);
    int64_t *items = C.take<int64_t>(m + 2);
    unsigned long long *cache = C.take<unsigned long long>((size_t)nsm * hub_bound);
    uint32_t *gbm = in_smem ? nullptr : C.take<uint32_t>((size_t)nsm * nwords);
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
    // validate and derive the per-graph structures
    k_rows<<<grid_for(nnz), kThreads, 0, s>>>(d_off, n, nnz, row);
    k_na_check<<<grid_for(nnz), kThreads, 0, s>>>(d_off, d_adj, row, n, nnz, ctr + 3);
    k_na_degrees<<<grid_for(n), kThreads, 0, s>>>(d_off, n, deg);
    unsigned long long bad = 0;
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
    k_hub_flags<<<grid_for(n), kThreads, 0, s>>>(deg, n, flag);
    NA_CUDA(cudaMemsetAsync(flag + n, 0, sizeof(uint32_t), s));
    NA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, n + 1, s));
    k_hub_ids<<<grid_for(n), kThreads, 0, s>>>(flag, pos, n, hubid);

    DevGraph G;
    G.off = d_off;
    G.adj = d_adj;
    G.deg = deg;
    G.offp = offp;
    G.adjp = adjp;
    G.hubid = hubid;
    G.tslot = tslot;
    G.ev = ev;
    G.eu = eu;
    G.order = order;
    G.n = n;
    G.m = m;
    G.micro = nullptr;
    G.sums = sums;
    k_tslot<<<grid_for(32 * m), kThreads, 0, s>>>(G, tslot);
    k_plan_keys<<<grid_for(m), kThreads, 0, s>>>(G, keys, ctr);
    NA_CUDA(cub::DeviceRadixSort::SortKeys(tmp, tb, keys, keys2, m, 0, 64, s));
    k_keys_pos<<<grid_for(m), kThreads, 0, s>>>(keys2, m, posv);
    unsigned long long nh = 0;
    uint32_t nhubs = 0;
    NA_CUDA(cudaMemcpyAsync(&nh, ctr, sizeof(nh), cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaMemcpyAsync(&nhubs, pos + n, sizeof(nhubs), cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    int64_t nitems = 0;
    if (nh > 0) {
        k_item_flags<<<grid_for(nh), kThreads, 0, s>>>(keys2, (int64_t)nh, iflag);
        NA_CUDA(cudaMemsetAsync(iflag + nh, 0, sizeof(uint32_t), s));
        NA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, iflag, ipos, (int64_t)nh + 1, s));
        uint32_t ni = 0;
        NA_CUDA(cudaMemcpyAsync(&ni, ipos + nh, sizeof(ni), cudaMemcpyDeviceToHost, s));
        NA_CUDA(cudaStreamSynchronize(s));
        nitems = ni;
        k_item_fill<<<grid_for(nh), kThreads, 0, s>>>(iflag, ipos, (int64_t)nh, items);
    }
    if (nitems > 0) {
        const int nh_slots = std::max(1, (int)nhubs);
        NA_CUDA(cudaMemsetAsync(cache, 0xff, (size_t)nsm * nh_slots * sizeof(unsigned long long), s));
        if (!in_smem) NA_CUDA(cudaMemsetAsync(gbm, 0, (size_t)nsm * nwords * 4, s));
        const size_t smem = in_smem ? (size_t)nwords * 4 : 0;
        NA_CUDA(cudaFuncSetAttribute(k_hub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        HubArgs H;
        H.G = G;
        H.hpos = posv;
        H.items = items;
        H.nitems = nitems;
        H.cache = cache;
        H.nhubs = nh_slots;
        H.gbitmap = gbm;
        H.nwords = nwords;
        H.smem_bitmap = in_smem ? 1 : 0;
        H.next = ctr + 1;
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
