// pgd_kernels.cuh -- device helpers shared by the decomposition kernels.
#pragma once

#include <stdint.h>

#include "pgd_gb300.h"

// First index i in [0, len) with a[i] >= x (len if none); a sorted ascending.
__device__ __forceinline__ int pgd_lower_bound(const int32_t *a, int len, int32_t x) {
    int lo = 0, hi = len;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool pgd_contains(const int32_t *a, int len, int32_t x) {
    int i = pgd_lower_bound(a, len, x);
    return i < len && a[i] == x;
}

__device__ __forceinline__ unsigned long long pgd_warp_sum(unsigned long long x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

__device__ __forceinline__ int pgd_warp_incl_scan(int x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// (unsigned long long)(x / 2.0) as the reference computes it: conversion to
// double (round to nearest), scale, truncate.  Below 2^53 the conversion and
// the halving are exact, so the result is x >> 1; only larger x take the
// double path (FP64 is slow on this part, and every edge needs several).
__device__ __forceinline__ unsigned long long pgd_half_d(unsigned long long x) {
    if ((x >> 53) == 0) return x >> 1;
    return __double2ull_rz(__dmul_rn(__ull2double_rn(x), 0.5));
}

// Per-edge closed forms of solve_graphlet_equations (graphlet_core.cpp:
// 1326-1364), added into the 15 partial sums.  Types as in the reference:
// degrees signed 64-bit, t and the sums unsigned 64-bit.
__device__ __forceinline__ void pgd_edge_sums(unsigned long long *s, long long dv, long long du,
                                              unsigned long long t, long long m, long long n) {
    typedef unsigned long long ull;
    ull star = (ull)dv - t - 1;
    star = star + (ull)du - t - 1;
    const ull disc = (ull)n - (star + t) - 2;
    const ull sv = (ull)dv - t - 1, su = (ull)du - t - 1;
    s[0] += t;
    s[1] += star;
    s[2] += disc;
    s[5] += pgd_half_d((t + star) * (t + star - 1));      // N1
    s[6] += pgd_half_d(star * (star - 1));                // N2
    s[7] += pgd_half_d(t * (t - 1));                      // N3
    s[8] += t * star;                                     // N4
    s[9] += sv * su;                                      // N5
    s[10] += (sv * (sv - 1)) / 2 + (su * (su - 1)) / 2;   // N6
    s[11] += (ull)(m - dv - du + 1);                      // N7
    s[12] += pgd_half_d(disc * (disc - 1));               // N8
    s[13] += star * disc;                                 // N9
    s[14] += t * disc;                                    // N10
}

// Column c of the per-edge output row (micro stores graphlet_core.cpp:
// 1559-1575 and the 2-star of the writer, graphlet_core.h:353-355).
__device__ __forceinline__ unsigned long long pgd_micro_col(int c, long long dv, long long du,
                                                           unsigned long long t, unsigned long long k4,
                                                           unsigned long long c4) {
    typedef unsigned long long ull;
    const long long sv = dv - (long long)t - 1, su = du - (long long)t - 1;
    switch (c) {
    case 0: return t;
    case 1: return ((ull)dv - t) + ((ull)du - t) - 2;
    case 2: return k4;
    case 3: {
        // (ull)((double)(t(t-1)) * 0.5 - (double)k4): exact below 2^53
        const ull tt = t * (t - 1);
        if ((tt >> 53) == 0 && (k4 >> 53) == 0) return (tt >> 1) - k4;
        return __double2ull_rz(__dsub_rn(__dmul_rn(__ull2double_rn(tt), 0.5), __ull2double_rn(k4)));
    }
    case 4: return 0;  // local_4_tailed_tris is never written (graphlet_core.cpp:1501)
    case 5: return c4;
    case 6: {
        // (ull)((double)a + (double)(su(su-1)) * 0.5), a = (ull)((double)(sv(sv-1)) * 0.5):
        // exact while every operand and the sum stay below 2^53
        const long long pv = sv * (sv - 1), pu = su * (su - 1);
        const long long lim = 1ll << 53;
        if (pv >= 0 && pv < lim && pu >= 0 && pu < lim) {
            const ull a = (ull)pv >> 1, b = (ull)pu >> 1;
            if (((a + b) >> 53) == 0) return a + b;
        }
        ull a = __double2ull_rz(__dmul_rn(__ll2double_rn(pv), 0.5));
        return __double2ull_rz(__dadd_rn(__ull2double_rn(a), __dmul_rn(__ll2double_rn(pu), 0.5)));
    }
    default: return (ull)(sv * su) - c4;
    }
}
