// closing.cpp -- closing identities of the decomposition, on the host.
//
// Follows graphlet_core.cpp:1449-1472 and compute_4indep (graphlet_core.h:
// 548-557).  The reference is compiled with -ffast-math, under which g++
// lowers x / 3.0 and x / 6.0 to x * (1.0/3.0) and x * (1.0/6.0) (rounded
// reciprocals); x / 2.0 and x / 4.0 are exact scalings either way.  Those
// multiplications are written out here and this file is compiled with
// -ffp-contract=off, so the result is the same on x86-64 and aarch64.
// total_3_indep's n(n-1)(n-2) is a signed 64-bit product in the reference
// (wraps for n > ~2.1M); total_4_indep's is unsigned.
#include "pgd_gb300.h"

extern "C" void pgd_close_counts(const uint64_t s[PGD_NSUMS], int64_t n_, int64_t m_, uint64_t out[PGD_NTOTALS]) {
    typedef unsigned long long ull;
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0;
    const long long n = n_, m = m_;
    const ull sum_t = s[0], sum_star = s[1], sum_disc = s[2], sum_k4 = s[3], sum_c4 = s[4];
    const ull N3 = s[7], N4 = s[8], N5 = s[9], N6 = s[10], N7 = s[11], N8 = s[12], N9 = s[13], N10 = s[14];

    const ull one_edge = (ull)m;
    const ull pairs = (ull)n * (ull)(n - 1);
    const ull two_indep = (ull)((double)(long long)pairs * 0.5 - (double)m);
    const ull tris = (ull)((double)sum_t * third);
    const ull two_star = (ull)((double)sum_star * 0.5);
    const ull three_1edge = sum_disc;
    const long long triples = (long long)((ull)n * (ull)(n - 1) * (ull)(n - 2));
    ull three_indep = (ull)(triples / 6);
    three_indep = three_indep - (tris + two_star + three_1edge);

    const ull clique = (ull)((double)sum_k4 * sixth);
    const ull chord = N3 - 6 * clique;
    const ull cycle = (ull)((double)sum_c4 * 0.25);
    const ull path = N5 - 4 * cycle;
    const ull tailed = (ull)((double)(N4 - 4 * chord) * 0.5);
    const ull star3 = (ull)((double)(N6 - tailed) * third);
    ull edge2 = N7 - 6 * clique - 4 * cycle - 4 * chord - 2 * path - 2 * tailed;
    edge2 = (ull)((double)edge2 * 0.5);
    const ull edge1 = N8 - 2 * edge2;
    const ull star2 = (ull)((double)(N9 - 2 * path) * 0.5);
    const ull tri4 = (ull)((double)(N10 - tailed) * third);
    const ull un = (ull)n;
    ull indep = (un * (un - 1) * (un - 2) * (un - 3)) / 24;
    indep = indep - (clique + chord + cycle + path + tailed + star3);
    indep = indep - (edge2 + edge1 + star2 + tri4);

    out[0] = one_edge;
    out[1] = two_indep;
    out[2] = tris;
    out[3] = two_star;
    out[4] = three_1edge;
    out[5] = three_indep;
    out[6] = clique;
    out[7] = chord;
    out[8] = tailed;
    out[9] = cycle;
    out[10] = star3;
    out[11] = path;
    out[12] = edge2;
    out[13] = edge1;
    out[14] = star2;
    out[15] = tri4;
    out[16] = indep;
}
