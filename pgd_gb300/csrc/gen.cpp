// gen.cpp -- seeded synthetic graph generators (include/pgd_gen.h).
//
// Host code: generation is outside every timed region; it produces the
// input pairs that are then uploaded to the device.  The mixer is the
// SplitMix64 output function (Steele, Lea, Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014), applied to a counter, so
// any draw can be computed independently and in parallel.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "pgd_gen.h"

namespace {

inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

inline double u01(uint64_t seed, uint64_t stream, uint64_t index) {
    uint64_t key = mix64(seed ^ mix64(stream));
    return (double)(mix64(key + index) >> 11) * (1.0 / 9007199254740992.0);
}

constexpr uint64_t kStreamRmat = 0x524d4154ull;   // "RMAT"
constexpr uint64_t kStreamEr = 0x4552ull;         // "ER"
constexpr uint64_t kStreamBa = 0x4241ull;         // "BA"
constexpr uint64_t kStreamRgg = 0x524747ull;      // "RGG"

}  // namespace

extern "C" double pgd_gen_u01(uint64_t seed, uint64_t stream, uint64_t index) { return u01(seed, stream, index); }

extern "C" void pgd_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int32_t *src,
                             int32_t *dst) {
    const int64_t k = (int64_t)edge_factor << scale;
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < k; i++) {
        uint32_t s = 0, d = 0;
        for (int l = 0; l < scale; l++) {
            double r = u01(seed, kStreamRmat, (uint64_t)i * (uint64_t)scale + (uint64_t)l);
            if (r < a) {
            } else if (r < ab) {
                d |= 1u << l;
            } else if (r < abc) {
                s |= 1u << l;
            } else {
                s |= 1u << l;
                d |= 1u << l;
            }
        }
        src[i] = (int32_t)s;
        dst[i] = (int32_t)d;
    }
}

extern "C" int64_t pgd_gen_er(int64_t n, double p, uint64_t seed, int32_t *src, int32_t *dst, int64_t cap) {
    int64_t k = 0;
    for (int64_t i = 0; i < n; i++) {
        for (int64_t j = i + 1; j < n; j++) {
            uint64_t idx = (uint64_t)i * (uint64_t)n + (uint64_t)j;
            if (u01(seed, kStreamEr, idx) < p) {
                if (k < cap) { src[k] = (int32_t)i; dst[k] = (int32_t)j; }
                k++;
            }
        }
    }
    return k;
}

extern "C" int64_t pgd_gen_ba(int64_t n, int m_attach, uint64_t seed, int32_t *src, int32_t *dst, int64_t cap) {
    if (m_attach < 1 || n < 2) return 0;
    int64_t m0 = std::min<int64_t>(m_attach + 1, n);
    std::vector<int32_t> ends;  // every edge endpoint once: degree-proportional sampling
    int64_t k = 0;
    auto emit = [&](int64_t x, int64_t y) {
        if (k < cap) { src[k] = (int32_t)x; dst[k] = (int32_t)y; }
        k++;
        ends.push_back((int32_t)x);
        ends.push_back((int32_t)y);
    };
    for (int64_t i = 0; i < m0; i++)
        for (int64_t j = i + 1; j < m0; j++) emit(i, j);
    std::vector<int32_t> chosen;
    uint64_t draw = 0;
    for (int64_t v = m0; v < n; v++) {
        chosen.clear();
        size_t pool = ends.size();
        while ((int)chosen.size() < m_attach) {
            double r = u01(seed, kStreamBa, draw++);
            int32_t x = ends[(size_t)(r * (double)pool)];
            if (std::find(chosen.begin(), chosen.end(), x) == chosen.end()) chosen.push_back(x);
        }
        for (int32_t x : chosen) emit(v, x);
    }
    return k;
}

extern "C" int64_t pgd_gen_rgg3d(int64_t n, double radius, uint64_t seed, int32_t *src, int32_t *dst, int64_t cap) {
    std::vector<float> xyz((size_t)(3 * n));
    for (int64_t i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) xyz[(size_t)(3 * i + c)] = (float)u01(seed, kStreamRgg, (uint64_t)(3 * i + c));
    int g = std::max(1, (int)floor(1.0 / radius));
    int64_t cells = (int64_t)g * g * g;
    auto cell_of = [&](int64_t i) {
        int cx = std::min(g - 1, (int)(xyz[3 * i] * g));
        int cy = std::min(g - 1, (int)(xyz[3 * i + 1] * g));
        int cz = std::min(g - 1, (int)(xyz[3 * i + 2] * g));
        return ((int64_t)cx * g + cy) * g + cz;
    };
    std::vector<int64_t> start((size_t)cells + 1, 0);
    std::vector<int32_t> members((size_t)n);
    for (int64_t i = 0; i < n; i++) start[(size_t)cell_of(i) + 1]++;
    for (int64_t c = 0; c < cells; c++) start[(size_t)c + 1] += start[(size_t)c];
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t i = 0; i < n; i++) members[(size_t)fill[(size_t)cell_of(i)]++] = (int32_t)i;
    const double r2 = radius * radius;
    // count per point (pairs j > i), then write with a prefix sum: the edge
    // order is a pure function of the inputs
    std::vector<int64_t> cnt((size_t)n + 1, 0);
    auto visit = [&](int64_t i, bool write, int64_t at) {
        int cx = std::min(g - 1, (int)(xyz[3 * i] * g));
        int cy = std::min(g - 1, (int)(xyz[3 * i + 1] * g));
        int cz = std::min(g - 1, (int)(xyz[3 * i + 2] * g));
        int64_t c = 0;
        for (int dx = -1; dx <= 1; dx++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dz = -1; dz <= 1; dz++) {
                    int x = cx + dx, y = cy + dy, z = cz + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= g || y >= g || z >= g) continue;
                    int64_t cell = ((int64_t)x * g + y) * g + z;
                    for (int64_t q = start[(size_t)cell]; q < start[(size_t)cell + 1]; q++) {
                        int64_t j = members[(size_t)q];
                        if (j <= i) continue;
                        double ddx = (double)xyz[3 * i] - xyz[3 * j], ddy = (double)xyz[3 * i + 1] - xyz[3 * j + 1],
                               ddz = (double)xyz[3 * i + 2] - xyz[3 * j + 2];
                        if (ddx * ddx + ddy * ddy + ddz * ddz < r2) {
                            if (write && at + c < cap) { src[at + c] = (int32_t)i; dst[at + c] = (int32_t)j; }
                            c++;
                        }
                    }
                }
        return c;
    };
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; i++) cnt[(size_t)i + 1] = visit(i, false, 0);
    for (int64_t i = 0; i < n; i++) cnt[(size_t)i + 1] += cnt[(size_t)i];
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; i++) visit(i, true, cnt[(size_t)i]);
    return cnt[(size_t)n];
}
