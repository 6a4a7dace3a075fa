// The pair-tile arithmetic of the batched boundness pass, host+device (energy.cu runs it on
// the GPU; the CPU tests run the same functions over whole groups against an FP64 sum).
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#ifdef __CUDACC__
#define PLAN_EN_HD __host__ __device__
#else
#define PLAN_EN_HD
#endif

#include "energy_tiles.h"

namespace plan {

constexpr int kPairTile = 128;  // the default tile width (and the widest but one)

// the size class of a group of n particles (host)
inline int energy_class(uint64_t n) {
    for (int k = 0; k < kEnergyClasses - 1; ++k)
        if (n < kEnergyClassBound[k]) return k;
    return kEnergyClasses - 1;
}

// a tile width the pass is built for
inline bool energy_tile_ok(int w) { return w == 32 || w == 64 || w == 128 || w == 256; }

// Tile (ti, tj), tj >= ti, of the upper triangle of a T x T tiling, with tiles numbered row
// by row: row ti starts at ti T - ti (ti - 1) / 2.
PLAN_EN_HD inline uint64_t tri_row_start(uint64_t T, uint64_t k) { return k * T - k * (k - 1) / 2; }

// The tile queue over all groups: item_off[g] is the first queue item of group g, whose
// n_g = offsets[g+1] - offsets[g] particles make T (T + 1) / 2 tiles of the upper triangle
// (T = ceil(n_g / tile)); item_off[ngroups] is the number of items. -1 when the offsets
// decrease.
inline int pair_items(const uint64_t *offsets, uint32_t ngroups, std::vector<uint64_t> &item_off, uint32_t tile = kPairTile) {
    item_off.assign((size_t)ngroups + 1, 0);
    for (uint32_t g = 0; g < ngroups; ++g) {
        if (offsets[g + 1] < offsets[g]) return -1;
        const uint64_t T = (offsets[g + 1] - offsets[g] + tile - 1) / tile;
        item_off[g + 1] = item_off[g] + T * (T + 1) / 2;
    }
    return 0;
}

PLAN_EN_HD inline void tile_of(uint64_t local, uint64_t T, uint64_t &ti, uint64_t &tj) {
    const double a = 2.0 * (double)T + 1.0;
    const double r = std::floor((a - std::sqrt(a * a - 8.0 * (double)local)) / 2.0);
    uint64_t t = r < 0 ? 0 : (uint64_t)r;
    if (t >= T) t = T - 1;
    while (t > 0 && tri_row_start(T, t) > local) --t;
    while (t + 1 < T && tri_row_start(T, t + 1) <= local) ++t;
    ti = t;
    tj = t + (local - tri_row_start(T, t));
}

struct PairParticle {
    float x, y, z, m;
};

// One row particle p against the columns col[0, cn) of its tile: sum of m_q / r in FP32 with
// Neumaier's compensation (the returned pair is sum, compensation); the caller multiplies by
// m_p in FP64, so no pair's mass product is rounded in FP32 (equal masses would otherwise
// round every term the same way). Columns k <= skip_to are left out (a diagonal tile: each
// pair once); coincident pairs are left out and counted. On the GPU 1/r is the hardware
// reciprocal square root (a few units in the last place of FP32, 10^-7 relative per term
// at most, against the stated 10^-6 on the sums); the CPU replay divides by the square root.
PLAN_EN_HD inline void pair_row_sum(const PairParticle &p, const PairParticle *col, uint32_t cn, int skip_to, float &sum, float &comp,
                                    uint32_t &zeros) {
    float s = 0.f, c = 0.f;
    for (uint32_t k = 0; k < cn; ++k) {
        if ((int)k <= skip_to) continue;
        const PairParticle q = col[k];
        const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 == 0.f) {
            ++zeros;
            continue;
        }
#ifdef __CUDA_ARCH__
        const float term = q.m * rsqrtf(d2);  // one special-function op per pair; error well below the tolerance
#else
        const float term = q.m / std::sqrt(d2);
#endif
        const float t = s + term;
        c += std::fabs(s) >= std::fabs(term) ? (s - t) + term : (term - t) + s;
        s = t;
    }
    sum = s;
    comp = c;
}

}  // namespace plan
