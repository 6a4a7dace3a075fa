// Density from a (1D quadratic spline)^3 kernel over the K nearest points, used instead of
// the median-sphere density when a snapshot holds fewer than four particles per horizontal
// grid cell (QseudoQuadraticSplinesKernel and QuadraticSpline, src/tree.hpp:3406-3434).
//
// Each neighbour's mass is spread over one grid cell and weighted by the product of the three
// 1D spline factors of its offset from the query point; the sum runs over the neighbours in
// ascending distance order, as the reference's sorted KNN list gives them. Every operation
// keeps the reference's order, so results are bit-identical. The reference's pow(v, 2.) is
// the square v * v: GCC's optimised builds replace that call by the multiplication.
//
// Host-compilable: the parity tests build these functions on the CPU as well.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define PLAN_HD __host__ __device__
#else
#define PLAN_HD
#endif

namespace plan {

// Grid-cell constants of the spline (src/tree.hpp:2893-2896, src/global.hpp:729-735)
struct SplineCells {
    double half[3];        // cell_length / 2.
    double sq[3];          // cell_length * cell_length
    double three_half[3];  // (cell_length / 2.) * 3.
    double len[3];         // cell_length
    double volume;         // cell_volume
};

inline SplineCells spline_cells(const double cell_length[3], double cell_volume) {
    SplineCells c;
    for (int d = 0; d < 3; ++d) {
        c.len[d] = cell_length[d];
        c.half[d] = cell_length[d] / 2.;
        c.sq[d] = cell_length[d] * cell_length[d];
        c.three_half[d] = c.half[d] * 3.;
    }
    c.volume = cell_volume;
    return c;
}

// QuadraticSpline of the offset (dx, dy, dz)
PLAN_HD inline double spline_weight(double dx, double dy, double dz, const SplineCells &c) {
    const double d[3] = {std::fabs(dx), std::fabs(dy), std::fabs(dz)};
    double w = 1;
    for (int i = 0; i < 3; ++i) {
        if (d[i] <= c.half[i]) {
            w = w * (0.75 - d[i] * d[i] / c.sq[i]);
        } else if (d[i] < c.three_half[i]) {
            const double v = 1.5 - d[i] / c.len[i];
            w = w * (0.5 * (v * v));
        } else {
            return 0.;
        }
    }
    return w;
}

// Sum over the k neighbours idx(0..k-1) of mass / cell_volume * weight, left to right; P has
// x, y, z and the mass in w. (sx, sy, sz) is the point the offsets are taken from: the query
// point for tree points, tree point 0 for the saddle queries of the merge sweeps.
template <class P, class Idx>
PLAN_HD inline double spline_density(const P *pos, Idx idx, int k, double sx, double sy, double sz, const SplineCells &c) {
    double dens = 0;
    for (int i = 0; i < k; ++i) {
        const P p = pos[idx(i)];
        dens = dens + p.w / c.volume * spline_weight(p.x - sx, p.y - sy, p.z - sz, c);
    }
    return dens;
}

}  // namespace plan
