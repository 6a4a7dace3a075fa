// The arithmetic of --Density_Vs_Scale, host+device (dvs.cu runs it on the GPU; the parity
// tests also compile it for the CPU and run it on the oracle's tree).
//
// BasicAnalysesWithTree (src/analyses.hpp:196-333) counts the tree points within a ball
// around every cell centre of the grid (z from the cell centre at the box centre down past
// the lowest point, up to the highest point), for radii of half a cell times 1, 2, 4, ...
// up to the box, plus eight sub-centres (half a cell off along each orthant) for the three
// smallest radii and one more per orthant (a quarter cell further) for the smallest. Each
// count walks the tree with RecursiveBallSearchCountWithShear (src/tree.hpp:3306-3402): far
// nodes are compared through their shearing-periodic image (x and y faces; the x image moves
// in y by the shear), points in a reached leaf by their plain distance. The largest count per
// radius becomes a density, count * m / (4 pi / 3 r^3).
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#ifdef __CUDACC__
#define PLAN_DVS_HD __host__ __device__
#else
#define PLAN_DVS_HD
#endif

namespace plan {

constexpr int kDvsMaxLevels = 24;
constexpr int kDvsStack = 256;

struct DvsGeom {
    double box_length[3], box_min[3], box_max[3];
    double shear;    // shear_speed * time
    double diag;     // sqrt(3) (to_diagonal)
    double radius[kDvsMaxLevels];
    double maxd[kDvsMaxLevels][3];
    double sub1[3], sub2[3];  // half and quarter cell
    int nlev, nsub;           // levels; levels with sub-centres (at most 3)
    uint32_t nx, ny, nz, nvar;
};

// The parameters the analysis reads (after the first snapshot's box and the run's settings).
struct DvsParams {
    double box_length[3], box_min[3], box_max[3], box_center[3];
    double box_half_width0, max_half_width, cell_length[3], shear_speed, mass_per_particle0;
};

// Geometry and cell-centre coordinates, with the reference's host arithmetic (the centres are
// accumulated x += cell as its loops do). zlo, zhi: extreme z of the tree points. 0; -1 when
// the grid gives more radii than kDvsMaxLevels; -2 when an axis would need more than 2^24
// centres (coordinates far outside any box the parameters describe, where the reference's
// loops would run for ever); -3 when the queries (one device thread each) would need more
// than 2^31 - 1 blocks of 128.
inline int dvs_setup(const DvsParams &p, double time, double zlo, double zhi, DvsGeom &g, std::vector<double> &xs, std::vector<double> &ys,
                     std::vector<double> &zs) {
    g = DvsGeom{};
    for (int d = 0; d < 3; ++d) {
        g.box_length[d] = p.box_length[d];
        g.box_min[d] = p.box_min[d];
        g.box_max[d] = p.box_max[d];
        g.sub1[d] = p.cell_length[d] / 2.0;
        g.sub2[d] = p.cell_length[d] / 4.0;
    }
    g.shear = p.shear_speed * time;
    g.diag = std::sqrt(3);
    const double kMaxCentres = 16777216.0;
    if (!(p.cell_length[0] > 0 && p.cell_length[1] > 0 && p.cell_length[2] > 0)) return -2;
    for (int d = 0; d < 2; ++d)
        if (!((p.box_max[d] - p.box_min[d]) / p.cell_length[d] < kMaxCentres)) return -2;
    if (!((zhi - zlo) / p.cell_length[2] < kMaxCentres) || !(std::fabs(p.box_center[2] - zlo) / p.cell_length[2] < kMaxCentres)) return -2;
    double z_min = p.box_center[2] - p.cell_length[2] / 2.0;
    const double z_max = zhi;
    while (z_min - p.cell_length[2] > zlo) z_min -= p.cell_length[2];
    const int nlev = (int)std::round(std::log10(p.box_half_width0 * 2 / p.cell_length[0]) / std::log10(2.0)) + 1;
    if (nlev < 1 || nlev > kDvsMaxLevels) return -1;
    g.nlev = nlev;
    g.nsub = nlev < 3 ? nlev : 3;
    for (int i = 0; i < nlev; ++i) {
        g.radius[i] = p.cell_length[0] / 2.0;
        g.radius[i] *= std::pow(2.0, i);
        for (int d = 0; d < 3; ++d) g.maxd[i][d] = p.box_length[d] - g.radius[i];
        g.maxd[i][2] = 100 * p.max_half_width;  // no periodic search in z
    }
    g.nvar = (uint32_t)(nlev + 8 * g.nsub + 8);
    xs.clear();
    ys.clear();
    zs.clear();
    for (double z = z_min; z < z_max; z += p.cell_length[2]) zs.push_back(z);
    for (double y = p.box_min[1] + 0.5 * p.cell_length[1]; y < p.box_max[1]; y += p.cell_length[1]) ys.push_back(y);
    for (double x = p.box_min[0] + 0.5 * p.cell_length[0]; x < p.box_max[0]; x += p.cell_length[0]) xs.push_back(x);
    g.nx = (uint32_t)xs.size();
    g.ny = (uint32_t)ys.size();
    g.nz = (uint32_t)zs.size();
    // each axis is below 2^24, so the product is checked in double before it is formed in 64 bits
    if ((double)g.nx * g.ny * g.nz * g.nvar > 2147483647.0 * 128.0) return -3;
    return 0;
}

// Query `tid` of nx ny nz nvar: its point and radius level. Variant v < nlev is the centre at
// level v; then eight sub-centres per level below nsub; then the eight quarter-cell centres
// of level 0 (the reference's inner loop offsets by the outer orthant eight times over,
// src/analyses.hpp:296-305, so it adds one centre per orthant).
PLAN_DVS_HD inline void dvs_query(const DvsGeom &g, const double *xs, const double *ys, const double *zs, uint64_t tid, double &x, double &y,
                                  double &z, int &lev) {
    const int orth[8][3] = {{-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {-1, 1, 1}, {1, 1, 1}};
    const uint32_t v = (uint32_t)(tid % g.nvar);
    const uint64_t ci = tid / g.nvar;
    const uint32_t ix = (uint32_t)(ci % g.nx), iy = (uint32_t)((ci / g.nx) % g.ny), iz = (uint32_t)(ci / ((uint64_t)g.nx * g.ny));
    x = xs[ix];
    y = ys[iy];
    z = zs[iz];
    if (v < (uint32_t)g.nlev) {
        lev = (int)v;
        return;
    }
    int o;
    if (v < (uint32_t)(g.nlev + 8 * g.nsub)) {
        o = (int)(v - g.nlev) % 8;
        lev = (int)(v - g.nlev) / 8;
    } else {
        o = (int)(v - g.nlev - 8 * g.nsub);
        lev = 0;
    }
    x = x + g.sub1[0] * orth[o][0];
    y = y + g.sub1[1] * orth[o][1];
    z = z + g.sub1[2] * orth[o][2];
    if (v >= (uint32_t)(g.nlev + 8 * g.nsub)) {
        x = x + g.sub2[0] * orth[o][0];
        y = y + g.sub2[1] * orth[o][1];
        z = z + g.sub2[2] * orth[o][2];
    }
}

// RecursiveBallSearchCountWithShear from the root, depth first on an explicit stack. Tree
// provides node(n, cx, cy, cz, hw), begin(n), end(n), first(n), daughters(n) and point(q, x,
// y, z). Returns the count; *overflow is set (and the walk stops) if the stack would overrun,
// which a 32-level octree cannot make happen.
template <class Tree>
PLAN_DVS_HD inline uint32_t dvs_count(const Tree &t, double cx, double cy, double cz, double r, const double *maxd, const DvsGeom &g,
                                      bool *overflow) {
    uint32_t stack[kDvsStack];
    int top = 0;
    stack[top++] = 0;
    uint32_t count = 0;
    const double c[3] = {cx, cy, cz};
    while (top > 0) {
        const uint32_t node = stack[--top];
        double nc[3], c2c[3], hw;
        t.node(node, nc[0], nc[1], nc[2], hw);
        // ShearedCenter2Center (src/tree.hpp:3308-3331)
        for (int i = 0; i < 3; ++i) {
            c2c[i] = c[i] - nc[i];
            if (std::fabs(c2c[i]) > maxd[i]) {
                if (c2c[i] > 0) c2c[i] -= g.box_length[i];
                else c2c[i] += g.box_length[i];
                if (i == 0) {
                    if (c[0] < 0) {
                        nc[1] -= g.shear;
                        nc[1] += (double)(int)((g.box_max[1] - nc[1]) / g.box_length[1]) * g.box_length[1];
                    } else {
                        nc[1] += g.shear;
                        nc[1] -= (double)(int)((nc[1] - g.box_min[1]) / g.box_length[1]) * g.box_length[1];
                    }
                }
            }
        }
        // SphereContainNodeWithShear (src/tree.hpp:3335-3346)
        const double tmp = hw * g.diag;
        const double t0 = std::fabs(c2c[0]) + tmp, t1 = std::fabs(c2c[1]) + tmp, t2 = std::fabs(c2c[2]) + tmp;
        if (t0 * t0 + t1 * t1 + t2 * t2 < r * r) {
            count += t.end(node) - t.begin(node);
            continue;
        }
        // SphereNodeIntersectWithShear (src/tree.hpp:3350-3380)
        const double cd = c2c[0] * c2c[0] + c2c[1] * c2c[1] + c2c[2] * c2c[2];
        const double tr = tmp + r;
        if (cd > tr * tr) continue;
        bool hit = cd < r || cd < hw;
        if (!hit) {
            double m2 = 0;
            for (int d = 0; d < 3; ++d) {
                const double lo = (c[d] - c2c[d]) - hw, hi = (c[d] - c2c[d]) + hw;
                if (c[d] < lo) m2 += (c[d] - lo) * (c[d] - lo);
                else if (c[d] > hi) m2 += (c[d] - hi) * (c[d] - hi);
            }
            hit = m2 <= r * r;
        }
        if (!hit) continue;
        const uint32_t nd = t.daughters(node);
        if (nd == 0) {  // the points themselves are compared without the image
            for (uint32_t q = t.begin(node); q != t.end(node); ++q) {
                double px, py, pz;
                t.point(q, px, py, pz);
                const double dx = c[0] - px, dy = c[1] - py, dz = c[2] - pz;
                if (dx * dx + dy * dy + dz * dz <= r * r) ++count;
            }
        } else {
            if (top + (int)nd > kDvsStack) {
                *overflow = true;
                return count;
            }
            for (int d = (int)nd - 1; d >= 0; --d) stack[top++] = t.first(node) + (uint32_t)d;
        }
    }
    return count;
}

// The reported density of each radius from the largest count (src/analyses.hpp:325-328).
inline double dvs_density(uint32_t max_count, double radius, double mass_per_particle0) {
    double v = max_count;
    v *= (mass_per_particle0 / (4.1887902047863910 * std::pow(radius, 3)));
    return v;
}

}  // namespace plan
