// Node tests and the stackless depth-first walk shared by the KNN, ball-search and
// clump-tree kernels (src/tree.hpp:3001-3049, 3086-3102, 3275-3293).
#pragma once

#include "pipeline.h"

namespace plan {

constexpr double kSqrt3 = 1.7320508075688772;  // std::sqrt(3), src/tree.hpp:2538

struct KTree {
    const double4_32a *pos;
    const double4_32a *ncf;
    const uint32_t *nbeg, *nend, *npar, *nfd, *nnd;
    const uint8_t *north;
    const uint32_t *leaf_of;
    TreeBox box;
    uint32_t nodes;
};

inline KTree ktree_of(const DevTree &tr) {
    KTree t;
    t.pos = tr.pos;
    t.ncf = tr.ncf;
    t.nbeg = tr.nbeg;
    t.nend = tr.nend;
    t.npar = tr.npar;
    t.nfd = tr.nfd;
    t.nnd = reinterpret_cast<const uint32_t *>(tr.nnd);
    t.north = tr.north;
    t.leaf_of = tr.leaf_of;
    t.box = tr.box;
    t.nodes = tr.nodes;
    return t;
}

__device__ __forceinline__ bool node_contained(const double4_32a nc, double qx, double qy, double qz, double r) {
    double t = nc.w * kSqrt3;
    double a = fabs(nc.x - qx) + t, b = fabs(nc.y - qy) + t, c = fabs(nc.z - qz) + t;
    double s = a * a;
    s = s + b * b;
    s = s + c * c;
    return s < r * r;
}

__device__ __forceinline__ bool node_intersects(const double4_32a nc, double qx, double qy, double qz, double r) {
    double dx = nc.x - qx, dy = nc.y - qy, dz = nc.z - qz;
    double c2c = dx * dx;
    c2c = c2c + dy * dy;
    c2c = c2c + dz * dz;
    double t = nc.w * kSqrt3 + r;
    if (c2c > t * t) return false;
    if (c2c < r || c2c < nc.w) return true;  // squared distance against r, as the reference
    double q[3] = {qx, qy, qz}, cc[3] = {nc.x, nc.y, nc.z};
    double m2 = 0;
    for (int d = 0; d < 3; ++d) {
        double lo = cc[d] - nc.w, hi = cc[d] + nc.w;
        if (q[d] < lo) m2 = m2 + (q[d] - lo) * (q[d] - lo);
        else if (q[d] > hi) m2 = m2 + (q[d] - hi) * (q[d] - hi);
    }
    return m2 <= r * r;
}

__device__ __forceinline__ double point_dr2(double qx, double qy, double qz, const double4_32a p) {
    double dx = qx - p.x, dy = qy - p.y, dz = qz - p.z;
    double s = dx * dx;
    s = s + dy * dy;
    s = s + dz * dz;
    return s;
}

// visit(begin, end, leaf_partial) for each contained node (leaf_partial = false) or each
// reached leaf that is not contained (leaf_partial = true); return false to stop early.
template <class Visit>
__device__ __forceinline__ bool traverse(const KTree &t, double qx, double qy, double qz, double r, Visit visit, unsigned *err) {
    uint32_t node = 0;
    for (uint32_t guard = 0; guard < 4u * t.nodes + 8u; ++guard) {
        if (node >= t.nodes) {
            atomicOr(err, (unsigned)kDevErrBadNode);
            return false;
        }
        double4_32a nc = t.ncf[node];
        bool down = false;
        if (node_contained(nc, qx, qy, qz, r)) {
            if (!visit(t.nbeg[node], t.nend[node], false)) return false;
        } else if (node_intersects(nc, qx, qy, qz, r)) {
            if (t.nnd[node] == 0) {
                if (!visit(t.nbeg[node], t.nend[node], true)) return false;
            } else {
                down = true;
            }
        }
        if (down) {
            node = t.nfd[node];
            continue;
        }
        while (node != 0) {
            uint32_t p = t.npar[node];
            if (node + 1 < t.nfd[p] + t.nnd[p]) {
                node = node + 1;
                break;
            }
            node = p;
        }
        if (node == 0) return true;
    }
    atomicOr(err, (unsigned)kDevErrLoopLimit);
    return false;
}

// KNN with the reference's semantics (src/tree.hpp:3198-3251, 3473-3491).
// Pos2Node + the parent walk of the first radius (src/tree.hpp:3210-3219, 2968-2997);
// for points outside the root box, the distance to the box (3220-3226).
__device__ inline double knn_first_radius(const KTree &t, double qx, double qy, double qz, uint32_t leaf_hint, uint32_t k, unsigned *err) {
    const TreeBox &b = t.box;
    double q[3] = {qx, qy, qz};
    bool within = true;
    for (int d = 0; d < 3; ++d)
        if (!(q[d] >= b.root_center[d] - b.half_width - b.epsilon && q[d] <= b.root_center[d] + b.half_width + b.epsilon)) within = false;
    double r2 = 0;
    if (within) {
        uint32_t node = leaf_hint;
        if (node == 0xffffffffu) {  // descend by the query's own Morton key
            double s[3];
            uint32_t u[3];
            for (int d = 0; d < 3; ++d) {
                s[d] = q[d] - b.boxmin[d];
                s[d] = s[d] * b.scale[d];
                u[d] = double_to_cell(s[d]);
            }
            node = 0;
            for (int level = 1; level <= 32 && t.nnd[node] != 0; ++level) {
                int sh = 32 - level;  // digit of level L uses bit (32-L) of each coordinate
                int o = ((u[0] >> sh) & 1) | (((u[1] >> sh) & 1) << 1) | (((u[2] >> sh) & 1) << 2);
                uint32_t found = 0xffffffffu;
                for (uint32_t dd = t.nfd[node]; dd < t.nfd[node] + t.nnd[node]; ++dd)
                    if (t.north[dd] == o) { found = dd; break; }
                if (found == 0xffffffffu) {  // the reference reports a missing leaf here
                    atomicOr(err, (unsigned)kDevErrKey2Leaf);
                    break;
                }
                node = found;
            }
        }
        for (int guard = 0; guard < 40 && (t.nend[node] - t.nbeg[node]) < k / 4; ++guard) {
            if (node == 0) break;
            node = t.npar[node];
        }
        double hw = t.ncf[node].w;
        r2 = hw * hw;
    } else {
        for (int d = 0; d < 3; ++d) {
            double dx = fmax(fmax(b.root_center[d] - b.half_width - q[d], 0.0), q[d] - b.root_center[d] - b.half_width);
            r2 = r2 + dx * dx;
        }
    }
    return sqrt(r2);
}

// One KNN query: returns the number of kept neighbours (k unless the tree is smaller) in
// the heap slab, sorted ascending by dr2.
// The radius of the collecting pass: doubled from r until the nodes the sphere contains or
// meets hold at least k points (count-only passes; the reference refills its heap per radius).
__device__ inline double knn_final_radius(const KTree &t, double qx, double qy, double qz, double r, uint32_t k, unsigned *err) {
    for (int it = 0; it < 200; ++it) {
        uint32_t cnt = 0;
        traverse(t, qx, qy, qz, r, [&](uint32_t b, uint32_t e, bool) { cnt += e - b; return cnt < k; }, err);
        if (cnt >= k) break;
        r = r * 2;
        if (it == 199) atomicOr(err, (unsigned)kDevErrLoopLimit);
    }
    return r;
}

__device__ inline int knn_query(const KTree &t, double qx, double qy, double qz, double r, uint32_t k, SlabHeap &h, unsigned *err) {
    r = knn_final_radius(t, qx, qy, qz, r, k, err);
    int size = 0;
    traverse(t, qx, qy, qz, r,
             [&](uint32_t b, uint32_t e, bool) {
                 // eight points loaded together, then added in order: the loads overlap
                 uint32_t p = b;
                 for (; p + 8 <= e; p += 8) {
                     double d[8];
#pragma unroll
                     for (int j = 0; j < 8; ++j) d[j] = point_dr2(qx, qy, qz, t.pos[p + j]);
#pragma unroll
                     for (int j = 0; j < 8; ++j) h.add(size, (int)k, p + j, d[j]);
                 }
                 for (; p < e; ++p) h.add(size, (int)k, p, point_dr2(qx, qy, qz, t.pos[p]));
                 return true;
             },
             err);
    h.sort(size);
    return size;
}

__device__ inline double knn_median_density(const KTree &t, const SlabHeap &h, int k, double four_pi_over_three) {
    // MedianSphericalDensityKernel (src/tree.hpp:3473-3491)
    int i = k;
    double m2 = 4 * h.dget(i / 2);
    for (i = i - 1; i >= 0; i--) {
        if (h.dget(i) > m2) continue;
        break;
    }
    double r2 = h.dget(i);
    double dens = 0;
    for (; i >= 0; i--) dens = dens + t.pos[h.iget(i)].w;
    return dens / (four_pi_over_three * cr_pow15(r2));
}


// Median-kernel density at arbitrary positions with per-query starting radius (0 = the
// reference's own first radius); used for the saddle tests of the merge sweeps.
int launch_density_at(Context &c, const double *d_q3, const double *d_est, uint32_t nq, uint32_t k, double *d_out, cudaStream_t s);

}  // namespace plan
