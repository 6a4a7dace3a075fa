// --Density_Vs_Scale: the densest sphere of each radius on the particle tree.
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
//
// Every (centre, radius, sub-centre) query is one thread here, with its own depth-first
// stack, and the maxima are atomics; all node and point tests are the reference's FP64
// expressions in the same order. The centre coordinates are accumulated on the host with
// the reference's additions (x += cell), so every query point has the reference's bits.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pipeline.h"
#include "tree_walk.cuh"

namespace plan {

namespace {

constexpr int kMaxLevels = 24;
constexpr int kStack = 256;

struct DvsGeom {
    double box_length[3], box_min[3], box_max[3];
    double shear;    // shear_speed * time
    double diag;     // sqrt(3) (to_diagonal)
    double radius[kMaxLevels];
    double maxd[kMaxLevels][3];
    double sub1[3], sub2[3];  // half and quarter cell
    int nlev, nsub;           // levels; levels with sub-centres (at most 3)
    uint32_t nx, ny, nz, nvar;
};

// ShearedCenter2Center + the contain / intersect tests + the leaf comparison, depth first
__device__ uint32_t count_sheared(const KTree &t, double cx, double cy, double cz, double r, const double *maxd, const DvsGeom &g,
                                  unsigned *err) {
    uint32_t stack[kStack];
    int top = 0;
    stack[top++] = 0;
    uint32_t count = 0;
    const double c[3] = {cx, cy, cz};
    while (top > 0) {
        const uint32_t node = stack[--top];
        const double4_32a nf = t.ncf[node];
        double nc[3] = {nf.x, nf.y, nf.z}, c2c[3];
        const double hw = nf.w;
        for (int i = 0; i < 3; ++i) {
            c2c[i] = c[i] - nc[i];
            if (fabs(c2c[i]) > maxd[i]) {
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
        const double tmp = hw * g.diag;
        const double t0 = fabs(c2c[0]) + tmp, t1 = fabs(c2c[1]) + tmp, t2 = fabs(c2c[2]) + tmp;
        if (t0 * t0 + t1 * t1 + t2 * t2 < r * r) {
            count += t.nend[node] - t.nbeg[node];
            continue;
        }
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
        const uint32_t nd = t.nnd[node];
        if (nd == 0) {
            for (uint32_t q = t.nbeg[node]; q != t.nend[node]; ++q) {
                const double4_32a p = t.pos[q];
                const double dx = c[0] - p.x, dy = c[1] - p.y, dz = c[2] - p.z;
                if (dx * dx + dy * dy + dz * dz <= r * r) ++count;
            }
        } else {
            if (top + (int)nd > kStack) {  // cannot happen for a 32-level octree; reported, never overrun
                atomicOr(err, (unsigned)kDevErrCapacity);
                return count;
            }
            for (int d = (int)nd - 1; d >= 0; --d) stack[top++] = t.nfd[node] + (uint32_t)d;
        }
    }
    return count;
}

__constant__ int c_orth[8][3] = {{-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {-1, 1, 1}, {1, 1, 1}};

// one thread per (centre, variant): variant v < nlev is the centre at level v; then eight
// sub-centres per level below nsub; then the eight quarter-cell centres of level 0
__global__ void k_dvs(KTree t, const double *xs, const double *ys, const double *zs, DvsGeom g, uint32_t *maxc, unsigned *err) {
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t ncent = (uint64_t)g.nx * g.ny * g.nz;
    if (tid >= ncent * g.nvar) return;
    const uint32_t v = (uint32_t)(tid % g.nvar);
    const uint64_t ci = tid / g.nvar;
    const uint32_t ix = (uint32_t)(ci % g.nx), iy = (uint32_t)((ci / g.nx) % g.ny), iz = (uint32_t)(ci / ((uint64_t)g.nx * g.ny));
    double x = xs[ix], y = ys[iy], z = zs[iz];
    int lev;
    if (v < (uint32_t)g.nlev) {
        lev = (int)v;
    } else if (v < (uint32_t)(g.nlev + 8 * g.nsub)) {
        const int o = (int)(v - g.nlev) % 8;
        lev = (int)(v - g.nlev) / 8;
        x = x + g.sub1[0] * c_orth[o][0];
        y = y + g.sub1[1] * c_orth[o][1];
        z = z + g.sub1[2] * c_orth[o][2];
    } else {
        const int o = (int)(v - g.nlev - 8 * g.nsub);
        lev = 0;
        x = x + g.sub1[0] * c_orth[o][0];
        y = y + g.sub1[1] * c_orth[o][1];
        z = z + g.sub1[2] * c_orth[o][2];
        x = x + g.sub2[0] * c_orth[o][0];
        y = y + g.sub2[1] * c_orth[o][1];
        z = z + g.sub2[2] * c_orth[o][2];
    }
    const uint32_t n = count_sheared(t, x, y, z, g.radius[lev], g.maxd[lev], g, err);
    atomicMax(&maxc[lev], n);
}

__global__ void k_z_extent(const double4_32a *pos, uint32_t n, unsigned long long *ext) {
    // ext[0] = min, ext[1] = max of z, as order-preserving keys of the doubles
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long b = __double_as_longlong(pos[i].z);
    const unsigned long long key = b < 0 ? ~(unsigned long long)b : (unsigned long long)b | 0x8000000000000000ull;
    atomicMin(&ext[0], key);
    atomicMax(&ext[1], key);
}

double key_to_double(unsigned long long key) {
    const unsigned long long b = (key & 0x8000000000000000ull) ? (key & 0x7fffffffffffffffull) : ~key;
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

}  // namespace

int density_vs_scale(Context &c, const plan_params &p, double time, std::vector<double> &radii, std::vector<double> &rho, cudaStream_t s) {
    const DevTree &tr = c.tree;
    if (!tr.Tu || !tr.pos) return kErrArgument;
    DvsGeom g{};
    for (int d = 0; d < 3; ++d) {
        g.box_length[d] = p.box_length[d];
        g.box_min[d] = p.box_min[d];
        g.box_max[d] = p.box_max[d];
        g.sub1[d] = p.cell_length[d] / 2.0;
        g.sub2[d] = p.cell_length[d] / 4.0;
    }
    g.shear = p.shear_speed * time;
    g.diag = std::sqrt(3);
    // z extent of the tree points (RecursiveFindExtreme gives the extreme values exactly)
    unsigned long long *d_ext = nullptr;
    PLAN_CUDA(cudaMallocAsync(&d_ext, 16, s));
    const unsigned long long init[2] = {~0ull, 0ull};
    PLAN_CUDA(cudaMemcpyAsync(d_ext, init, 16, cudaMemcpyHostToDevice, s));
    k_z_extent<<<grid_for(tr.Tu, 256), 256, 0, s>>>(tr.pos, tr.Tu, d_ext);
    c.launches++;
    unsigned long long ext[2];
    PLAN_CUDA(cudaMemcpyAsync(ext, d_ext, 16, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    PLAN_CUDA(cudaFreeAsync(d_ext, s));
    const double zlo = key_to_double(ext[0]), zhi = key_to_double(ext[1]);
    double z_min = p.box_center[2] - p.cell_length[2] / 2.0;
    const double z_max = zhi;
    while (z_min - p.cell_length[2] > zlo) z_min -= p.cell_length[2];
    const int nlev = (int)std::round(std::log10(p.box_half_width[0] * 2 / p.cell_length[0]) / std::log10(2.0)) + 1;
    if (nlev < 1 || nlev > kMaxLevels) {
        c.last_error = "density vs scale: the grid gives " + std::to_string(nlev) + " radii";
        return kErrUnsupported;
    }
    g.nlev = nlev;
    g.nsub = nlev < 3 ? nlev : 3;
    radii.assign(nlev, p.cell_length[0] / 2.0);
    for (int i = 0; i < nlev; ++i) {
        radii[i] *= std::pow(2.0, i);
        g.radius[i] = radii[i];
        for (int d = 0; d < 3; ++d) g.maxd[i][d] = p.box_length[d] - radii[i];
        g.maxd[i][2] = 100 * p.max_half_width;  // no periodic search in z
    }
    g.nvar = (uint32_t)(nlev + 8 * g.nsub + 8);
    // the centres, accumulated as the reference's loops do
    std::vector<double> xs, ys, zs;
    for (double z = z_min; z < z_max; z += p.cell_length[2]) zs.push_back(z);
    for (double y = p.box_min[1] + 0.5 * p.cell_length[1]; y < p.box_max[1]; y += p.cell_length[1]) ys.push_back(y);
    for (double x = p.box_min[0] + 0.5 * p.cell_length[0]; x < p.box_max[0]; x += p.cell_length[0]) xs.push_back(x);
    g.nx = (uint32_t)xs.size();
    g.ny = (uint32_t)ys.size();
    g.nz = (uint32_t)zs.size();
    std::vector<uint32_t> maxc(nlev, 0);
    const uint64_t nthreads = (uint64_t)g.nx * g.ny * g.nz * g.nvar;
    if (nthreads) {
        double *d_x = nullptr, *d_y = nullptr, *d_z = nullptr;
        uint32_t *d_max = nullptr;
        PLAN_CUDA(cudaMallocAsync(&d_x, xs.size() * 8, s));
        PLAN_CUDA(cudaMallocAsync(&d_y, ys.size() * 8, s));
        PLAN_CUDA(cudaMallocAsync(&d_z, zs.size() * 8, s));
        PLAN_CUDA(cudaMallocAsync(&d_max, (size_t)nlev * 4, s));
        PLAN_CUDA(cudaMemcpyAsync(d_x, xs.data(), xs.size() * 8, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(d_y, ys.data(), ys.size() * 8, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(d_z, zs.data(), zs.size() * 8, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemsetAsync(d_max, 0, (size_t)nlev * 4, s));
        k_dvs<<<(unsigned)((nthreads + 127) / 128), 128, 0, s>>>(ktree_of(tr), d_x, d_y, d_z, g, d_max, c.d_err);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        PLAN_CUDA(cudaMemcpyAsync(maxc.data(), d_max, (size_t)nlev * 4, cudaMemcpyDeviceToHost, s));
        PLAN_CUDA(cudaStreamSynchronize(s));
        cudaFreeAsync(d_x, s);
        cudaFreeAsync(d_y, s);
        cudaFreeAsync(d_z, s);
        cudaFreeAsync(d_max, s);
    }
    rho.assign(nlev, 0.0);
    for (int i = 0; i < nlev; ++i) {
        double v = maxc[i];
        v *= (p.mass_per_particle[0] / (4.1887902047863910 * std::pow(radii[i], 3)));
        rho[i] = v;
    }
    return kOk;
}

}  // namespace plan
