// --Density_Vs_Scale on the GPU: every (cell centre, radius, sub-centre) query of
// BasicAnalysesWithTree is one thread walking the particle tree with the reference's sheared
// node tests (dvs.cuh, the same code the CPU tests run on the oracle's tree); the largest
// count per radius is an atomic maximum. The host sets up the grid with the reference's own
// arithmetic and turns the counts into densities.
#include <cstring>
#include <string>
#include <vector>

#include "dvs.cuh"
#include "pipeline.h"
#include "tree_walk.cuh"

namespace plan {

namespace {

struct DevTreeView {
    KTree t;
    __device__ void node(uint32_t n, double &x, double &y, double &z, double &hw) const {
        const double4_32a f = t.ncf[n];
        x = f.x;
        y = f.y;
        z = f.z;
        hw = f.w;
    }
    __device__ uint32_t begin(uint32_t n) const { return t.nbeg[n]; }
    __device__ uint32_t end(uint32_t n) const { return t.nend[n]; }
    __device__ uint32_t first(uint32_t n) const { return t.nfd[n]; }
    __device__ uint32_t daughters(uint32_t n) const { return t.nnd[n]; }
    __device__ void point(uint32_t q, double &x, double &y, double &z) const {
        const double4_32a p = t.pos[q];
        x = p.x;
        y = p.y;
        z = p.z;
    }
};

__global__ void k_dvs(DevTreeView tv, const double *xs, const double *ys, const double *zs, DvsGeom g, uint32_t *maxc, unsigned *err) {
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (tid >= (uint64_t)g.nx * g.ny * g.nz * g.nvar) return;
    double x, y, z;
    int lev;
    dvs_query(g, xs, ys, zs, tid, x, y, z, lev);
    bool overflow = false;
    const uint32_t n = dvs_count(tv, x, y, z, g.radius[lev], g.maxd[lev], g, &overflow);
    if (overflow) atomicOr(err, (unsigned)kDevErrCapacity);
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
    // z extent of the tree points (RecursiveFindExtreme finds the extreme values exactly)
    StreamBuf<unsigned long long> d_ext(s);
    PLAN_CUDA(d_ext.alloc(2));
    const unsigned long long init[2] = {~0ull, 0ull};
    PLAN_CUDA(cudaMemcpyAsync(d_ext.p, init, 16, cudaMemcpyHostToDevice, s));
    k_z_extent<<<grid_for(tr.Tu, 256), 256, 0, s>>>(tr.pos, tr.Tu, d_ext.p);
    c.launches++;
    PLAN_CUDA(cudaGetLastError());
    unsigned long long ext[2];
    PLAN_CUDA(cudaMemcpyAsync(ext, d_ext.p, 16, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    DvsParams dp;
    for (int d = 0; d < 3; ++d) {
        dp.box_length[d] = p.box_length[d];
        dp.box_min[d] = p.box_min[d];
        dp.box_max[d] = p.box_max[d];
        dp.box_center[d] = p.box_center[d];
        dp.cell_length[d] = p.cell_length[d];
    }
    dp.box_half_width0 = p.box_half_width[0];
    dp.max_half_width = p.max_half_width;
    dp.shear_speed = p.shear_speed;
    dp.mass_per_particle0 = p.mass_per_particle[0];
    DvsGeom g;
    std::vector<double> xs, ys, zs;
    const int src = dvs_setup(dp, time, key_to_double(ext[0]), key_to_double(ext[1]), g, xs, ys, zs);
    if (src) {
        c.last_error = src == -1   ? "density vs scale: the grid gives more radii than supported"
                       : src == -2 ? "density vs scale: the points or the box need more than 2^24 cell centres along an axis"
                                   : "density vs scale: the grid has more queries than one launch can take";
        return kErrUnsupported;
    }
    std::vector<uint32_t> maxc(g.nlev, 0);
    const uint64_t nthreads = (uint64_t)g.nx * g.ny * g.nz * g.nvar;
    if (nthreads) {
        StreamBuf<double> d_x(s), d_y(s), d_z(s);
        StreamBuf<uint32_t> d_max(s);
        PLAN_CUDA(d_x.alloc(xs.size()));
        PLAN_CUDA(d_y.alloc(ys.size()));
        PLAN_CUDA(d_z.alloc(zs.size()));
        PLAN_CUDA(d_max.alloc(g.nlev));
        PLAN_CUDA(cudaMemcpyAsync(d_x.p, xs.data(), xs.size() * 8, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(d_y.p, ys.data(), ys.size() * 8, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(d_z.p, zs.data(), zs.size() * 8, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemsetAsync(d_max.p, 0, (size_t)g.nlev * 4, s));
        k_dvs<<<(unsigned)((nthreads + 127) / 128), 128, 0, s>>>(DevTreeView{ktree_of(tr)}, d_x.p, d_y.p, d_z.p, g, d_max.p, c.d_err);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        PLAN_CUDA(cudaMemcpyAsync(maxc.data(), d_max.p, (size_t)g.nlev * 4, cudaMemcpyDeviceToHost, s));
        PLAN_CUDA(cudaStreamSynchronize(s));
    }
    radii.assign(g.radius, g.radius + g.nlev);
    rho.resize(g.nlev);
    for (int i = 0; i < g.nlev; ++i) rho[i] = dvs_density(maxc[i], g.radius[i], dp.mass_per_particle0);
    return kOk;
}

}  // namespace plan
