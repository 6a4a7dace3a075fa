// Batched boundness of particle groups: kinetic and pairwise potential energy of every group
// in one pass over all of them.
//
// For a group with centre of mass x_c and velocity v_c,
//   E_kin = 1/2 sum_i m_i |v_c - s (x_c,x - x_i,x) - v_i|^2   (s = (0, q Omega, 0): the shear
//           correction of the reference's boundness test, src/tree.hpp:4657-4659)
//   E_pot = -G sum_{i<j} m_i m_j / |x_i - x_j|                 (no softening, as the reference)
// and the group is bound when E_kin + E_pot < 0.
//
// Kinetic terms and centres are FP64 sums, one block per group. The potential is the O(n^2)
// part: every group is cut into w x w tiles of pairs (the upper triangle, diagonal tiles
// included), w by the group's size class (energy_tiles.h: 32-wide tiles for groups of tens of
// particles, up to 128 or 256 for large ones), and per class a persistent grid of blocks takes
// tiles from one queue across that class's groups, so groups from tens to millions of
// particles share the GPU without a launch per group. A tile stages its w column particles in
// shared memory; each thread sums its row's m_j / r_ij in FP32 with compensated (Neumaier)
// addition and multiplies by its m_i in FP64; the block adds the threads' sums in FP64 into
// the tile's own slot, and one block per group adds its tiles' slots in tile order: the
// result does not depend on which block ran which tile. Coincident pairs (r = 0) are left out
// and counted. The particles arrive as three plain arrays and are packed on the device.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "energy.cuh"
#include "pipeline.h"

namespace plan {

namespace {

__global__ void __launch_bounds__(256) k_group_kinetic(const float4 *pm, const float4 *vel, const uint64_t *off, uint32_t ngroups,
                                                       double shear_y, double *e_kin, double4_32a *com) {
    __shared__ double s[256][7];
    const uint32_t g = blockIdx.x;
    if (g >= ngroups) return;
    const uint64_t b = off[g], e = off[g + 1];
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};  // M, M x, M y, M z, M vx, M vy, M vz
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const float4 p = pm[i], v = vel[i];
        const double m = p.w;
        acc[0] += m;
        acc[1] += m * (double)p.x;
        acc[2] += m * (double)p.y;
        acc[3] += m * (double)p.z;
        acc[4] += m * (double)v.x;
        acc[5] += m * (double)v.y;
        acc[6] += m * (double)v.z;
    }
    for (int k = 0; k < 7; ++k) s[threadIdx.x][k] = acc[k];
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int k = 0; k < 7; ++k) s[threadIdx.x][k] += s[threadIdx.x + h][k];
        __syncthreads();
    }
    const double M = s[0][0];
    // an empty (or massless) group has no centre: zeros, and no kinetic energy below
    const double xc = M > 0.0 ? s[0][1] / M : 0.0, yc = M > 0.0 ? s[0][2] / M : 0.0, zc = M > 0.0 ? s[0][3] / M : 0.0;
    const double vx = M > 0.0 ? s[0][4] / M : 0.0, vy = M > 0.0 ? s[0][5] / M : 0.0, vz = M > 0.0 ? s[0][6] / M : 0.0;
    __syncthreads();
    double ek = 0;
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const float4 p = pm[i], v = vel[i];
        const double dx = vx - (double)v.x;
        const double dy = vy - shear_y * (xc - (double)p.x) - (double)v.y;
        const double dz = vz - (double)v.z;
        ek += 0.5 * (double)p.w * (dx * dx + dy * dy + dz * dz);
    }
    s[threadIdx.x][0] = ek;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) s[threadIdx.x][0] += s[threadIdx.x + h][0];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        e_kin[g] = s[0][0];
        com[g] = make_double4_32a(xc, yc, zc, M);
    }
}

__global__ void k_pack(const float *pos3, const float *vel3, const float *mass, uint64_t n, float4 *pm, float4 *vel) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pm[i] = make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], mass[i]);
    vel[i] = make_float4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.f);
}

// The tiles of one size class: groups glist[0, ng), their queue items item_off (by list
// position); each tile's FP64 sum goes to part[item].
template <int W>
__global__ void __launch_bounds__(W) k_pair_tiles(const float4 *pm, const uint64_t *off, const uint32_t *glist, const uint64_t *item_off,
                                                  uint32_t ng, uint64_t nitems, unsigned long long *next, double *part,
                                                  unsigned long long *zero_pairs) {
    __shared__ PairParticle col[W];
    __shared__ double red[W];
    __shared__ unsigned long long s_item;
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(next, 1ull);
        __syncthreads();
        const uint64_t item = s_item;
        __syncthreads();
        if (item >= nitems) return;
        // the group: last list position k with item_off[k] <= item
        uint32_t lo = 0, hi = ng;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (item_off[mid] <= item) lo = mid;
            else hi = mid;
        }
        const uint32_t g = glist[lo];
        const uint64_t b = off[g], n = off[g + 1] - b;
        const uint64_t T = (n + W - 1) / W;
        uint64_t ti, tj;
        tile_of(item - item_off[lo], T, ti, tj);
        const uint64_t c0 = tj * W, r = ti * W + threadIdx.x;
        if (c0 + threadIdx.x < n) {
            const float4 q = pm[b + c0 + threadIdx.x];
            col[threadIdx.x] = PairParticle{q.x, q.y, q.z, q.w};
        }
        __syncthreads();
        float s = 0.f, comp = 0.f;
        uint32_t zeros = 0;
        double mrow = 0;
        if (r < n) {
            const float4 q = pm[b + r];
            const uint32_t cn = (uint32_t)(n - c0 < (uint64_t)W ? n - c0 : (uint64_t)W);
            pair_row_sum(PairParticle{q.x, q.y, q.z, q.w}, col, cn, ti == tj ? (int)threadIdx.x : -1, s, comp, zeros);
            mrow = q.w;
        }
        red[threadIdx.x] = mrow * ((double)s + (double)comp);
        if (zeros) atomicAdd(zero_pairs, (unsigned long long)zeros);
        __syncthreads();
        for (int h = W / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[item] = red[0];
        __syncthreads();
    }
}

// One block per group: the sum of its tiles' slots part[base, base + count) in a fixed order
// (strided partial sums, then a tree of fixed shape).
__global__ void __launch_bounds__(256) k_group_pot(const double *part, const uint64_t *base, const uint64_t *count, uint32_t ngroups,
                                                   double *sum) {
    __shared__ double red[256];
    const uint32_t g = blockIdx.x;
    if (g >= ngroups) return;
    double a = 0.0;
    for (uint64_t k = threadIdx.x; k < count[g]; k += blockDim.x) a += part[base[g] + k];
    red[threadIdx.x] = a;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) sum[g] = red[0];
}

template <int W>
int launch_tiles(const float4 *pm, const uint64_t *off, const uint32_t *glist, const uint64_t *item_off, uint32_t ng, uint64_t nitems,
                 unsigned long long *next, double *part, unsigned long long *zeros, int sms, cudaStream_t s) {
    const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)sms * (2048 / W), nitems);
    k_pair_tiles<W><<<grid, W, 0, s>>>(pm, off, glist, item_off, ng, nitems, next, part, zeros);
    return cudaGetLastError() == cudaSuccess ? kOk : kErrDevice;
}

}  // namespace

// The tile width of each size class: the measured table, or PLAN_ENERGY_TILES ("w0,w1,w2,w3").
static void energy_tiles(int w[kEnergyClasses]) {
    for (int k = 0; k < kEnergyClasses; ++k) w[k] = kEnergyTile[k];
    const char *e = std::getenv("PLAN_ENERGY_TILES");
    if (!e) return;
    int v[kEnergyClasses], k = 0;
    const char *p = e;
    while (k < kEnergyClasses && *p) {
        char *end = nullptr;
        const long x = std::strtol(p, &end, 10);
        if (end == p || !energy_tile_ok((int)x)) return;
        v[k++] = (int)x;
        p = *end == ',' ? end + 1 : end;
    }
    if (k == kEnergyClasses)
        for (int j = 0; j < kEnergyClasses; ++j) w[j] = v[j];
}

int group_energies(Context &c, const float *pos3, const float *vel3, const float *mass, const uint64_t *offsets, uint32_t ngroups, double G,
                   double shear_y, double *e_kin, double *e_pot, uint64_t *zero_pairs, cudaStream_t s) {
    if (ngroups == 0) return kOk;
    for (uint32_t g = 0; g < ngroups; ++g)
        if (offsets[g + 1] < offsets[g]) return kErrArgument;
    const uint64_t n = offsets[ngroups];
    int w[kEnergyClasses];
    energy_tiles(w);
    // per class: its groups in order, their queue items; per group: where its tiles' slots are
    std::vector<uint32_t> glist[kEnergyClasses];
    for (uint32_t g = 0; g < ngroups; ++g) glist[energy_class(offsets[g + 1] - offsets[g])].push_back(g);
    std::vector<uint64_t> iofs[kEnergyClasses], gbase(ngroups, 0), gcount(ngroups, 0);
    uint64_t cbase[kEnergyClasses + 1] = {0};
    for (int k = 0; k < kEnergyClasses; ++k) {
        iofs[k].assign(glist[k].size() + 1, 0);
        for (size_t j = 0; j < glist[k].size(); ++j) {
            const uint32_t g = glist[k][j];
            const uint64_t T = (offsets[g + 1] - offsets[g] + w[k] - 1) / w[k];
            iofs[k][j + 1] = iofs[k][j] + T * (T + 1) / 2;
            gbase[g] = cbase[k] + iofs[k][j];
            gcount[g] = iofs[k][j + 1] - iofs[k][j];
        }
        cbase[k + 1] = cbase[k] + iofs[k][glist[k].size()];
    }
    const uint64_t nitems = cbase[kEnergyClasses];
    StreamBuf<float> d_p3(s), d_v3(s), d_m(s);
    StreamBuf<float4> d_pm(s), d_v(s);
    StreamBuf<uint64_t> d_off(s), d_items(s), d_gbase(s), d_gcount(s);
    StreamBuf<uint32_t> d_gl(s);
    StreamBuf<double> d_ek(s), d_sum(s), d_part(s);
    StreamBuf<double4_32a> d_com(s);
    StreamBuf<unsigned long long> d_next(s);  // one tile queue per class, then the coincident pairs
    PLAN_CUDA(d_p3.alloc(3 * n + 1));
    PLAN_CUDA(d_v3.alloc(3 * n + 1));
    PLAN_CUDA(d_m.alloc(n + 1));
    PLAN_CUDA(d_pm.alloc(n + 1));
    PLAN_CUDA(d_v.alloc(n + 1));
    PLAN_CUDA(d_off.alloc(ngroups + 1));
    PLAN_CUDA(d_items.alloc(ngroups + kEnergyClasses));
    PLAN_CUDA(d_gl.alloc(ngroups + 1));
    PLAN_CUDA(d_gbase.alloc(ngroups));
    PLAN_CUDA(d_gcount.alloc(ngroups));
    PLAN_CUDA(d_ek.alloc(ngroups));
    PLAN_CUDA(d_sum.alloc(ngroups));
    PLAN_CUDA(d_part.alloc(nitems + 1));
    PLAN_CUDA(d_com.alloc(ngroups));
    PLAN_CUDA(d_next.alloc(kEnergyClasses + 1));
    if (n) {
        PLAN_CUDA(cudaMemcpyAsync(d_p3.p, pos3, 3 * n * 4, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(d_v3.p, vel3, 3 * n * 4, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(d_m.p, mass, n * 4, cudaMemcpyHostToDevice, s));
        k_pack<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_p3.p, d_v3.p, d_m.p, n, d_pm.p, d_v.p);
        c.launches++;
    }
    PLAN_CUDA(cudaMemcpyAsync(d_off.p, offsets, (ngroups + 1) * 8, cudaMemcpyHostToDevice, s));
    std::vector<uint32_t> gl_all;
    std::vector<uint64_t> io_all;
    size_t gl_at[kEnergyClasses], io_at[kEnergyClasses];
    for (int k = 0; k < kEnergyClasses; ++k) {
        gl_at[k] = gl_all.size();
        io_at[k] = io_all.size();
        gl_all.insert(gl_all.end(), glist[k].begin(), glist[k].end());
        io_all.insert(io_all.end(), iofs[k].begin(), iofs[k].end());
    }
    PLAN_CUDA(cudaMemcpyAsync(d_gl.p, gl_all.data(), gl_all.size() * 4, cudaMemcpyHostToDevice, s));
    PLAN_CUDA(cudaMemcpyAsync(d_items.p, io_all.data(), io_all.size() * 8, cudaMemcpyHostToDevice, s));
    PLAN_CUDA(cudaMemcpyAsync(d_gbase.p, gbase.data(), ngroups * 8, cudaMemcpyHostToDevice, s));
    PLAN_CUDA(cudaMemcpyAsync(d_gcount.p, gcount.data(), ngroups * 8, cudaMemcpyHostToDevice, s));
    PLAN_CUDA(cudaMemsetAsync(d_next.p, 0, (kEnergyClasses + 1) * 8, s));
    k_group_kinetic<<<ngroups, 256, 0, s>>>(d_pm.p, d_v.p, d_off.p, ngroups, shear_y, d_ek.p, d_com.p);
    c.launches++;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int k = 0; k < kEnergyClasses; ++k) {
        const uint64_t ni = cbase[k + 1] - cbase[k];
        if (!ni) continue;
        const uint32_t ng = (uint32_t)glist[k].size();
        const uint32_t *gl = d_gl.p + gl_at[k];
        const uint64_t *io = d_items.p + io_at[k];
        double *part = d_part.p + cbase[k];
        int rc = kErrArgument;
        switch (w[k]) {
            case 32: rc = launch_tiles<32>(d_pm.p, d_off.p, gl, io, ng, ni, d_next.p + k, part, d_next.p + kEnergyClasses, sms, s); break;
            case 64: rc = launch_tiles<64>(d_pm.p, d_off.p, gl, io, ng, ni, d_next.p + k, part, d_next.p + kEnergyClasses, sms, s); break;
            case 128: rc = launch_tiles<128>(d_pm.p, d_off.p, gl, io, ng, ni, d_next.p + k, part, d_next.p + kEnergyClasses, sms, s); break;
            case 256: rc = launch_tiles<256>(d_pm.p, d_off.p, gl, io, ng, ni, d_next.p + k, part, d_next.p + kEnergyClasses, sms, s); break;
        }
        if (rc) return rc;
        c.launches++;
    }
    k_group_pot<<<ngroups, 256, 0, s>>>(d_part.p, d_gbase.p, d_gcount.p, ngroups, d_sum.p);
    c.launches++;
    PLAN_CUDA(cudaGetLastError());
    std::vector<double> sum(ngroups);
    unsigned long long zeros = 0;
    PLAN_CUDA(cudaMemcpyAsync(e_kin, d_ek.p, ngroups * 8, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaMemcpyAsync(sum.data(), d_sum.p, ngroups * 8, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaMemcpyAsync(&zeros, d_next.p + kEnergyClasses, 8, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    for (uint32_t g = 0; g < ngroups; ++g) e_pot[g] = -G * sum[g];
    if (zero_pairs) *zero_pairs = zeros;
    return kOk;
}

}  // namespace plan
