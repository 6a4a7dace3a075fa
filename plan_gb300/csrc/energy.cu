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
// part: every group is cut into 128 x 128 tiles of pairs (the upper triangle, diagonal tiles
// included) and a persistent grid of blocks takes tiles from one queue across all groups, so
// groups from tens to millions of particles share the GPU without a launch per size. A tile
// stages its 128 column particles in shared memory; each thread sums its row's m_j / r_ij in
// FP32 with compensated (Neumaier) addition and multiplies by its m_i in FP64; the block adds
// the threads' sums in FP64 and one FP64 atomic per tile adds that to the group. Coincident pairs (r = 0) are left out and counted.
#include <algorithm>
#include <cmath>
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

__global__ void __launch_bounds__(kPairTile) k_pair_potential(const float4 *pm, const uint64_t *off, const uint64_t *item_off, uint32_t ngroups,
                                                              uint64_t nitems, unsigned long long *next, double *sum, unsigned long long *zero_pairs) {
    __shared__ PairParticle col[kPairTile];
    __shared__ double red[kPairTile];
    __shared__ unsigned long long s_item;
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(next, 1ull);
        __syncthreads();
        const uint64_t item = s_item;
        __syncthreads();
        if (item >= nitems) return;
        // the group: last g with item_off[g] <= item
        uint32_t lo = 0, hi = ngroups;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (item_off[mid] <= item) lo = mid;
            else hi = mid;
        }
        const uint32_t g = lo;
        const uint64_t b = off[g], n = off[g + 1] - b;
        const uint64_t T = (n + kPairTile - 1) / kPairTile;
        uint64_t ti, tj;
        tile_of(item - item_off[g], T, ti, tj);
        const uint64_t c0 = tj * kPairTile, r = ti * kPairTile + threadIdx.x;
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
            const uint32_t cn = (uint32_t)(n - c0 < (uint64_t)kPairTile ? n - c0 : (uint64_t)kPairTile);
            pair_row_sum(PairParticle{q.x, q.y, q.z, q.w}, col, cn, ti == tj ? (int)threadIdx.x : -1, s, comp, zeros);
            mrow = q.w;
        }
        red[threadIdx.x] = mrow * ((double)s + (double)comp);
        if (zeros) atomicAdd(zero_pairs, (unsigned long long)zeros);
        __syncthreads();
        for (int h = kPairTile / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) atomicAdd(&sum[g], red[0]);
        __syncthreads();
    }
}

}  // namespace

int group_energies(Context &c, const float *pos3, const float *vel3, const float *mass, const uint64_t *offsets, uint32_t ngroups, double G,
                   double shear_y, double *e_kin, double *e_pot, uint64_t *zero_pairs, cudaStream_t s) {
    if (ngroups == 0) return kOk;
    const uint64_t n = offsets[ngroups];
    std::vector<uint64_t> item_off;
    if (pair_items(offsets, ngroups, item_off)) return kErrArgument;
    const uint64_t nitems = item_off[ngroups];
    std::vector<float4> hpm(n), hv(n);
    for (uint64_t i = 0; i < n; ++i) {
        hpm[i] = make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], mass[i]);
        hv[i] = make_float4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.f);
    }
    StreamBuf<float4> d_pm(s), d_v(s);
    StreamBuf<uint64_t> d_off(s), d_items(s);
    StreamBuf<double> d_ek(s), d_sum(s);
    StreamBuf<double4_32a> d_com(s);
    StreamBuf<unsigned long long> d_next(s);  // [0] the tile queue, [1] coincident pairs
    PLAN_CUDA(d_pm.alloc(n));
    PLAN_CUDA(d_v.alloc(n));
    PLAN_CUDA(d_off.alloc(ngroups + 1));
    PLAN_CUDA(d_items.alloc(ngroups + 1));
    PLAN_CUDA(d_ek.alloc(ngroups));
    PLAN_CUDA(d_sum.alloc(ngroups));
    PLAN_CUDA(d_com.alloc(ngroups));
    PLAN_CUDA(d_next.alloc(2));
    PLAN_CUDA(cudaMemcpyAsync(d_pm.p, hpm.data(), n * sizeof(float4), cudaMemcpyHostToDevice, s));
    PLAN_CUDA(cudaMemcpyAsync(d_v.p, hv.data(), n * sizeof(float4), cudaMemcpyHostToDevice, s));
    PLAN_CUDA(cudaMemcpyAsync(d_off.p, offsets, (ngroups + 1) * 8, cudaMemcpyHostToDevice, s));
    PLAN_CUDA(cudaMemcpyAsync(d_items.p, item_off.data(), (ngroups + 1) * 8, cudaMemcpyHostToDevice, s));
    PLAN_CUDA(cudaMemsetAsync(d_sum.p, 0, ngroups * 8, s));
    PLAN_CUDA(cudaMemsetAsync(d_next.p, 0, 16, s));
    k_group_kinetic<<<ngroups, 256, 0, s>>>(d_pm.p, d_v.p, d_off.p, ngroups, shear_y, d_ek.p, d_com.p);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)sms * 8, nitems ? nitems : 1);
    k_pair_potential<<<grid, kPairTile, 0, s>>>(d_pm.p, d_off.p, d_items.p, ngroups, nitems, d_next.p, d_sum.p, d_next.p + 1);
    c.launches += 2;
    PLAN_CUDA(cudaGetLastError());
    std::vector<double> sum(ngroups);
    unsigned long long zeros = 0;
    PLAN_CUDA(cudaMemcpyAsync(e_kin, d_ek.p, ngroups * 8, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaMemcpyAsync(sum.data(), d_sum.p, ngroups * 8, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaMemcpyAsync(&zeros, d_next.p + 1, 8, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    for (uint32_t g = 0; g < ngroups; ++g) e_pot[g] = -G * sum[g];
    if (zero_pairs) *zero_pairs = zeros;
    return kOk;
}

}  // namespace plan
