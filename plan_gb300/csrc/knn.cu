// KNN density and densest-neighbour search with the reference's exact traversal.
//
// The reference's KNN (KNN_Search_OpenMP, src/tree.hpp:3198-3251) is not an exact k-nearest
// search: it starts from a radius given by the tree (the half width of the smallest
// ancestor of the query's leaf holding >= k/4 points), collects every point of every node
// the sphere contains or intersects (the intersect test keeps the reference's comparison of
// a squared distance against r at src/tree.hpp:3030), doubles the radius until >= k points
// were visited and keeps the k closest visited points in a heap. This kernel reproduces it
// point for point: a count-only traversal per radius (node tests, no per-point work), then
// one collecting traversal at the final radius that feeds a heap with the library's
// sifting order, so ties resolve as in the reference. FP64 throughout, no contraction.
#include <cmath>
#include <type_traits>

#include "pipeline.h"
#include "tree_walk.cuh"

namespace plan {

namespace {

template <int KMAX>
__global__ void __launch_bounds__(128) k_density(KTree t, uint32_t n, uint32_t k, double four_pi_over_three, double *dens, unsigned *err) {
    extern __shared__ unsigned char smem[];
    double *sd = reinterpret_cast<double *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sd + KMAX * blockDim.x);
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    SlabHeap h{sd + threadIdx.x, si + threadIdx.x, (int)blockDim.x};
    double4_32a q = t.pos[i];
    double r = knn_first_radius(t, q.x, q.y, q.z, t.leaf_of[i], k, err);
    int got = knn_query(t, q.x, q.y, q.z, r, k, h, err);
    if (got < (int)k) {
        atomicOr(err, (unsigned)kDevErrCapacity);
        dens[i] = 0;
        return;
    }
    dens[i] = knn_median_density(t, h, (int)k, four_pi_over_three);
}

template <int KMAX>
__global__ void __launch_bounds__(128) k_densest(KTree t, uint32_t n, uint32_t k, double threshold, const double *dens,
                                                 uint32_t *densest, unsigned *err) {
    extern __shared__ unsigned char smem[];
    double *sd = reinterpret_cast<double *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sd + KMAX * blockDim.x);
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double di = dens[i];
    uint32_t best = i;
    if (di >= threshold) {  // src/tree.hpp:3719-3735
        SlabHeap h{sd + threadIdx.x, si + threadIdx.x, (int)blockDim.x};
        double4_32a q = t.pos[i];
        double r = knn_first_radius(t, q.x, q.y, q.z, t.leaf_of[i], k, err);
        int got = knn_query(t, q.x, q.y, q.z, r, k, h, err);
        double bd = di;
        for (int j = 0; j < got; ++j) {
            uint32_t c = h.iget(j);
            double dc = dens[c];
            if (bd < dc) { best = c; bd = dc; }
            else if (bd == dc && best > c) best = c;
        }
    }
    densest[i] = best;
}

template <int KMAX>
__global__ void __launch_bounds__(128) k_knn_positions(KTree t, const double *q3, uint32_t nq, uint32_t k, double est, uint32_t *oidx,
                                                       double *odr2, unsigned *err) {
    extern __shared__ unsigned char smem[];
    double *sd = reinterpret_cast<double *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sd + KMAX * blockDim.x);
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    SlabHeap h{sd + threadIdx.x, si + threadIdx.x, (int)blockDim.x};
    double qx = q3[3 * i], qy = q3[3 * i + 1], qz = q3[3 * i + 2];
    double r = est != 0 ? est : knn_first_radius(t, qx, qy, qz, 0xffffffffu, k, err);
    int got = knn_query(t, qx, qy, qz, r, k, h, err);
    for (int j = 0; j < (int)k; ++j) {
        oidx[(size_t)i * k + j] = j < got ? h.iget(j) : 0xffffffffu;
        odr2[(size_t)i * k + j] = j < got ? h.dget(j) : -1.0;
    }
}


template <int KMAX>
__global__ void __launch_bounds__(128) k_density_at(KTree t, const double *q3, const double *est, uint32_t nq, uint32_t k,
                                                    double four_pi_over_three, double *out, unsigned *err) {
    extern __shared__ unsigned char smem[];
    double *sd = reinterpret_cast<double *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sd + KMAX * blockDim.x);
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    SlabHeap h{sd + threadIdx.x, si + threadIdx.x, (int)blockDim.x};
    double qx = q3[3 * i], qy = q3[3 * i + 1], qz = q3[3 * i + 2];
    double r = est[i] != 0 ? est[i] : knn_first_radius(t, qx, qy, qz, 0xffffffffu, k, err);
    int got = knn_query(t, qx, qy, qz, r, k, h, err);
    out[i] = got == (int)k ? knn_median_density(t, h, (int)k, four_pi_over_three) : 0.0;
}

template <class F>
int launch_by_k(uint32_t k, F f) {
    if (k <= 32) return f(std::integral_constant<int, 32>(), 128);
    if (k <= 64) return f(std::integral_constant<int, 64>(), 64);
    if (k <= 128) return f(std::integral_constant<int, 128>(), 32);
    return kErrUnsupported;
}

}  // namespace

int launch_density(Context &c, const plan_params &p, uint32_t k, cudaStream_t s) {
    KTree t = ktree_of(c.tree);
    const double fpo3 = 3.14159265358979323846 * 4. / 3.;
    return launch_by_k(k, [&](auto km, int threads) {
        constexpr int KM = decltype(km)::value;
        size_t sm = (size_t)KM * threads * 12;
        k_density<KM><<<grid_for(c.tree.Tu, threads), threads, sm, s>>>(t, c.tree.Tu, k, fpo3, c.tree.dens, c.d_err);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return (int)kOk;
    });
}

int launch_densest(Context &c, const plan_params &p, uint32_t k, double threshold, uint32_t *densest, cudaStream_t s) {
    KTree t = ktree_of(c.tree);
    return launch_by_k(k, [&](auto km, int threads) {
        constexpr int KM = decltype(km)::value;
        size_t sm = (size_t)KM * threads * 12;
        k_densest<KM><<<grid_for(c.tree.Tu, threads), threads, sm, s>>>(t, c.tree.Tu, k, threshold, c.tree.dens, densest, c.d_err);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return (int)kOk;
    });
}

int launch_density_at(Context &c, const double *d_q3, const double *d_est, uint32_t nq, uint32_t k, double *d_out, cudaStream_t s) {
    if (nq == 0) return kOk;
    KTree t = ktree_of(c.tree);
    const double fpo3 = 3.14159265358979323846 * 4. / 3.;
    return launch_by_k(k, [&](auto km, int threads) {
        constexpr int KM = decltype(km)::value;
        size_t sm = (size_t)KM * threads * 12;
        k_density_at<KM><<<grid_for(nq, threads), threads, sm, s>>>(t, d_q3, d_est, nq, k, fpo3, d_out, c.d_err);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return (int)kOk;
    });
}

int knn_positions(Context &c, const double *pos3, uint32_t nq, uint32_t k, double est, uint32_t *idx, double *dr2) {
    if (!c.tree.Tu || k == 0 || k > c.tree.Tu) return kErrArgument;
    cudaStream_t s = c.stream;
    double *d_q = nullptr, *d_d = nullptr;
    uint32_t *d_i = nullptr;
    PLAN_CUDA(cudaMallocAsync(&d_q, (size_t)nq * 3 * 8, s));
    PLAN_CUDA(cudaMallocAsync(&d_d, (size_t)nq * k * 8, s));
    PLAN_CUDA(cudaMallocAsync(&d_i, (size_t)nq * k * 4, s));
    PLAN_CUDA(cudaMemcpyAsync(d_q, pos3, (size_t)nq * 3 * 8, cudaMemcpyHostToDevice, s));
    KTree t = ktree_of(c.tree);
    int rc = launch_by_k(k, [&](auto km, int threads) {
        constexpr int KM = decltype(km)::value;
        size_t sm = (size_t)KM * threads * 12;
        k_knn_positions<KM><<<grid_for(nq, threads), threads, sm, s>>>(t, d_q, nq, k, est, d_i, d_d, c.d_err);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return (int)kOk;
    });
    if (rc) return rc;
    PLAN_CUDA(cudaMemcpyAsync(idx, d_i, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaMemcpyAsync(dr2, d_d, (size_t)nq * k * 8, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaFreeAsync(d_q, s));
    PLAN_CUDA(cudaFreeAsync(d_d, s));
    PLAN_CUDA(cudaFreeAsync(d_i, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    return kOk;
}

}  // namespace plan
