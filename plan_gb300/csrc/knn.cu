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
#include <cstdlib>
#include <type_traits>

#include "exact64.cuh"
#include "pipeline.h"
#include "tree_walk.cuh"
#include "knn_f32.cuh"

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


// exact heap path, thread per query; list: the queries to answer (null: all nq)
template <int KMAX, int SPL>
__global__ void __launch_bounds__(128) k_density_at(KTree t, const double *q3, const double *est, const uint32_t *list, uint32_t nq, uint32_t k,
                                                    double four_pi_over_three, SplineCells sc, double *out, unsigned *err) {
    extern __shared__ unsigned char smem[];
    double *sd = reinterpret_cast<double *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sd + KMAX * blockDim.x);
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    if (list) i = list[i];
    SlabHeap h{sd + threadIdx.x, si + threadIdx.x, (int)blockDim.x};
    double qx = q3[3 * i], qy = q3[3 * i + 1], qz = q3[3 * i + 2];
    double r = est[i] != 0 ? est[i] : knn_first_radius(t, qx, qy, qz, 0xffffffffu, k, err);
    int got = knn_query(t, qx, qy, qz, r, k, h, err);
    if (got != (int)k) {
        out[i] = 0.0;
    } else if constexpr (SPL) {
        // the reference passes self_id = 0: offsets are taken from tree point 0 (src/tree.hpp:4889, 4905)
        const double4_32a p0 = t.pos[0];
        out[i] = spline_density(t.pos, [&](int j) { return h.iget(j); }, (int)k, p0.x, p0.y, p0.z, sc);
    } else {
        out[i] = knn_median_density(t, h, (int)k, four_pi_over_three);
    }
}

// Ascending sort of (key, index) pairs [0, n) by one warp (bitonic, in shared memory; the
// entries up to the next power of two are padded, so C, a power of two, bounds n).
template <int C>
__device__ inline void warp_sort_pairs(unsigned long long *key, uint32_t *ix, uint32_t n, int lane) {
    uint32_t P = 1;
    while (P < n) P <<= 1;
    for (uint32_t j = n + lane; j < P; j += 32) {
        key[j] = ~0ull;
        ix[j] = 0xffffffffu;
    }
    __syncwarp();
    for (uint32_t size = 2; size <= P; size <<= 1)
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t u = lane; u < P / 2; u += 32) {
                const uint32_t a = 2 * u - (u & (stride - 1)), b = a + stride;
                const bool up = (a & size) == 0;
                const unsigned long long ka = key[a], kb = key[b];
                const uint32_t ia = ix[a], ib = ix[b];
                const bool gt = ka > kb || (ka == kb && ia > ib);
                if (gt == up) {
                    key[a] = kb;
                    key[b] = ka;
                    ix[a] = ib;
                    ix[b] = ia;
                }
            }
            __syncwarp();
        }
}

// Warp-cooperative form of k_density_at for queries that visit many points (the saddle
// tests of the merge sweeps reach 10^5 points and more): one warp per query walks the tree
// exactly as the reference does (every lane on the same path), the lanes take 32 points of
// a visited range at a time, and every point within the running k-th smallest squared
// distance goes to a per-warp buffer that a warp sort compacts. A squared distance is
// non-negative, so its bits order like its value. With no tie at the k-boundary or inside
// the k-set, the k kept are the reference heap's contents in its sorted order; a query with
// such a tie, or one whose ties overflow the buffer, is listed for the exact heap path.
template <int KM, int SPL>
__global__ void __launch_bounds__(128) k_density_at_w(KTree t, const double *q3, const double *est, uint32_t nq, uint32_t k, double fpo3,
                                                      SplineCells sc, double *out, uint32_t *redo, uint32_t *nredo, unsigned *err) {
    constexpr uint32_t C = 4 * KM;  // candidates per warp
    __shared__ unsigned long long s_key[4][C];
    __shared__ uint32_t s_ix[4][C];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t i = blockIdx.x * 4 + w;
    if (i >= nq) return;
    const unsigned full = 0xffffffffu;
    unsigned long long *key = s_key[w];
    uint32_t *ix = s_ix[w];
    const double qx = q3[3 * i], qy = q3[3 * i + 1], qz = q3[3 * i + 2];
    double r = est[i] != 0 ? est[i] : knn_first_radius(t, qx, qy, qz, 0xffffffffu, k, err);
    r = knn_final_radius(t, qx, qy, qz, r, k, err);
    uint32_t n = 0, visited = 0;     // buffered candidates, points visited (the same in every lane)
    unsigned long long tau = ~0ull;  // the running k-th smallest (bits); a point above it is out
    bool overflow = false;
    auto compact = [&]() {
        warp_sort_pairs<C>(key, ix, n, lane);
        if (n >= k) {
            tau = key[k - 1];
            uint32_t m = k;
            while (m < n && key[m] == tau) ++m;
            n = m;
        }
    };
    traverse(t, qx, qy, qz, r,
             [&](uint32_t b, uint32_t e, bool) {
                 for (uint32_t p0 = b; p0 < e; p0 += 32) {
                     const uint32_t p = p0 + (uint32_t)lane;
                     unsigned long long kb = ~0ull;
                     if (p < e) kb = dbits(point_dr2(qx, qy, qz, t.pos[p]));
                     unsigned m = __ballot_sync(full, p < e && kb <= tau);
                     if (!m) continue;
                     if (n + __popc(m) > C) {
                         compact();
                         m = __ballot_sync(full, p < e && kb <= tau);
                         if (n + __popc(m) > C) {
                             overflow = true;
                             return false;
                         }
                     }
                     if ((m >> lane) & 1u) {
                         const uint32_t at = n + __popc(m & ((1u << lane) - 1u));
                         key[at] = kb;
                         ix[at] = p;
                     }
                     n += __popc(m);
                     __syncwarp();
                 }
                 visited += e - b;
                 return true;
             },
             err);
    bool redo_it = overflow;
    if (!redo_it) {
        compact();
        if (visited < k) {  // fewer points than neighbours: the reference's zero
            if (lane == 0) out[i] = 0.0;
            return;
        }
        bool tie = n > k;  // a point beyond the k-th at the same distance
        for (uint32_t j = 1 + (uint32_t)lane; j < k; j += 32) tie = tie || key[j] == key[j - 1];
        redo_it = __any_sync(full, tie);
    }
    if (redo_it) {
        if (lane == 0) redo[atomicAdd(nredo, 1u)] = i;
        return;
    }
    if (lane == 0) {
        if constexpr (SPL) {
            const double4_32a p0 = t.pos[0];  // self_id = 0, as in the exact path
            out[i] = spline_density(t.pos, [&](int j) { return ix[j]; }, (int)k, p0.x, p0.y, p0.z, sc);
        } else {
            // MedianSphericalDensityKernel on the sorted k-set, as knn_median_density
            int j = (int)k;
            const double m2 = 4 * dfrom(key[j / 2]);
            for (j = j - 1; j >= 0; j--)
                if (!(dfrom(key[j]) > m2)) break;
            const double r2 = dfrom(key[j]);
            double dens = 0;
            for (; j >= 0; j--) dens = dens + t.pos[ix[j]].w;
            out[i] = dens / (fpo3 * cr_pow15(r2));
        }
    }
}

// ---------------------------------------------------------------- FP32-filtered kernels
__global__ void k_split_points(const double4_32a *pos, uint32_t n, float4 *hi, float4 *lo) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a p = pos[i];
    float hx = (float)p.x, hy = (float)p.y, hz = (float)p.z;
    hi[i] = make_float4(hx, hy, hz, 0.f);
    lo[i] = make_float4((float)(p.x - (double)hx), (float)(p.y - (double)hy), (float)(p.z - (double)hz), 0.f);
}

__global__ void k_split_nodes(const double4_32a *ncf, uint32_t n, float4 *hi, float4 *lo) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a c = ncf[i];
    float hx = (float)c.x, hy = (float)c.y, hz = (float)c.z, hw = (float)c.w;
    hi[i] = make_float4(hx, hy, hz, hw);
    lo[i] = make_float4((float)(c.x - (double)hx), (float)(c.y - (double)hy), (float)(c.z - (double)hz), (float)(c.w - (double)hw));
}

__device__ __forceinline__ double f_median_density(const KTree &t, const double *d64, const uint32_t *i64, int k, double fpo3) {
    int i = k;
    double m2 = 4 * d64[i / 2];
    for (i = i - 1; i >= 0; i--) {
        if (d64[i] > m2) continue;
        break;
    }
    double r2 = d64[i];
    double dens = 0;
    for (; i >= 0; i--) dens = dens + t.pos[i64[i]].w;
    return dens / (fpo3 * cr_pow15(r2));
}

template <int CAP, int SPL>
__global__ void __launch_bounds__(128) k_density_f(KTree t, FTree f, uint32_t n, uint32_t k, double fpo3, SplineCells sc, double *dens,
                                                   uint32_t *redo, uint32_t *nredo, unsigned *err) {
    extern __shared__ unsigned char smem[];
    float *sk = reinterpret_cast<float *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sk + CAP * blockDim.x);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < n;  // every lane reaches the reconvergence point below
    FHeap fh{sk + threadIdx.x, si + threadIdx.x, (int)blockDim.x};
    double d64[CAP];
    uint32_t i64[CAP];
    double4_32a q = make_double4_32a(0, 0, 0, 0);
    int z = -1;
    if (act) {
        q = t.pos[i];
        const double r = knn_first_radius(t, q.x, q.y, q.z, t.leaf_of[i], k, err);
        z = knn_collect_f32(t, f, i, r, k, CAP, fh, err);
    }
    __syncwarp();  // the walks diverge; the FP64 part runs with the whole warp
    const int got = z >= 0 ? knn_exact_f32(t, q.x, q.y, q.z, k, z, fh, d64, i64) : -1;
    if (!act) return;
    if (got < 0) {
        redo[atomicAdd(nredo, 1u)] = i;
        return;
    }
    if constexpr (SPL) dens[i] = spline_density(t.pos, [&](int j) { return i64[j]; }, (int)k, q.x, q.y, q.z, sc);
    else dens[i] = f_median_density(t, d64, i64, (int)k, fpo3);
}

template <int CAP>
__global__ void __launch_bounds__(128) k_densest_f(KTree t, FTree f, uint32_t n, uint32_t k, double threshold, const double *dens,
                                                   uint32_t *densest, uint32_t *redo, uint32_t *nredo, unsigned *err) {
    extern __shared__ unsigned char smem[];
    float *sk = reinterpret_cast<float *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sk + CAP * blockDim.x);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < n;  // every lane reaches the reconvergence point below
    const double di = act ? dens[i] : 0.0;
    uint32_t best = i;
    const bool walk = act && di >= threshold;  // src/tree.hpp:3719-3735
    FHeap fh{sk + threadIdx.x, si + threadIdx.x, (int)blockDim.x};
    double d64[CAP];
    uint32_t i64[CAP];
    double4_32a q = make_double4_32a(0, 0, 0, 0);
    int z = -1;
    if (walk) {
        q = t.pos[i];
        const double r = knn_first_radius(t, q.x, q.y, q.z, t.leaf_of[i], k, err);
        z = knn_collect_f32(t, f, i, r, k, CAP, fh, err);
    }
    __syncwarp();  // the walks diverge; the FP64 part runs with the whole warp
    const int got = z >= 0 ? knn_exact_f32(t, q.x, q.y, q.z, k, z, fh, d64, i64) : -1;
    if (!act) return;
    if (walk) {
        if (got < 0) {
            redo[atomicAdd(nredo, 1u)] = i;
            return;
        }
        double bd = di;
        for (int j = 0; j < got; ++j) {
            uint32_t c = i64[j];
            double dc = dens[c];
            if (bd < dc) { best = c; bd = dc; }
            else if (bd == dc && best > c) best = c;
        }
    }
    densest[i] = best;
}

// exact FP64 path for a list of queries
template <int KMAX, int SPL>
__global__ void __launch_bounds__(128) k_density_list(KTree t, const uint32_t *list, uint32_t n, uint32_t k, double fpo3, SplineCells sc,
                                                      double *dens, unsigned *err) {
    extern __shared__ unsigned char smem[];
    double *sd = reinterpret_cast<double *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sd + KMAX * blockDim.x);
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t i = list[j];
    SlabHeap h{sd + threadIdx.x, si + threadIdx.x, (int)blockDim.x};
    double4_32a q = t.pos[i];
    double r = knn_first_radius(t, q.x, q.y, q.z, t.leaf_of[i], k, err);
    int got = knn_query(t, q.x, q.y, q.z, r, k, h, err);
    if (got < (int)k) {
        atomicOr(err, (unsigned)kDevErrCapacity);
        dens[i] = 0;
        return;
    }
    if constexpr (SPL) dens[i] = spline_density(t.pos, [&](int jj) { return h.iget(jj); }, (int)k, q.x, q.y, q.z, sc);
    else dens[i] = knn_median_density(t, h, (int)k, fpo3);
}

template <int KMAX>
__global__ void __launch_bounds__(128) k_densest_list(KTree t, const uint32_t *list, uint32_t n, uint32_t k, double threshold,
                                                      const double *dens, uint32_t *densest, unsigned *err) {
    extern __shared__ unsigned char smem[];
    double *sd = reinterpret_cast<double *>(smem);
    uint32_t *si = reinterpret_cast<uint32_t *>(sd + KMAX * blockDim.x);
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t i = list[j];
    SlabHeap h{sd + threadIdx.x, si + threadIdx.x, (int)blockDim.x};
    double4_32a q = t.pos[i];
    double r = knn_first_radius(t, q.x, q.y, q.z, t.leaf_of[i], k, err);
    int got = knn_query(t, q.x, q.y, q.z, r, k, h, err);
    uint32_t best = i;
    double bd = dens[i];
    for (int jj = 0; jj < got; ++jj) {
        uint32_t c = h.iget(jj);
        double dc = dens[c];
        if (bd < dc) { best = c; bd = dc; }
        else if (bd == dc && best > c) best = c;
    }
    densest[i] = best;
}

template <class F>
int launch_by_k(uint32_t k, F f) {
    if (k <= 32) return f(std::integral_constant<int, 32>(), 128);
    if (k <= 64) return f(std::integral_constant<int, 64>(), 64);
    if (k <= 128) return f(std::integral_constant<int, 128>(), 32);
    return kErrUnsupported;
}

}  // namespace

// FP32 hi/lo copies of points and node centres for the filtered kernels
static int ensure_split(Context &c, cudaStream_t s) {
    DevTree &tr = c.tree;
    if (tr.phi) return kOk;
    tr.phi = c.arena.get<float4>(tr.Tu);
    tr.plo = c.arena.get<float4>(tr.Tu);
    tr.nhi = c.arena.get<float4>(tr.nodes);
    tr.nlo = c.arena.get<float4>(tr.nodes);
    if (c.arena.failed) return kErrOutOfMemory;
    k_split_points<<<grid_for(tr.Tu, 256), 256, 0, s>>>(tr.pos, tr.Tu, tr.phi, tr.plo);
    k_split_nodes<<<grid_for(tr.nodes, 256), 256, 0, s>>>(tr.ncf, tr.nodes, tr.nhi, tr.nlo);
    c.launches += 2;
    PLAN_CUDA(cudaGetLastError());
    return kOk;
}

template <class F>
static int launch_by_cap(uint32_t k, F f) {
    if (k <= 16) return f(std::integral_constant<int, 24>());
    if (k <= 32) return f(std::integral_constant<int, 40>());
    if (k <= 64) return f(std::integral_constant<int, 72>());
    return kErrUnsupported;
}

int launch_density(Context &c, const plan_params &p, uint32_t k, cudaStream_t s) {
    KTree t = ktree_of(c.tree);
    const double fpo3 = 3.14159265358979323846 * 4. / 3.;
    int rc = ensure_split(c, s);
    if (rc) return rc;
    FTree f{c.tree.phi, c.tree.plo, c.tree.nhi, c.tree.nlo};
    const uint32_t n = c.tree.Tu;
    uint32_t *redo = c.scratch.get<uint32_t>(n + 1), *nredo = c.scratch.get<uint32_t>(4);
    if (!redo || !nredo) return kErrOutOfMemory;
    PLAN_CUDA(cudaMemsetAsync(nredo, 0, 4, s));
    const bool spl = !c.fs.median_kernel;
    const SplineCells sc = c.fs.spline;
    rc = launch_by_cap(k, [&](auto capc) {
        constexpr int CAP = decltype(capc)::value;
        size_t sm = (size_t)CAP * 128 * 8;
        auto kern = spl ? k_density_f<CAP, 1> : k_density_f<CAP, 0>;
        if (sm > 48 * 1024) PLAN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PLAN_CUDA(cudaEventRecord(c.kev[0], s));
        kern<<<grid_for(n, 128), 128, sm, s>>>(t, f, n, k, fpo3, sc, c.tree.dens, redo, nredo, c.d_err);
        PLAN_CUDA(cudaEventRecord(c.kev[1], s));
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return (int)kOk;
    });
    if (rc) return rc;
    uint32_t h = 0;
    PLAN_CUDA(cudaMemcpyAsync(&h, nredo, 4, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    float kms = 0;
    cudaEventElapsedTime(&kms, c.kev[0], c.kev[1]);
    c.stage_ms[20] = kms;  // the FP32-filtered density kernel alone
    c.counters[17] = h;
    if (!h) return kOk;
    return launch_by_k(k, [&](auto km, int threads) {
        constexpr int KM = decltype(km)::value;
        size_t sm = (size_t)KM * threads * 12;
        auto kern = spl ? k_density_list<KM, 1> : k_density_list<KM, 0>;
        kern<<<grid_for(h, threads), threads, sm, s>>>(t, redo, h, k, fpo3, sc, c.tree.dens, c.d_err);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return (int)kOk;
    });
}

int launch_densest(Context &c, const plan_params &p, uint32_t k, double threshold, uint32_t *densest, cudaStream_t s) {
    KTree t = ktree_of(c.tree);
    int rc = ensure_split(c, s);
    if (rc) return rc;
    FTree f{c.tree.phi, c.tree.plo, c.tree.nhi, c.tree.nlo};
    const uint32_t n = c.tree.Tu;
    uint32_t *redo = c.scratch.get<uint32_t>(n + 1), *nredo = c.scratch.get<uint32_t>(4);
    if (!redo || !nredo) return kErrOutOfMemory;
    PLAN_CUDA(cudaMemsetAsync(nredo, 0, 4, s));
    rc = launch_by_cap(k, [&](auto capc) {
        constexpr int CAP = decltype(capc)::value;
        size_t sm = (size_t)CAP * 128 * 8;
        if (sm > 48 * 1024) PLAN_CUDA(cudaFuncSetAttribute(k_densest_f<CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PLAN_CUDA(cudaEventRecord(c.kev[0], s));
        k_densest_f<CAP><<<grid_for(n, 128), 128, sm, s>>>(t, f, n, k, threshold, c.tree.dens, densest, redo, nredo, c.d_err);
        PLAN_CUDA(cudaEventRecord(c.kev[1], s));
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return (int)kOk;
    });
    if (rc) return rc;
    uint32_t h = 0;
    PLAN_CUDA(cudaMemcpyAsync(&h, nredo, 4, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    float kms = 0;
    cudaEventElapsedTime(&kms, c.kev[0], c.kev[1]);
    c.stage_ms[21] = kms;  // the FP32-filtered densest-neighbour kernel alone
    c.counters[18] = h;
    if (!h) return kOk;
    return launch_by_k(k, [&](auto km, int threads) {
        constexpr int KM = decltype(km)::value;
        size_t sm = (size_t)KM * threads * 12;
        k_densest_list<KM><<<grid_for(h, threads), threads, sm, s>>>(t, redo, h, k, threshold, c.tree.dens, densest, c.d_err);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return (int)kOk;
    });
}

int launch_density_at(Context &c, const double *d_q3, const double *d_est, uint32_t nq, uint32_t k, double *d_out, cudaStream_t s) {
    if (nq == 0) return kOk;
    KTree t = ktree_of(c.tree);
    const double fpo3 = 3.14159265358979323846 * 4. / 3.;
    const bool spl = !c.fs.median_kernel;
    const size_t mark = c.scratch.used;
    uint32_t *redo = c.scratch.get<uint32_t>(nq + 1), *nredo = c.scratch.get<uint32_t>(4);
    if (!redo || !nredo) {
        c.scratch.used = mark;
        return kErrOutOfMemory;
    }
    PLAN_CUDA(cudaMemsetAsync(nredo, 0, 4, s));
    // a warp per query; the queries with distance ties go to the exact heap path
    int rc = launch_by_k(k, [&](auto km, int) {
        constexpr int KM = decltype(km)::value;
        auto kern = spl ? k_density_at_w<KM, 1> : k_density_at_w<KM, 0>;
        kern<<<(nq + 3) / 4, 128, 0, s>>>(t, d_q3, d_est, nq, k, fpo3, c.fs.spline, d_out, redo, nredo, c.d_err);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return (int)kOk;
    });
    uint32_t h = 0;
    if (!rc) {
        PLAN_CUDA(cudaMemcpyAsync(&h, nredo, 4, cudaMemcpyDeviceToHost, s));
        PLAN_CUDA(cudaStreamSynchronize(s));
        c.counters[27] += h;
    }
    if (!rc && h)
        rc = launch_by_k(k, [&](auto km, int threads) {
            constexpr int KM = decltype(km)::value;
            size_t sm = (size_t)KM * threads * 12;
            auto kern = spl ? k_density_at<KM, 1> : k_density_at<KM, 0>;
            kern<<<grid_for(h, threads), threads, sm, s>>>(t, d_q3, d_est, redo, h, k, fpo3, c.fs.spline, d_out, c.d_err);
            c.launches++;
            PLAN_CUDA(cudaGetLastError());
            return (int)kOk;
        });
    if (h) PLAN_CUDA(cudaStreamSynchronize(s));  // the redo list is scratch, released here
    c.scratch.used = mark;
    return rc;
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
