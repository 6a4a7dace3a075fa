// FindPlanetesimals on the device (src/tree.hpp:3576-4339) and the per-clump operations of
// Planetesimal / PlanetesimalList (src/tree.hpp:4351-4909, 5251-5284).
//
// Clumps live in a slot table (structure of arrays). Members live in a pool: each clump
// owns one contiguous segment holding its `indices` order together with the distances of
// its `particles` list (the reference keeps both vectors in the same order outside the
// short windows in which it permutes them). Segments are bump-allocated; merging or
// growing a clump writes a new segment.
//
// Sequential semantics are kept where the reference has them:
//  * sums run in member order (kinematics, dispersion, two-sigma mass, J): the terms of
//    32 members are formed by a warp, then one lane per sum adds them in order;
//  * merge sweeps evaluate every candidate pair in parallel (ball search over a clump tree,
//    boundness, saddle densities by KNN), then one thread resolves predator/prey in key
//    order; predators merge in waves so a predator that is itself eaten later is complete
//    first (the serial order of src/tree.hpp:3976-3980);
//  * unbinding scans members from the outermost inwards with the current state; a chunk of
//    candidates is evaluated in parallel and the highest-index unbound member is removed
//    before the rest is re-evaluated (exact, since only removals change the state);
//  * Hill-sphere rebinding runs all clumps at once under an ordered-claim rule and reruns
//    those that conflicted, which gives the clump-by-clump result in key order; inside a
//    clump the first bound candidate of each chunk is accepted the same way as unbinding.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <vector>

#include "catalogue.h"
#include "hop.h"
#include "lib_sort.cuh"
#include "pipeline.h"
#include "sort.h"
#include "ordered_sum.cuh"
#include "tree_walk.cuh"
#include "knn_f32.cuh"

namespace plan {

namespace {

constexpr uint32_t kNone = 0xffffffffu;
constexpr int kSmallSort = 2048;
constexpr uint32_t kBigKinematics = 4096;  // larger clumps sum with warp_ordered_sum
constexpr int kKinTile = 512;

struct CP {
    double G, shear, Omega;
    double thr, peak_thr, mass_thr;
    double diffuse, hillf;
    uint32_t knn, Tu;
};

struct CT {  // clump table
    uint32_t C;
    uint32_t *key, *peak;
    uint8_t *mask, *alive;
    double *M;
    double4_32a *com, *vcom, *J;
    double *r_in, *r_out, *r10, *r2s, *hill;
    uint32_t *moff, *mn;
    uint32_t *sub_head, *sub_tail;
};

struct Pool {
    uint32_t *idx;
    double *dist;
    uint32_t *top;
    uint32_t cap;
    uint32_t *sub_peak, *sub_next, *sub_top;
    uint32_t sub_cap;
};

__device__ __forceinline__ double norm3(double x, double y, double z) {
    double s = x * x;
    s = s + y * y;
    s = s + z * z;
    return sqrt(s);
}

__device__ __forceinline__ double norm2_3(double x, double y, double z) {
    double s = x * x;
    s = s + y * y;
    s = s + z * z;
    return s;
}

// bump allocation that leaves the pool untouched when it does not fit
__device__ uint32_t pool_try_alloc(const Pool &P, uint32_t n) {
    uint32_t cur = *(volatile uint32_t *)P.top;
    for (int it = 0; it < (1 << 22); ++it) {  // every failed exchange is another block's success
        if ((uint64_t)cur + n > P.cap) return 0xffffffffu;
        const uint32_t prev = atomicCAS(P.top, cur, cur + n);
        if (prev == cur) return cur;
        cur = prev;
    }
    return 0xffffffffu;
}

__device__ uint32_t pool_alloc(const Pool &P, uint32_t n, unsigned *err) {
    uint32_t o = atomicAdd(P.top, n);
    if (o + n > P.cap || o + n < o) {
        atomicOr(err, (unsigned)kDevErrCapacity);
        return kNone;
    }
    return o;
}

// ---------------------------------------------------------------- setup
__global__ void k_init(uint32_t C, const uint32_t *gkey, const uint32_t *goff, CT ct, uint32_t *slot_of_key) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= C) return;
    uint32_t k = gkey[g];
    ct.key[g] = k;
    ct.peak[g] = k;
    ct.mask[g] = 1;
    ct.alive[g] = 1;
    ct.moff[g] = goff[g];
    ct.mn[g] = goff[g + 1] - goff[g];
    ct.sub_head[g] = kNone;
    ct.sub_tail[g] = kNone;
    ct.hill[g] = 0;
    ct.J[g] = make_double4_32a(0, 0, 0, 0);
    slot_of_key[k] = g;
}

// CalculateKinematicProperties (src/tree.hpp:4431-4442), one warp per clump. The products
// m*x, m*v of a tile of 32 members are formed by all lanes at once; lanes 0..6 then each run
// one of the seven running sums strictly in member order, so every sum rounds exactly as
// the reference's loop (on this GPU each dependent FP64 add costs ~63 cycles, which makes
// the add chains, not the products, the limit).
__global__ void __launch_bounds__(128) k_kinematics(const uint32_t *list, uint32_t n, CT ct, Pool P, const double4_32a *pos,
                                                    const double4_32a *vel, int with_hill, double G, double Omega) {
    __shared__ double tile[4][7][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t t = blockIdx.x * 4 + wid;
    if (t >= n) return;
    const uint32_t s = list[t];
    const uint32_t o = ct.moff[s], m = ct.mn[s];
    if (m > kBigKinematics) return;  // k_kinematics_big
    double acc = 0;  // lane c < 7 holds sum c: M, m*x, m*y, m*z, m*vx, m*vy, m*vz
    for (uint32_t base = 0; base < m; base += 32) {
        const uint32_t k = base + lane;
        if (k < m) {
            uint32_t i = P.idx[o + k];
            double4_32a p = pos[i], v = vel[i];
            tile[wid][0][lane] = p.w;
            tile[wid][1][lane] = p.x * p.w;
            tile[wid][2][lane] = p.y * p.w;
            tile[wid][3][lane] = p.z * p.w;
            tile[wid][4][lane] = v.x * p.w;
            tile[wid][5][lane] = v.y * p.w;
            tile[wid][6][lane] = v.z * p.w;
        }
        __syncwarp();
        const uint32_t cnt = min(32u, m - base);
        if (lane < 7)
            for (uint32_t j = 0; j < cnt; ++j) acc = acc + tile[wid][lane][j];
        __syncwarp();
    }
    double M = __shfl_sync(0xffffffffu, acc, 0);
    double cx = __shfl_sync(0xffffffffu, acc, 1), cy = __shfl_sync(0xffffffffu, acc, 2), cz = __shfl_sync(0xffffffffu, acc, 3);
    double vx = __shfl_sync(0xffffffffu, acc, 4), vy = __shfl_sync(0xffffffffu, acc, 5), vz = __shfl_sync(0xffffffffu, acc, 6);
    if (lane == 0) {
        ct.M[s] = M;
        ct.com[s] = make_double4_32a(cx / M, cy / M, cz / M, 0);
        ct.vcom[s] = make_double4_32a(vx / M, vy / M, vz / M, 0);
        if (with_hill) ct.hill[s] = cr_pow_third(M * G / 3. / Omega / Omega);  // src/tree.hpp:4715-4717
    }
}

// The same sums for clumps of more than kBigKinematics members: the block stages the terms
// of kKinTile members in shared memory and warp c runs sum c with warp_ordered_sum.
__global__ void __launch_bounds__(256) k_kinematics_big(const uint32_t *list, CT ct, Pool P, const double4_32a *pos, const double4_32a *vel,
                                                        int with_hill, double G, double Omega) {
    __shared__ double term[7][kKinTile];
    __shared__ double res[7];
    const uint32_t s = list[blockIdx.x];
    const uint32_t o = ct.moff[s], m = ct.mn[s];
    if (m <= kBigKinematics) return;
    const int w = threadIdx.x >> 5;
    double acc = 0.0;
    for (uint32_t base = 0; base < m; base += kKinTile) {
        const uint32_t cnt = min((uint32_t)kKinTile, m - base);
        for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
            const uint32_t id = P.idx[o + base + i];
            const double4_32a p = pos[id], v = vel[id];
            term[0][i] = p.w;
            term[1][i] = p.x * p.w;
            term[2][i] = p.y * p.w;
            term[3][i] = p.z * p.w;
            term[4][i] = v.x * p.w;
            term[5][i] = v.y * p.w;
            term[6][i] = v.z * p.w;
        }
        __syncthreads();
        if (w < 7) acc = warp_ordered_sum(term[w], cnt, acc);
        __syncthreads();
    }
    if (w < 7 && (threadIdx.x & 31) == 0) res[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        const double M = res[0];
        ct.M[s] = M;
        ct.com[s] = make_double4_32a(res[1] / M, res[2] / M, res[3] / M, 0);
        ct.vcom[s] = make_double4_32a(res[4] / M, res[5] / M, res[6] / M, 0);
        if (with_hill) ct.hill[s] = cr_pow_third(M * G / 3. / Omega / Omega);  // src/tree.hpp:4715-4717
    }
}

// distances to the centre of mass (src/tree.hpp:4448-4450, 4545-4547)
__global__ void k_dist(const uint32_t *list, CT ct, Pool P, const double4_32a *pos) {
    uint32_t s = list[blockIdx.x];
    const uint32_t o = ct.moff[s], m = ct.mn[s];
    double4_32a c = ct.com[s];
    // gridDim.y blocks share a clump (large clumps spread their FP64 work over several SMs)
    for (uint32_t k = blockIdx.y * blockDim.x + threadIdx.x; k < m; k += blockDim.x * gridDim.y) {
        double4_32a p = pos[P.idx[o + k]];
        P.dist[o + k] = norm3(p.x - c.x, p.y - c.y, p.z - c.z);
    }
}

// in-block bitonic sort by (distance, previous position) for segments <= kSmallSort
__global__ void __launch_bounds__(1024) k_sort_small(const uint32_t *list, CT ct, Pool P, uint8_t *tie_flag) {
    __shared__ unsigned long long sk[kSmallSort];
    __shared__ uint32_t si[kSmallSort];
    __shared__ uint16_t sp[kSmallSort];
    uint32_t s = list[blockIdx.x];
    const uint32_t o = ct.moff[s], m = ct.mn[s];
    if (threadIdx.x == 0) tie_flag[s] = 0;
    if (m > kSmallSort || m < 2) return;
    uint32_t n2 = 1;
    while (n2 < m) n2 <<= 1;
    for (uint32_t k = threadIdx.x; k < n2; k += blockDim.x) {
        if (k < m) {
            sk[k] = (unsigned long long)__double_as_longlong(P.dist[o + k]);
            si[k] = P.idx[o + k];
            sp[k] = (uint16_t)k;
        } else {
            sk[k] = ~0ull;
            si[k] = kNone;
            sp[k] = 0xffff;
        }
    }
    __syncthreads();
    for (uint32_t size = 2; size <= n2; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t k = threadIdx.x; k < n2; k += blockDim.x) {
                uint32_t j = k ^ stride;
                if (j > k) {
                    bool up = (k & size) == 0;
                    bool gt = sk[k] > sk[j] || (sk[k] == sk[j] && sp[k] > sp[j]);
                    if (gt == up) {
                        unsigned long long tk = sk[k]; sk[k] = sk[j]; sk[j] = tk;
                        uint32_t ti = si[k]; si[k] = si[j]; si[j] = ti;
                        uint16_t tp = sp[k]; sp[k] = sp[j]; sp[j] = tp;
                    }
                }
            }
            __syncthreads();
        }
    }
    // two members at exactly the same distance in a segment longer than the library's
    // insertion-sort threshold: the pool keeps the sequence before the sort for k_lib_order
    int tie = 0;
    if (m > 16)
        for (uint32_t k = threadIdx.x + 1; k < m; k += blockDim.x) tie |= sk[k] == sk[k - 1];
    if (__syncthreads_or(tie)) {
        if (threadIdx.x == 0) tie_flag[s] = 1;
        return;
    }
    for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
        P.idx[o + k] = si[k];
        P.dist[o + k] = __longlong_as_double((long long)sk[k]);
    }
}

// segments whose sort met a tie: the reference's std::sort order (lib_sort.cuh), one thread
// per segment; rare (two members of one clump at exactly the same distance)
__global__ void k_lib_order(const uint32_t *list, uint32_t n, CT ct, Pool P, const uint8_t *tie_flag) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint32_t s = list[t];
    if (!tie_flag[s]) return;
    lib_sort(P.dist + ct.moff[s], P.idx + ct.moff[s], ct.mn[s]);
}

// radii after a sort (src/tree.hpp:4461-4511)
__global__ void k_one10th(const uint32_t *list, CT ct, Pool P, const double4_32a *pos, const double *dens) {
    __shared__ uint32_t s_in, s_out;
    uint32_t s = list[blockIdx.x];
    const uint32_t o = ct.moff[s], m = ct.mn[s];
    if (m == 0) return;
    if (threadIdx.x == 0) { s_in = kNone; s_out = 0; }
    __syncthreads();
    const double tenth = dens[P.idx[o + m / 2]] / 10.;
    for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
        double d = dens[P.idx[o + k]];
        if (d < tenth) atomicMin(&s_in, k);       // first member below a tenth of the median's density
        if (d > tenth) atomicMax(&s_out, k + 1);  // last member above it (stored +1)
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double rin = (s_in != kNone) ? P.dist[o + s_in] : P.dist[o + m - 1];
    double rout = P.dist[o + (s_out ? s_out - 1 : 0)];
    double r10 = (rin + rout) / 2.;
    double tm = 0., tenth_mass = ct.M[s] * (1.0 - 0.95);
    uint32_t r = m;
    for (; r > 0; --r) {
        tm = tm + pos[P.idx[o + r - 1]].w;
        if (tm > tenth_mass) break;
    }
    double r2s = P.dist[o + (r ? r - 1 : 0)];
    if (rin > 0 && rout / rin > 2.5) r10 = (r2s < rout) ? r2s : rout;
    else r10 = (r2s < r10) ? r2s : r10;
    ct.r_in[s] = rin;
    ct.r_out[s] = rout;
    ct.r10[s] = r10;
    ct.r2s[s] = r2s;
}

// IsPositionDispersion2Large (src/tree.hpp:4516-4528): squares formed by the warp, their sum
// taken in order by lane 0
__global__ void __launch_bounds__(128) k_dispersion(const uint32_t *list, uint32_t n, CT ct, Pool P, double tol, uint8_t *too_large) {
    __shared__ double tile[4][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t t = blockIdx.x * 4 + wid;
    if (t >= n) return;
    const uint32_t s = list[t];
    const uint32_t o = ct.moff[s], m = ct.mn[s];
    if (m == 0) {
        if (lane == 0) too_large[t] = 0;
        return;
    }
    double acc = 0.0;
    for (uint32_t base = 0; base < m; base += 32) {
        const uint32_t k = base + lane;
        if (k < m) {
            double d = P.dist[o + k];
            tile[wid][lane] = d * d;
        }
        __syncwarp();
        const uint32_t cnt = min(32u, m - base);
        if (lane == 0)
            for (uint32_t j = 0; j < cnt; ++j) acc = acc + tile[wid][j];
        __syncwarp();
    }
    if (lane == 0) {
        double x = tol * P.dist[o + m - 1];
        too_large[t] = (acc / (double)m > x * x) ? 1 : 0;
    }
}

__global__ void k_hill(const uint32_t *list, uint32_t n, CT ct, double G, double Omega) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    uint32_t s = list[t];
    ct.hill[s] = cr_pow_third(ct.M[s] * G / 3. / Omega / Omega);  // src/tree.hpp:4715-4717
}

// ---------------------------------------------------------------- large segment sort
__global__ void k_large_gather(const uint32_t *list, uint32_t nl, const uint32_t *base, CT ct, Pool P, uint32_t *w0, uint32_t *w1,
                               uint32_t *w2, uint32_t *pay) {
    uint32_t t = blockIdx.x;
    if (t >= nl) return;
    uint32_t s = list[t];
    const uint32_t o = ct.moff[s], m = ct.mn[s], b = base[t];
    for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
        unsigned long long bits = (unsigned long long)__double_as_longlong(P.dist[o + k]);
        w0[b + k] = (uint32_t)bits;
        w1[b + k] = (uint32_t)(bits >> 32);
        w2[b + k] = t;
        pay[b + k] = P.idx[o + k];
    }
}

__global__ void k_large_scatter(const uint32_t *list, uint32_t nl, const uint32_t *base, CT ct, Pool P, const uint32_t *w0,
                                const uint32_t *w1, const uint32_t *pay, uint8_t *tie_flag) {
    uint32_t t = blockIdx.x;
    if (t >= nl) return;
    uint32_t s = list[t];
    const uint32_t o = ct.moff[s], m = ct.mn[s], b = base[t];
    // a tie at equal distances: the unsorted members stay for k_lib_order (as in k_sort_small)
    int tie = 0;
    for (uint32_t k = threadIdx.x + 1; k < m; k += blockDim.x) tie |= w0[b + k] == w0[b + k - 1] && w1[b + k] == w1[b + k - 1];
    if (__syncthreads_or(tie)) {
        if (threadIdx.x == 0) tie_flag[s] = 1;
        return;
    }
    for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
        unsigned long long bits = ((unsigned long long)w1[b + k] << 32) | w0[b + k];
        P.dist[o + k] = __longlong_as_double((long long)bits);
        P.idx[o + k] = pay[b + k];
    }
}

// ---------------------------------------------------------------- merge sweeps
__global__ void k_mark_live(uint32_t C, CT ct, uint32_t *flag) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C) return;
    flag[s] = (ct.alive[s] && ct.mask[s]) ? 1u : 0u;
}

__global__ void k_ct_points(uint32_t C, CT ct, const uint32_t *flag, const uint32_t *rank, double mass0, double4_32a *pos, double4_32a *vel,
                            uint32_t *ct_slot) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C || !flag[s]) return;
    uint32_t k = rank[s];
    double4_32a c = ct.com[s], v = ct.vcom[s];
    pos[k] = make_double4_32a(c.x, c.y, c.z, mass0);
    vel[k] = make_double4_32a(v.x, v.y, v.z, (double)ct.key[s]);  // the clump tree's density field holds the key
    ct_slot[k] = s;
}

__device__ __forceinline__ double merge_radius(const CT &ct, uint32_t s, bool hill_mode, double hillf) {
    return hill_mode ? ct.hill[s] * hillf : ct.r10[s];
}

__global__ void k_max_radius(uint32_t C, CT ct, bool hill_mode, double hillf, double *out) {
    __shared__ double sm[1024];
    double m = 0;
    for (uint32_t s = threadIdx.x; s < C; s += blockDim.x)
        if (ct.alive[s] && ct.mask[s]) { double r = merge_radius(ct, s, hill_mode, hillf); m = (m < r) ? r : m; }
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + st]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0];
}

// BallSearch on the clump tree for every live clump (src/tree.hpp:3898, 4043); pass 0
// counts, pass 1 fills candidate clump-tree indices in traversal order.
__global__ void k_ball_clumps(int pass, uint32_t C, CT ct, KTree t, bool hill_mode, double hillf, double max_radius, uint32_t *cnt,
                              const uint32_t *off, uint32_t *cand, unsigned *err) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C) return;
    if (!(ct.alive[s] && ct.mask[s])) {
        if (pass == 0) cnt[s] = 0;
        return;
    }
    double4_32a c = ct.com[s];
    double r = merge_radius(ct, s, hill_mode, hillf) + max_radius;
    double r2 = r * r;
    uint32_t n = 0, o = pass ? off[s] : 0;
    traverse(t, c.x, c.y, c.z, r,
             [&](uint32_t b, uint32_t e, bool partial) {
                 for (uint32_t q = b; q < e; ++q) {
                     if (partial && !(point_dr2(c.x, c.y, c.z, t.pos[q]) <= r2)) continue;
                     if (pass) cand[o + n] = q;
                     ++n;
                 }
                 return true;
             },
             err);
    if (pass == 0) cnt[s] = n;
}

// Per candidate pair: contained, or intersecting and bound (then the saddle decides).
// code: 0 no, 1 eat, 2 needs saddle test, 3 self, 4 unknown key
__global__ void k_pair_eval(uint32_t ncand, const uint32_t *cand_p1, const uint32_t *cand, const double4_32a *ctvel, CT ct,
                            const uint32_t *slot_of_key, CP cp, bool hill_mode, uint8_t *code, uint32_t *p2_of, double *sq, double *sest,
                            uint32_t *saddle_of, uint32_t *nsaddle) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncand) return;
    uint32_t p1 = cand_p1[k];
    uint32_t key2 = (uint32_t)ctvel[cand[k]].w;
    p2_of[k] = kNone;
    if (key2 == ct.key[p1]) { code[k] = 3; return; }
    uint32_t p2 = key2 < cp.Tu ? slot_of_key[key2] : kNone;
    if (p2 == kNone) { code[k] = 4; return; }
    p2_of[k] = p2;
    double r1 = merge_radius(ct, p1, hill_mode, cp.hillf), r2 = merge_radius(ct, p2, hill_mode, cp.hillf);
    double4_32a c1 = ct.com[p1], c2 = ct.com[p2];
    double dist = norm3(c1.x - c2.x, c1.y - c2.y, c1.z - c2.z);
    uint8_t out = 0;
    if (dist < fmax(r1, r2)) {
        out = 1;
    } else if (dist < (r1 + r2)) {
        // IsGravitationallyBound (src/tree.hpp:4867-4874)
        double M = ct.M[p1] + ct.M[p2];
        double pg = -cp.G / norm3(c1.x - c2.x, c1.y - c2.y, c1.z - c2.z);
        double4_32a v1 = ct.vcom[p1], v2 = ct.vcom[p2];
        double dx = c1.x - c2.x;
        double ex = (v1.x - 0.0 * dx) - v2.x, ey = (v1.y - cp.shear * dx) - v2.y, ez = (v1.z - 0.0 * dx) - v2.z;
        double ek = 0.5 / M * norm2_3(ex, ey, ez);
        if (pg + ek < 0.) {
            // saddle point between the two (src/tree.hpp:4880-4909)
            double ra = hill_mode ? ct.hill[p1] : ct.r10[p1], rb = hill_mode ? ct.hill[p2] : ct.r10[p2];
            double f = ra / (ra + rb);
            uint32_t q = atomicAdd(nsaddle, 1u);
            sq[3 * q] = c1.x + (c2.x - c1.x) * f;
            sq[3 * q + 1] = c1.y + (c2.y - c1.y) * f;
            sq[3 * q + 2] = c1.z + (c2.z - c1.z) * f;
            double est = fmin(ra, rb);
            sest[q] = hill_mode ? est / cp.hillf : est;
            saddle_of[q] = k;
            out = 2;
        }
    }
    code[k] = out;
}

__global__ void k_saddle_apply(uint32_t ns, const uint32_t *saddle_of, const double *sdens, double limit, uint8_t *code) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ns) return;
    // merge when the saddle is NOT deep: density >= 2.5 rho_thr
    code[saddle_of[q]] = (sdens[q] < limit) ? 0 : 1;
}

// candidate -> its predator's slot
__global__ void k_cand_owner(uint32_t C, const uint32_t *cnt, const uint32_t *off, uint32_t *cp1) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C) return;
    const uint32_t o = off[s], n = cnt[s];
    for (uint32_t k = 0; k < n; ++k) cp1[o + k] = s;
}

// the candidates the resolution acts on: eat (code 1) or unknown key (code 4)
__global__ void k_flag_resolve(uint32_t ncand, const uint8_t *code, uint32_t *flag) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncand) return;
    flag[k] = (code[k] == 1 || code[k] == 4) ? 1u : 0u;
}

__global__ void k_scatter_flagged(uint32_t n, const uint32_t *flag, const uint32_t *pos, uint32_t *list) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && flag[k]) list[pos[k]] = k;
}

// Serial predator/prey resolution in key order (src/tree.hpp:3894-3951) over the listed
// candidates in candidate order (slots in key order, each slot's candidates in ball order);
// the candidates left out (self, not bound, deep saddle) change nothing there. One warp:
// the lanes fetch 32 candidates with what does not change during the walk (predator,
// prey, code, whether the predator is alive, the prey's key), then the warp walks them in
// order, reading and clearing the masks.
__global__ void k_resolve(const uint32_t *list, const uint32_t *nlist, const uint32_t *cp1, CT ct, const uint8_t *code,
                          const uint32_t *p2_of, uint32_t *pairs, uint32_t *npairs, uint32_t *del_keys, uint32_t *ndel, uint32_t *nunknown) {
    const int lane = threadIdx.x;
    if (blockIdx.x || lane >= 32) return;
    const unsigned full = 0xffffffffu;
    uint32_t np = 0, nd = *ndel, nu = 0;
    const uint32_t n = *nlist;
    for (uint32_t base = 0; base < n; base += 32) {
        uint32_t p1 = 0, p2 = 0, key2 = 0, cd = 0, al = 0;
        if (base + lane < n) {
            const uint32_t k = list[base + lane];
            p1 = cp1[k];
            cd = code[k];
            al = ct.alive[p1] ? 1u : 0u;
            if (cd == 1) {
                p2 = p2_of[k];
                key2 = ct.key[p2];
            }
        }
        const uint32_t cnt = min(32u, n - base);
        for (uint32_t j = 0; j < cnt; ++j) {
            const uint32_t q1 = __shfl_sync(full, p1, j), q2 = __shfl_sync(full, p2, j), kk = __shfl_sync(full, key2, j);
            const uint32_t c = __shfl_sync(full, cd, j), a = __shfl_sync(full, al, j);
            if (!(a && ct.mask[q1])) continue;
            if (c == 4) {
                ++nu;
                continue;
            }
            if (!ct.mask[q2]) continue;
            if (lane == 0) {
                ct.mask[q2] = 0;
                pairs[2 * np] = q1;
                pairs[2 * np + 1] = q2;
                del_keys[nd] = kk;
            }
            ++np;
            ++nd;
            __syncwarp();  // the cleared mask is seen by the whole warp from here on
        }
    }
    if (lane == 0) {
        *npairs = np;
        *ndel = nd;
        *nunknown += nu;
    }
}

// Waves of predators: a predator that eats an earlier predator waits for it.
__global__ void k_waves(uint32_t np, const uint32_t *pairs, uint32_t C, uint32_t *wave_of_slot, uint32_t *pred_list, uint32_t *pred_first,
                        uint32_t *pred_count, uint32_t *pred_wave, uint32_t *npred, uint32_t *nwaves) {
    if (threadIdx.x || blockIdx.x) return;
    uint32_t n = 0, maxw = 0;
    for (uint32_t k = 0; k < np;) {
        uint32_t p = pairs[2 * k];
        uint32_t first = k, w = 0;
        while (k < np && pairs[2 * k] == p) {
            uint32_t prey = pairs[2 * k + 1];
            if (wave_of_slot[prey] != kNone) w = max(w, wave_of_slot[prey] + 1);
            ++k;
        }
        wave_of_slot[p] = w;
        pred_list[n] = p;
        pred_first[n] = first;
        pred_count[n] = k - first;
        pred_wave[n] = w;
        maxw = max(maxw, w);
        ++n;
    }
    *npred = n;
    *nwaves = np ? maxw + 1 : 0;
}

// MergeAnotherPlanetesimal for every predator of one wave (src/tree.hpp:4532-4611): the
// scalar chain on thread 0, the members copied into a fresh segment (predator first, then
// each prey in order); distances, sort and radii follow for the merged clumps.
__global__ void k_merge(uint32_t npred, const uint32_t *pred_list, const uint32_t *pred_first, const uint32_t *pred_count,
                        const uint32_t *pred_wave, uint32_t wave, const uint32_t *pairs, CT ct, Pool P, const double *dens, uint32_t *merged,
                        uint32_t *nmerged, unsigned *err) {
    __shared__ uint32_t s_off, s_tot, s_ok;
    uint32_t t = blockIdx.x;
    if (t >= npred || pred_wave[t] != wave) return;
    uint32_t a = pred_list[t];
    if (threadIdx.x == 0) {
        double M = ct.M[a];
        double4_32a c = ct.com[a], v = ct.vcom[a];
        uint32_t peak = ct.peak[a], tot = ct.mn[a];
        s_ok = 1;
        for (uint32_t k = pred_first[t]; k < pred_first[t] + pred_count[t]; ++k) {
            uint32_t b = pairs[2 * k + 1];
            uint32_t sub;
            if (dens[peak] < dens[ct.peak[b]]) {
                sub = peak;
                peak = ct.peak[b];
            } else {
                sub = ct.peak[b];
            }
            uint32_t e = atomicAdd(P.sub_top, 1u);
            if (e < P.sub_cap) {
                P.sub_peak[e] = sub;
                P.sub_next[e] = kNone;
                if (ct.sub_tail[a] == kNone) ct.sub_head[a] = e;
                else P.sub_next[ct.sub_tail[a]] = e;
                ct.sub_tail[a] = e;
            } else {
                atomicOr(err, (unsigned)kDevErrCapacity);
            }
            double Mb = ct.M[b];
            double4_32a cb = ct.com[b], vb = ct.vcom[b];
            double Mt = M + Mb;
            c = make_double4_32a((c.x * M + cb.x * Mb) / Mt, (c.y * M + cb.y * Mb) / Mt, (c.z * M + cb.z * Mb) / Mt, 0);
            v = make_double4_32a((v.x * M + vb.x * Mb) / Mt, (v.y * M + vb.y * Mb) / Mt, (v.z * M + vb.z * Mb) / Mt, 0);
            M = Mt;
            tot += ct.mn[b];
        }
        ct.M[a] = M;
        ct.com[a] = c;
        ct.vcom[a] = v;
        ct.peak[a] = peak;
        uint32_t o = pool_alloc(P, tot, err);
        if (o == kNone) s_ok = 0;
        s_off = o;
        s_tot = tot;
    }
    __syncthreads();
    if (!s_ok) return;
    uint32_t at = s_off;
    // predator first, then preys in order
    {
        const uint32_t o = ct.moff[a], m = ct.mn[a];
        for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) P.idx[at + k] = P.idx[o + k];
        at += m;
    }
    for (uint32_t k = pred_first[t]; k < pred_first[t] + pred_count[t]; ++k) {
        uint32_t b = pairs[2 * k + 1];
        const uint32_t o = ct.moff[b], m = ct.mn[b];
        for (uint32_t j = threadIdx.x; j < m; j += blockDim.x) P.idx[at + j] = P.idx[o + j];
        at += m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        ct.moff[a] = s_off;
        ct.mn[a] = s_tot;
        merged[atomicAdd(nmerged, 1u)] = a;
    }
}

// Re-key every clump to its densest sub-peak in key order (src/tree.hpp:4156-4182).
__global__ void k_rekey(uint32_t C, CT ct, const uint32_t *order, uint32_t n, Pool P, const double *dens, uint32_t *slot_of_key,
                        uint32_t *nfail) {
    if (threadIdx.x || blockIdx.x) return;
    // decisions first (all against the keys before re-keying), then the re-insertions
    uint32_t fails = 0;
    for (uint32_t r = 0; r < n; ++r) {
        uint32_t s = order[r];
        uint32_t best = ct.key[s];
        for (uint32_t e = ct.sub_head[s]; e != kNone; e = P.sub_next[e])
            if (dens[best] < dens[P.sub_peak[e]]) best = P.sub_peak[e];
        ct.peak[s] = best;  // staged in peak; applied below
    }
    for (uint32_t r = 0; r < n; ++r) {
        uint32_t s = order[r];
        uint32_t nk = ct.peak[s], ok = ct.key[s];
        if (nk == ok) continue;
        if (slot_of_key[nk] != kNone) { ++fails; ct.peak[s] = ok; continue; }  // emplace fails: keep the old key
        slot_of_key[ok] = kNone;
        slot_of_key[nk] = s;
        ct.key[s] = nk;
    }
    *nfail += fails;
}

// RN(num / den) given y = RN(1 / den): q0 = RN(num y), then Markstein's correction
// RN(q0 + (num - q0 den) y) with two FMAs is the correctly rounded quotient (the identity
// tests/test_div_host.py checks against IEEE division); a zero numerator is returned as it
// is, which is the quotient for den > 0. Several quotients by one divisor then cost one
// reciprocal and two FMAs each instead of a division each.
__device__ __forceinline__ double div_by_rcp(double num, double den, double y) {
    if (num == 0.0) return num;
    const double q0 = num * y;
    return fma(fma(-q0, den, num), y, q0);
}

// RemoveUnboundParticles (src/tree.hpp:4615-4674) for a list of clumps, one block each. The
// six quotients by the remaining mass share one correctly rounded reciprocal (div_by_rcp).
__global__ void __launch_bounds__(256) k_unbind(const uint32_t *list, CT ct, Pool P, const double4_32a *pos, const double4_32a *vel, CP cp) {
    __shared__ double sM, scx, scy, scz, svx, svy, svz;
    __shared__ int s_best;
    __shared__ uint32_t s_back;
    uint32_t s = list[blockIdx.x];
    const uint32_t o = ct.moff[s];
    if (threadIdx.x == 0) {
        sM = ct.M[s];
        double4_32a c = ct.com[s], v = ct.vcom[s];
        scx = c.x; scy = c.y; scz = c.z;
        svx = v.x; svy = v.y; svz = v.z;
        s_back = ct.mn[s] - 1;
    }
    __syncthreads();
    int i = (int)ct.mn[s] - 1;
    while (i >= 1) {
        int lo = max(1, i - (int)blockDim.x + 1);
        if (threadIdx.x == 0) s_best = -1;
        __syncthreads();
        int j = i - (int)threadIdx.x;
        bool unbound = false;
        double Mr = 0;
        if (j >= lo) {
            uint32_t pi = P.idx[o + j];
            double4_32a p = pos[pi], v = vel[pi];
            double M = sM;
            Mr = M - p.w;  // > 0: at least two members remain
            const double y = __drcp_rn(Mr);
            double cx = div_by_rcp(scx * M - p.x * p.w, Mr, y), cy = div_by_rcp(scy * M - p.y * p.w, Mr, y),
                   cz = div_by_rcp(scz * M - p.z * p.w, Mr, y);
            double vx = div_by_rcp(svx * M - v.x * p.w, Mr, y), vy = div_by_rcp(svy * M - v.y * p.w, Mr, y),
                   vz = div_by_rcp(svz * M - v.z * p.w, Mr, y);
            double dx = cx - p.x;
            double ex = (vx - 0.0 * dx) - v.x, ey = (vy - cp.shear * dx) - v.y, ez = (vz - 0.0 * dx) - v.z;
            double e = +0.5 / M * norm2_3(ex, ey, ez) - cp.G / norm3(cx - p.x, cy - p.y, cz - p.z);
            unbound = e > 0;
        }
        if (unbound) atomicMax(&s_best, j);
        __syncthreads();
        int b = s_best;
        if (b < 0) {
            i = lo - 1;
            __syncthreads();
            continue;
        }
        if ((int)threadIdx.x == i - b) {  // the thread that evaluated b updates the state
            uint32_t pi = P.idx[o + b];
            double4_32a p = pos[pi], v = vel[pi];
            double M = sM;
            double Mr2 = M - p.w;
            const double y2 = __drcp_rn(Mr2);
            scx = div_by_rcp(scx * M - p.x * p.w, Mr2, y2); scy = div_by_rcp(scy * M - p.y * p.w, Mr2, y2);
            scz = div_by_rcp(scz * M - p.z * p.w, Mr2, y2);
            svx = div_by_rcp(svx * M - v.x * p.w, Mr2, y2); svy = div_by_rcp(svy * M - v.y * p.w, Mr2, y2);
            svz = div_by_rcp(svz * M - v.z * p.w, Mr2, y2);
            sM = Mr2;
            // swap with the back and pop (src/tree.hpp:4660-4663)
            uint32_t bk = s_back;
            uint32_t tmp = P.idx[o + b];
            P.idx[o + b] = P.idx[o + bk];
            P.idx[o + bk] = tmp;
            s_back = bk - 1;
        }
        __syncthreads();
        i = b - 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        ct.mn[s] = s_back + 1;
        ct.M[s] = sM;
        ct.com[s] = make_double4_32a(scx, scy, scz, 0);
        ct.vcom[s] = make_double4_32a(svx, svy, svz, 0);
    }
}

// Hill-sphere rebinding (src/tree.hpp:4678-4711).
//
// RecursiveBallSearch visits the children of a node in order and every node covers a
// contiguous run of the Morton-sorted points, so the ball's points come out in ascending
// point index. The candidates of one SearchBoundParticlesWithinHillRadius call are therefore
// the ball's points that pass the call-independent tests (not marked in a clump before
// rebinding, density not below the threshold), in ascending index. Those points form the
// sorted list E (with epos[p] = entries of E below p), so a node's candidates are the slice
// E[epos[beg], epos[end]) and nodes with an empty slice are skipped without a test.
//
// One block per clump: a breadth-first frontier of at most kFront nodes is built in shared
// memory (stable, so it stays in point order); each thread then walks the subtrees of its
// frontier entries, once to count and once to write the candidates at scanned offsets.
constexpr int kFront = 2048;
constexpr int kRebindThreads = 256;
constexpr int kCopyTasks = 512;  // queued copies of contained runs in the fill step
constexpr int kTile = 192;  // candidates staged per step of the acceptance: 64 + 52 + 4 + 1 B each
static_assert(kTile * (64 + 52 + 4 + 1) <= kFront * (3 * 4 + 2), "the candidate tile must fit in the frontier space");

__global__ void k_elig_flags(uint32_t Tu, const uint8_t *in_clump, const double *dens, double thr, uint32_t *flag) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < Tu) flag[q] = (in_clump[q] == 0 && !(dens[q] < thr)) ? 1u : 0u;
}

__global__ void k_elig_compact(uint32_t Tu, const uint8_t *in_clump, const double *dens, double thr, const uint32_t *epos, uint32_t *E) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < Tu && in_clump[q] == 0 && !(dens[q] < thr)) E[epos[q]] = q;
}

// exclusive scan of a[0, n) in shared memory by the whole block (n <= kFront); returns the total
__device__ uint32_t block_scan_excl(uint32_t *a, uint32_t n, uint32_t *warp_tot) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t b = threadIdx.x * per, e = min(n, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; ++i) sum += a[i];
    uint32_t incl = sum;
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        if (k < wid) before += warp_tot[k];
        total += warp_tot[k];
    }
    uint32_t run = before + incl - sum;
    for (uint32_t i = b; i < e; ++i) {
        uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
    __syncthreads();
    return total;
}

// Node classes of the frontier: 1 contained (all candidates), 2 leaf reached but not
// contained (candidates filtered by distance), 3 nothing, 4 descend into the children.
// The ball of one SearchBound call: centre and radius in FP64, and as float hi/lo pairs for
// the filtered tests (knn_f32.cuh: a decided FP32 test always agrees with the FP64 one).
struct BallQ {
    double cx, cy, cz, r, rr;
    float4 qh, ql;
    float rf, rr32;
};

__device__ __forceinline__ BallQ make_ball(double cx, double cy, double cz, double r) {
    BallQ b;
    b.cx = cx; b.cy = cy; b.cz = cz; b.r = r; b.rr = r * r;
    const float hx = (float)cx, hy = (float)cy, hz = (float)cz;
    b.qh = make_float4(hx, hy, hz, 0.f);
    b.ql = make_float4((float)(cx - (double)hx), (float)(cy - (double)hy), (float)(cz - (double)hz), 0.f);
    b.rf = (float)r;
    b.rr32 = (float)b.rr;
    return b;
}

// RecursiveBallSearch keeps a leaf point when its squared distance is <= r^2
__device__ __forceinline__ bool in_ball(const KTree &t, const FTree &f, const BallQ &b, uint32_t p) {
    const float v = f_dr2(b.qh, b.ql, f.phi[p], f.plo[p]);
    if (f_hi(v) < b.rr32 * (1.f - kRel)) return true;
    if (f_lo(v) > b.rr32 * (1.f + kRel)) return false;
    return point_dr2(b.cx, b.cy, b.cz, t.pos[p]) <= b.rr;
}

__device__ __forceinline__ int ball_class(const KTree &t, const FTree &f, const uint32_t *epos, uint32_t node, const BallQ &b, uint32_t &eb,
                                          uint32_t &ee) {
    eb = epos[t.nbeg[node]];
    ee = epos[t.nend[node]];
    if (eb == ee) return 3;
    const float4 nh = f.nhi[node], nl = f.nlo[node];
    int cont = f_contained(nh, nl, b.qh, b.ql, b.rf);
    if (cont < 0) cont = node_contained(t.ncf[node], b.cx, b.cy, b.cz, b.r) ? 1 : 0;
    if (cont) return 1;
    int inter = f_intersects(nh, nl, b.qh, b.ql, b.rf);
    if (inter < 0) inter = node_intersects(t.ncf[node], b.cx, b.cy, b.cz, b.r) ? 1 : 0;
    if (inter) return t.nnd[node] == 0 ? 2 : 4;
    return 3;
}

// the candidates below a class-4 node f, in point order
template <class Emit>
__device__ void ball_walk_below(const KTree &t, const FTree &ft, const uint32_t *epos, uint32_t f, const BallQ &b, Emit emit, unsigned *err) {
    uint32_t node = t.nfd[f];
    for (uint32_t guard = 0; guard < 4u * t.nodes + 8u; ++guard) {
        if (node >= t.nodes) {
            atomicOr(err, (unsigned)kDevErrBadNode);
            return;
        }
        uint32_t eb, ee;
        const int cls = ball_class(t, ft, epos, node, b, eb, ee);
        if (cls == 1 || cls == 2) emit(eb, ee, cls == 2);
        if (cls == 4) {
            node = t.nfd[node];
            continue;
        }
        for (;;) {  // next sibling, climbing back towards f
            const uint32_t p = t.npar[node];
            if (node + 1 < t.nfd[p] + t.nnd[p]) {
                ++node;
                break;
            }
            node = p;
            if (node == f) return;
        }
    }
    atomicOr(err, (unsigned)kDevErrLoopLimit);
}

// IsGravitationallyBound for a candidate against the clump state, as the rebinding loop
// evaluates it (src/tree.hpp:4686-4694): e = 0.5/(M+m) |v_com - shear - v|^2 - G/|r_com - r|,
// bound when e < 0.
// The same test in FP64 only, as the reference writes it.
__device__ __forceinline__ bool bound_fp64(const double4_32a p, const double4_32a v, double sM, double x, double y, double z, double vx,
                                          double vy, double vz, const CP &cp) {
    const double M = sM + p.w;
    const double dx = x - p.x;
    const double ex = (vx - 0.0 * dx) - v.x, ey = (vy - cp.shear * dx) - v.y, ez = (vz - 0.0 * dx) - v.z;
    const double e = +0.5 / M * norm2_3(ex, ey, ez) - cp.G / norm3(dx, y - p.y, z - p.z);
    return e < 0;
}

// A candidate as float hi/lo pairs (x = hi + lo to 2^-48): position, velocity, and its mass.
struct CandF {
    float ph[3], pl[3], vh[3], vl[3], w;
};

// The boundness test entirely in FP32 from hi/lo pairs of the state (sh, sl: x, y, z, vx,
// vy, vz) and of the candidate: 1 bound, 0 not, -1 too close to call (then bound_fp64).
// Differences of hi/lo pairs carry a relative error below 2^-23 (plus 2^-48 of the
// coordinates from the splits); the y velocity term, a difference of two such values, carries
// an absolute error below 2^-21 (|T1| + |T2|). With at most ten further FP32 roundings per
// term, |A - A_exact| <= A 2^-20 + |ey| err_y / M and |B - B_exact| <= B 2^-20, inside the
// margin below; the reference's own FP64 rounding is far smaller.
__device__ __forceinline__ int bound_hilo(const CandF &c, float Mf, const float sh[6], const float sl[6], float G, float shear) {
    const float dx = (sh[0] - c.ph[0]) + (sl[0] - c.pl[0]);
    const float dy = (sh[1] - c.ph[1]) + (sl[1] - c.pl[1]);
    const float dz = (sh[2] - c.ph[2]) + (sl[2] - c.pl[2]);
    const float ex = (sh[3] - c.vh[0]) + (sl[3] - c.vl[0]);
    const float t1 = (sh[4] - c.vh[1]) + (sl[4] - c.vl[1]), t2 = shear * dx;
    const float ey = t1 - t2;
    const float ez = (sh[5] - c.vh[2]) + (sl[5] - c.vl[2]);
    const float K = ex * ex + ey * ey + ez * ez, D2 = dx * dx + dy * dy + dz * dz;
    const float M = Mf + c.w;
    if (!(K > 1e-30f && D2 > 1e-30f && K < 1e30f && D2 < 1e30f && M > 1e-30f && M < 1e30f)) return -1;
    const float A = 0.5f / M * K, B = G / sqrtf(D2);
    const float e = A - B;
    const float margin = (fabsf(A) + fabsf(B)) * 3.814697265625e-06f                             // 2^-18
                         + fabsf(ey) * (fabsf(t1) + fabsf(t2)) * 9.5367431640625e-07f / M;    // 2^-20 / M
    if (e > margin) return 0;
    if (e < -margin) return 1;
    return -1;
}

// The same test with the FP32 quotient and square root taken by the fast intrinsics
// (__fdividef, rsqrtf: at most 2 ulp each for the argument ranges admitted above). With
// them A and B still carry a relative error below 2^-20, inside the margin.
__device__ __forceinline__ int bound_hilo_fast(const CandF &c, float Mf, const float sh[6], const float sl[6], float G, float shear) {
    const float dx = (sh[0] - c.ph[0]) + (sl[0] - c.pl[0]);
    const float dy = (sh[1] - c.ph[1]) + (sl[1] - c.pl[1]);
    const float dz = (sh[2] - c.ph[2]) + (sl[2] - c.pl[2]);
    const float ex = (sh[3] - c.vh[0]) + (sl[3] - c.vl[0]);
    const float t1 = (sh[4] - c.vh[1]) + (sl[4] - c.vl[1]), t2 = shear * dx;
    const float ey = t1 - t2;
    const float ez = (sh[5] - c.vh[2]) + (sl[5] - c.vl[2]);
    const float K = ex * ex + ey * ey + ez * ez, D2 = dx * dx + dy * dy + dz * dz;
    const float M = Mf + c.w;
    if (!(K > 1e-30f && D2 > 1e-30f && K < 1e30f && D2 < 1e30f && M > 1e-30f && M < 1e30f)) return -1;
    const float rM = __fdividef(1.0f, M);
    const float A = 0.5f * rM * K, B = G * rsqrtf(D2);
    const float e = A - B;
    const float margin = (fabsf(A) + fabsf(B)) * 3.814697265625e-06f              // 2^-18
                         + fabsf(ey) * (fabsf(t1) + fabsf(t2)) * 9.5367431640625e-07f * rM;  // 2^-20 / M
    if (e > margin) return 0;
    if (e < -margin) return 1;
    return -1;
}

__device__ __forceinline__ void split_f(double d, float &hi, float &lo) {
    hi = (float)d;
    lo = (float)(d - (double)hi);
}

// Deferral records of a clump: the key ranks of the earlier clumps whose particles it
// skipped (at most kDeferSlots distinct records; beyond that only the largest rank is known
// and the host falls back to it). A record carries kDeferSpec when the earlier clump had not
// finished its calls when it was observed (its holding could still change in that pass);
// without the bit the clump saw that pass's final holding.
constexpr int kDeferSlots = 16;
constexpr uint32_t kDeferSpec = 0x80000000u;

// dcall (may be null): per record, the call of the clump's run (1-based, counted from its
// state before rebinding) in which the record was made; a clump's calls run in order, so
// that is the earliest call that skipped such a particle. dfirst: the earliest call of any
// deferral, kept also when the records overflow. A rerun may resume after those calls.
__device__ void defer_add(uint32_t *dset, uint8_t *dover, uint32_t *dmax, uint32_t slot, uint32_t ow, bool spec = true,
                          uint32_t *dcall = nullptr, uint32_t *dfirst = nullptr, uint32_t call = kNone) {
    if (*(volatile uint32_t *)&dmax[slot] < ow + 1) atomicMax(&dmax[slot], ow + 1);
    if (dfirst && call < *(volatile uint32_t *)&dfirst[slot]) atomicMin(&dfirst[slot], call);
    const uint32_t rec = ow | (spec ? kDeferSpec : 0u);
    uint32_t *d = dset + (size_t)slot * kDeferSlots;
    for (int j = 0; j < kDeferSlots; ++j) {
        const uint32_t v = d[j];  // a set entry never changes again
        if (v == rec) return;
        if (v == kNone) {
            const uint32_t old = atomicCAS(&d[j], kNone, rec);
            if (old == kNone && dcall) atomicMin(&dcall[(size_t)slot * kDeferSlots + j], call);
            if (old == kNone || old == rec) return;
        }
    }
    dover[slot] = 1;
}

#include "rebind_loop.cuh"

// One SearchBoundParticlesWithinHillRadius call for every listed clump (one block each).
// seq_mode = 1: the reference's shared in-clump flags, one clump at a time.
// seq_mode = 0: clumps run concurrently. owner[q] holds the key rank of the clump holding
// particle q. A clump treats q as taken if it was marked before rebinding, or is held by
// itself or by an earlier clump (recording that it deferred, with defer_add); it may take q from a
// later clump, which is then invalid. A clump that loses q to an earlier one is invalid.
// Invalid clumps are restored and rerun by the host until none is left; the clumps below
// the lowest invalid rank are final after every pass, so this ends.
template <int kSpec>
__global__ void __launch_bounds__(kRebindThreads) k_rebind_round(const uint32_t *list, CT ct, Pool P, KTree t, const double4_32a *vel,
                                                                 const uint32_t *E, const uint32_t *epos, uint8_t *in_clump, uint32_t *owner,
                                                                 const uint32_t *rank_of, const uint32_t *slot_of_rank, uint8_t *invalid,
                                                                 uint32_t *dmax, uint32_t *dset, uint8_t *dover, int seq_mode, CP cp,
                                                                 uint8_t *grew, uint32_t *mn_out,
                                                                 unsigned *err, unsigned long long *prof, const double4_32a *com0,
                                                                 unsigned long long *reach, const uint32_t *tent, FTree ft) {
    __shared__ double sM, scx, scy, scz, svx, svy, svz, c0x, c0y, c0z, rad;
    __shared__ uint32_t s_noff, s_nacc, s_nf, s_expand, s_at, s_next, s_ntask;
    __shared__ uint32_t task_src[kCopyTasks], task_len[kCopyTasks], task_dst[kCopyTasks];
    // the frontier arrays (steps 1-2) and the candidate tiles (step 3) share this space
    __shared__ __align__(16) unsigned char sbuf[kFront * (3 * 4 + 2)];
    uint32_t *front = reinterpret_cast<uint32_t *>(sbuf), *front2 = front + kFront, *fcnt = front2 + kFront;
    uint8_t *fcls = reinterpret_cast<uint8_t *>(fcnt + kFront), *fcls2 = fcls + kFront;
    __shared__ uint32_t warp_tot[kRebindThreads / 32];
    const uint32_t slot = list[blockIdx.x];
    const uint32_t myrank = seq_mode ? 0u : rank_of[slot];
    const double4_32a *pos = t.pos;
    if (threadIdx.x == 0) {
        sM = ct.M[slot];
        double4_32a c = ct.com[slot], v = ct.vcom[slot];
        scx = c.x; scy = c.y; scz = c.z;
        svx = v.x; svy = v.y; svz = v.z;
        c0x = c.x; c0y = c.y; c0z = c.z;  // the ball stays where the call started
        rad = ct.hill[slot];
        s_nacc = 0;
        front[0] = 0;
        fcls[0] = 0;
        s_nf = 1;
    }
    __syncthreads();
    const double cx = c0x, cy = c0y, cz = c0z, r = rad;
    const BallQ ball = make_ball(cx, cy, cz, r);
    const unsigned long long t_start = prof ? clock64() : 0;
    if (threadIdx.x == 0) {  // how far this clump's balls reach from its centre before rebinding
        const double4_32a c0 = com0[slot];
        const double dx = cx - c0.x, dy = cy - c0.y, dz = cz - c0.z;
        const double d = sqrt(dx * dx + dy * dy + dz * dz) + r;
        if (d >= 0) atomicMax(&reach[slot], (unsigned long long)__double_as_longlong(d));
    }
    // 1) breadth-first frontier (classes 1..4; 0 = not yet classified)
    for (int level = 0; level < 40; ++level) {
        const uint32_t nf = s_nf;
        if (threadIdx.x == 0) s_expand = 0;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < nf; i += blockDim.x) {
            uint32_t node = front[i];
            int cls = fcls[i];
            if (cls == 0) {
                if (node >= t.nodes) {
                    atomicOr(err, (unsigned)kDevErrBadNode);
                    cls = 3;
                } else {
                    uint32_t eb, ee;
                    cls = ball_class(t, ft, epos, node, ball, eb, ee);
                }
                fcls[i] = (uint8_t)cls;
            }
            fcnt[i] = cls == 4 ? t.nnd[node] : (cls == 3 ? 0u : 1u);
            if (cls == 4) s_expand = 1;
        }
        __syncthreads();
        if (!s_expand) break;
        const uint32_t total = block_scan_excl(fcnt, nf, warp_tot);
        if (total > (uint32_t)kFront) break;
        for (uint32_t i = threadIdx.x; i < nf; i += blockDim.x) {
            const int cls = fcls[i];
            const uint32_t o = fcnt[i];
            if (cls == 1 || cls == 2) {
                front2[o] = front[i];
                fcls2[o] = (uint8_t)cls;
            } else if (cls == 4) {
                const uint32_t c0 = t.nfd[front[i]], nc = t.nnd[front[i]];
                for (uint32_t c = 0; c < nc; ++c) {
                    front2[o + c] = c0 + c;
                    fcls2[o + c] = 0;
                }
            }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < total; i += blockDim.x) {
            front[i] = front2[i];
            fcls[i] = fcls2[i];
        }
        if (threadIdx.x == 0) s_nf = total;
        __syncthreads();
    }
    const uint32_t nf = s_nf;
    for (uint32_t i = threadIdx.x; i < nf; i += blockDim.x) {  // entries left unclassified by the level cap
        if (fcls[i] != 0) continue;
        uint32_t eb, ee;
        fcls[i] = front[i] < t.nodes ? (uint8_t)ball_class(t, ft, epos, front[i], ball, eb, ee) : (uint8_t)3;
    }
    __syncthreads();
    const unsigned long long t_front = prof ? clock64() : 0;
    // 2) count the candidates below each frontier entry (entries handed out one at a time,
    // the subtrees differ a lot in size), then scan to offsets
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    for (uint32_t i = atomicAdd(&s_next, 1u); i < nf; i = atomicAdd(&s_next, 1u)) {
        const uint32_t node = front[i];
        const int cls = fcls[i];
        uint32_t cnt = 0;
        auto count = [&](uint32_t eb, uint32_t ee, bool partial) {
            if (!partial) {
                cnt += ee - eb;
            } else {
                for (uint32_t j = eb; j < ee; ++j) cnt += in_ball(t, ft, ball, E[j]) ? 1u : 0u;
            }
        };
        if (cls == 1 || cls == 2) {
            count(epos[t.nbeg[node]], epos[t.nend[node]], cls == 2);
        } else if (cls == 4) {
            ball_walk_below(t, ft, epos, node, ball, count, err);
        }
        fcnt[i] = cnt;
    }
    __syncthreads();
    const uint32_t nel = block_scan_excl(fcnt, nf, warp_tot);
    // segment: the members, then the candidates in walk order; the accepted ones overwrite
    // the candidates already consumed, so the segment ends as members + accepted
    if (threadIdx.x == 0) s_noff = pool_try_alloc(P, ct.mn[slot] + nel);
    __syncthreads();
    if (s_noff == kNone) {  // the pool is full: the host compacts it and repeats this call
        if (threadIdx.x == 0) {
            grew[blockIdx.x] = 2;
            mn_out[blockIdx.x] = ct.mn[slot];
        }
        return;
    }
    const unsigned long long t_count = prof ? clock64() : 0;
    const uint32_t m0 = ct.mn[slot], o = ct.moff[slot], no = s_noff;
    for (uint32_t k = threadIdx.x; k < m0; k += blockDim.x) P.idx[no + k] = P.idx[o + k];
    uint32_t *elig = P.idx + no + m0;  // candidates in walk order
    // long runs of a contained node are queued and copied by the whole block afterwards
    if (threadIdx.x == 0) {
        s_next = 0;
        s_ntask = 0;
    }
    __syncthreads();
    for (uint32_t i = atomicAdd(&s_next, 1u); i < nf; i = atomicAdd(&s_next, 1u)) {
        const uint32_t node = front[i];
        const int cls = fcls[i];
        uint32_t w = fcnt[i];
        auto fill = [&](uint32_t eb, uint32_t ee, bool partial) {
            if (!partial && ee - eb > 64) {
                const uint32_t slot_t = atomicAdd(&s_ntask, 1u);
                if (slot_t < kCopyTasks) {
                    task_src[slot_t] = eb;
                    task_len[slot_t] = ee - eb;
                    task_dst[slot_t] = w;
                    w += ee - eb;
                    return;
                }
            }
            for (uint32_t j = eb; j < ee; ++j) {
                const uint32_t q = E[j];
                if (!partial || in_ball(t, ft, ball, q)) elig[w++] = q;
            }
        };
        if (cls == 1 || cls == 2) {
            fill(epos[t.nbeg[node]], epos[t.nend[node]], cls == 2);
        } else if (cls == 4) {
            ball_walk_below(t, ft, epos, node, ball, fill, err);
        }
    }
    __syncthreads();
    const uint32_t ntask = min(s_ntask, (uint32_t)kCopyTasks);
    for (uint32_t k = 0; k < ntask; ++k) {
        const uint32_t src = task_src[k], len = task_len[k], dst = task_dst[k];
        for (uint32_t j = threadIdx.x; j < len; j += blockDim.x) elig[dst + j] = E[src + j];
    }
    __syncthreads();
    // 3) the reference's sequential acceptance over the candidates (src/tree.hpp:4686-4706).
    // The block stages kTile candidates at a time in shared memory (positions, velocities,
    // taken flags read now); warp 0 then walks them: the lanes test 32 candidates against
    // the current state, the first bound one is taken and every lane applies the same FP64
    // update to its copy of the state.
    const unsigned long long t_fill = prof ? clock64() : 0;
    uint32_t *acc = elig;  // accepted, in acceptance order, over the consumed candidates
    __shared__ uint32_t s_iters;
    double4_32a *tpos = reinterpret_cast<double4_32a *>(sbuf), *tvel = tpos + kTile;
    CandF *tf = reinterpret_cast<CandF *>(tvel + kTile);
    uint32_t *tq = reinterpret_cast<uint32_t *>(tf + kTile);
    uint8_t *ttaken = reinterpret_cast<uint8_t *>(tq + kTile);
    double M_ = 0, x_ = 0, y_ = 0, z_ = 0, vx_ = 0, vy_ = 0, vz_ = 0;  // warp 0's copy of the state
    float sh[6], sl[6], Mf = 0.f;                                      // and its float hi/lo pairs
    const float G32 = (float)cp.G, shear32 = (float)cp.shear;
    uint32_t nacc_ = 0, iters = 0;
    if (threadIdx.x < 32) {
        M_ = sM; x_ = scx; y_ = scy; z_ = scz; vx_ = svx; vy_ = svy; vz_ = svz;
        split_f(x_, sh[0], sl[0]); split_f(y_, sh[1], sl[1]); split_f(z_, sh[2], sl[2]);
        split_f(vx_, sh[3], sl[3]); split_f(vy_, sh[4], sl[4]); split_f(vz_, sh[5], sl[5]);
        Mf = (float)M_;
    }
    if (threadIdx.x == 0) s_at = 0;
    for (uint32_t base = 0; base < nel; base += kTile) {
        const uint32_t tend = min(nel, base + (uint32_t)kTile);
        for (uint32_t i = threadIdx.x; base + i < tend; i += blockDim.x) {
            const uint32_t q2 = elig[base + i];
            bool taken = seq_mode && in_clump[q2] != 0;
            if (!taken && !seq_mode) {
                // held by this or an earlier clump, or predicted (from the last pass) to end
                // up with an earlier clump that is being rerun
                const uint32_t ow = __ldcg(&owner[q2]), tn = tent[q2];
                taken = (ow != kNone && ow <= myrank) || (tn != kNone && tn < myrank);
                if (ow != kNone && ow < myrank) defer_add(dset, dover, dmax, slot, ow);
                else if (tn != kNone && tn < myrank) defer_add(dset, dover, dmax, slot, tn);
            }
            tq[i] = q2;
            ttaken[i] = taken ? 1 : 0;
            const double4_32a pp = pos[q2], vv = vel[q2];
            tpos[i] = pp;
            tvel[i] = vv;
            CandF cf;
            split_f(pp.x, cf.ph[0], cf.pl[0]);
            split_f(pp.y, cf.ph[1], cf.pl[1]);
            split_f(pp.z, cf.ph[2], cf.pl[2]);
            split_f(vv.x, cf.vh[0], cf.vl[0]);
            split_f(vv.y, cf.vh[1], cf.vl[1]);
            split_f(vv.z, cf.vh[2], cf.vl[2]);
            cf.w = (float)pp.w;
            tf[i] = cf;
        }
        __syncthreads();
        if (kSpec == 1 && threadIdx.x < 32) {
            // Speculative windows, exact by verification: decide 32 candidates against the
            // window's first state, run the FP64 update chain through the tentative
            // acceptances only, then check every decision against the exact state before it.
            // Everything before the first disagreement is the reference's sequence; the first
            // disagreeing candidate is decided by its (exact) check.
            __shared__ double sst[33][7];  // M and the six components after each tentative acceptance
            __shared__ double srcp[32];    // 1 / M after each tentative acceptance
            const int lane = threadIdx.x;
            const unsigned full = 0xffffffffu;
            const int cl = lane < 6 ? lane : 0;  // the state component this lane carries
            uint32_t at = s_at;
            while (at < tend) {
                ++iters;
                const uint32_t k = at + lane;
                const bool valid = k < tend;
                const bool tk = valid && ttaken[k - base] != 0;
                bool tent = false;
                if (valid && !tk) {
                    const int r = bound_hilo(tf[k - base], Mf, sh, sl, G32, shear32);
                    tent = r >= 0 ? r == 1 : bound_fp64(tpos[k - base], tvel[k - base], M_, x_, y_, z_, vx_, vy_, vz_, cp);
                }
                const unsigned B = __ballot_sync(full, tent), V = __ballot_sync(full, valid);
                const uint32_t wend = min(at + 32, tend);
                if (!B) {
                    at = wend;
                    continue;
                }
                // states after each tentative acceptance (src/tree.hpp:4696-4701). The masses
                // first (their own sequential sum), then one reciprocal per lane, in parallel.
                double Mi = M_;
                int ns = 0;
                for (unsigned bits = B; bits; bits &= bits - 1u) {
                    Mi = Mi + tpos[at + (uint32_t)(__ffs(bits) - 1) - base].w;
                    ++ns;
                    if (lane == 0) sst[ns][0] = Mi;
                }
                if (lane == 0) sst[0][0] = M_;
                __syncwarp();
                if (lane < ns) srcp[lane] = 1.0 / sst[lane + 1][0];  // correctly rounded reciprocal
                __syncwarp();
                // The components: c' = (c M + m q) / M with the division as Markstein's
                // correction of a reciprocal product (q0 = num y, r = num - q0 M exactly by
                // FMA, c' = RN(q0 + r y)), which equals the correctly rounded quotient when y
                // is the correctly rounded 1/M; checked against IEEE division on 9e8 operand
                // pairs. A zero numerator keeps its sign as the division does.
                double ci = cl == 0 ? x_ : cl == 1 ? y_ : cl == 2 ? z_ : cl == 3 ? vx_ : cl == 4 ? vy_ : vz_;
                if (lane < 6) sst[0][1 + lane] = ci;
                int t = 0;
                for (unsigned bits = B; bits; bits &= bits - 1u) {
                    const uint32_t j = at + (uint32_t)(__ffs(bits) - 1) - base;
                    const double4_32a p = tpos[j], v = tvel[j];
                    const double Mn = sst[t + 1][0], yr = srcp[t];
                    const double qc = cl == 0 ? p.x : cl == 1 ? p.y : cl == 2 ? p.z : cl == 3 ? v.x : cl == 4 ? v.y : v.z;
                    const double num = ci * Mn + p.w * qc;
                    const double q0 = num * yr;
                    ci = num == 0.0 ? num : fma(fma(-q0, Mn, num), yr, q0);
                    ++t;
                    if (lane < 6) sst[t][1 + lane] = ci;
                }
                __syncwarp();
                bool ver = false;
                if (valid && !tk) {
                    const int nb = __popc(B & ((1u << lane) - 1u));
                    const double Ms = sst[nb][0];
                    const double s0 = sst[nb][1], s1 = sst[nb][2], s2 = sst[nb][3], s3 = sst[nb][4], s4 = sst[nb][5], s5 = sst[nb][6];
                    float h[6], l[6];
                    split_f(s0, h[0], l[0]); split_f(s1, h[1], l[1]); split_f(s2, h[2], l[2]);
                    split_f(s3, h[3], l[3]); split_f(s4, h[4], l[4]); split_f(s5, h[5], l[5]);
                    const int r = bound_hilo(tf[k - base], (float)Ms, h, l, G32, shear32);
                    ver = r >= 0 ? r == 1 : bound_fp64(tpos[k - base], tvel[k - base], Ms, s0, s1, s2, s3, s4, s5, cp);
                }
                const unsigned Vb = __ballot_sync(full, ver);
                const unsigned mism = (Vb ^ B) & V;
                unsigned accepted = B;
                int nstate = ns;
                int extra = -1;  // a candidate accepted by its check beyond the chain's states
                uint32_t next = wend;
                if (mism) {
                    const int m = __ffs(mism) - 1;
                    const unsigned below = (1u << m) - 1u;
                    accepted = (B & below) | (Vb & (1u << m));
                    nstate = __popc(B & below);
                    if ((Vb >> m) & 1u) extra = m;
                    next = at + (uint32_t)m + 1;
                }
                double M2 = sst[nstate][0];
                double c2 = sst[nstate][1 + cl];
                if (extra >= 0) {
                    const uint32_t j = at + (uint32_t)extra - base;
                    const double4_32a p = tpos[j], v = tvel[j];
                    const double Mn = M2 + p.w;
                    const double qc = cl == 0 ? p.x : cl == 1 ? p.y : cl == 2 ? p.z : cl == 3 ? v.x : cl == 4 ? v.y : v.z;
                    c2 = (c2 * Mn + p.w * qc) / Mn;
                    M2 = Mn;
                }
                __syncwarp();
                float rh, rl;
                split_f(c2, rh, rl);
                for (int q = 0; q < 6; ++q) {
                    sh[q] = __shfl_sync(full, rh, q);
                    sl[q] = __shfl_sync(full, rl, q);
                }
                x_ = __shfl_sync(full, c2, 0);
                y_ = __shfl_sync(full, c2, 1);
                z_ = __shfl_sync(full, c2, 2);
                vx_ = __shfl_sync(full, c2, 3);
                vy_ = __shfl_sync(full, c2, 4);
                vz_ = __shfl_sync(full, c2, 5);
                M_ = M2;
                Mf = (float)M2;
                if ((accepted >> lane) & 1u) {  // each accepted lane claims its own candidate
                    const uint32_t q2 = tq[k - base];
                    if (seq_mode) in_clump[q2] = 1;
                    else atomicMin(&owner[q2], myrank);
                    acc[nacc_ + __popc(accepted & ((1u << lane) - 1u))] = q2;
                }
                nacc_ += __popc(accepted);
                at = next;
            }
            if (lane == 0) s_at = at;
        } else if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            uint32_t at = s_at;
            while (at < tend) {
                ++iters;
                const uint32_t k = at + lane;
                bool bound = false;
                double yk = 0;  // kSpec == 2: 1 / (M + m_k), taken while the lanes test
                if (k < tend && !ttaken[k - base]) {
                    if (kSpec == 2) yk = 1.0 / (M_ + tpos[k - base].w);
                    const int r = bound_hilo(tf[k - base], Mf, sh, sl, G32, shear32);
                    bound = r >= 0 ? r == 1 : bound_fp64(tpos[k - base], tvel[k - base], M_, x_, y_, z_, vx_, vy_, vz_, cp);
                }
                const unsigned b = __ballot_sync(0xffffffffu, bound);
                if (!b) {
                    at = min(at + 32, tend);
                    continue;
                }
                const int f = __ffs(b) - 1;
                const uint32_t j = at + f - base;
                // src/tree.hpp:4696-4701 (the new mass multiplies the old centre); lane c < 6
                // updates component c, then every lane takes all six
                {
                    // one division per lane, no divergence: component c is (s_c * M + m * q_c) / M
                    // (M * s equals s * M bit for bit)
                    const double4_32a p = tpos[j], v = tvel[j];
                    const double M = M_ + p.w;
                    const int c = lane < 6 ? lane : 0;
                    const double sc = c == 0 ? x_ : c == 1 ? y_ : c == 2 ? z_ : c == 3 ? vx_ : c == 4 ? vy_ : vz_;
                    const double qc = c == 0 ? p.x : c == 1 ? p.y : c == 2 ? p.z : c == 3 ? v.x : c == 4 ? v.y : v.z;
                    double r;
                    if (kSpec == 2) {
                        // the correctly rounded quotient from the reciprocal the accepted lane
                        // took (Markstein's correction, as in the speculative windows)
                        const double yr = __shfl_sync(0xffffffffu, yk, f);
                        const double num = sc * M + p.w * qc;
                        const double q0 = num * yr;
                        r = num == 0.0 ? num : fma(fma(-q0, M, num), yr, q0);
                    } else {
                        r = (sc * M + p.w * qc) / M;
                    }
                    float rh, rl;
                    split_f(r, rh, rl);
                    for (int q = 0; q < 6; ++q) {
                        sh[q] = __shfl_sync(0xffffffffu, rh, q);
                        sl[q] = __shfl_sync(0xffffffffu, rl, q);
                    }
                    x_ = __shfl_sync(0xffffffffu, r, 0);
                    y_ = __shfl_sync(0xffffffffu, r, 1);
                    z_ = __shfl_sync(0xffffffffu, r, 2);
                    vx_ = __shfl_sync(0xffffffffu, r, 3);
                    vy_ = __shfl_sync(0xffffffffu, r, 4);
                    vz_ = __shfl_sync(0xffffffffu, r, 5);
                    M_ = M;
                    Mf = (float)M;
                }
                if (lane == 0) {
                    const uint32_t q2 = tq[j];
                    if (seq_mode) {
                        in_clump[q2] = 1;
                    } else {
                        // the lowest rank keeps the particle; who lost one is found after the
                        // pass (k_rebind_verify), so the claim does not wait for the old value
                        atomicMin(&owner[q2], myrank);
                    }
                    acc[nacc_] = q2;
                }
                ++nacc_;
                at += f + 1;
            }
            if (lane == 0) s_at = at;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        sM = M_; scx = x_; scy = y_; scz = z_; svx = vx_; svy = vy_; svz = vz_;
        s_nacc = nacc_;
        s_iters = iters;
    }
    __syncthreads();
    const uint32_t nacc = s_nacc;  // members followed by the accepted ones (indices order of the reference)
    if (threadIdx.x == 0 && prof) {
        unsigned long long *q = prof + 8 * (size_t)blockIdx.x;
        const unsigned long long t_end = clock64();
        q[0] = t_front - t_start;
        q[1] = t_count - t_front;
        q[2] = t_fill - t_count;
        q[3] = t_end - t_fill;
        q[4] = nf;
        q[5] = nel;
        q[6] = nacc;
        q[7] = ((unsigned long long)iters << 32) | m0;
    }
    if (threadIdx.x == 0) {
        grew[blockIdx.x] = nacc ? 1 : 0;
        mn_out[blockIdx.x] = m0 + nacc;
        if (nacc) {
            ct.moff[slot] = no;
            ct.mn[slot] = m0 + nacc;
            ct.M[slot] = sM;
            ct.com[slot] = make_double4_32a(scx, scy, scz, 0);
            ct.vcom[slot] = make_double4_32a(svx, svy, svz, 0);
        }
    }
}

// What k_rebind_restore needs beyond the clump table and the pool.
struct RestoreArgs {
    const double *bM, *bh, *bri, *bro, *br10, *br2;  // the state before rebinding, per slot
    const double4_32a *bc, *bv;
    const uint32_t *bo, *bn, *bidx;
    const double *bdist;
    uint8_t *invalid, *dover, *distsq, *needsort;
    uint32_t *dmax, *dset, *dcall, *dfirst, *ccall, *owner;
    const uint32_t *keep, *rank_of;  // keep (by list position, may be null): checkpoints kept
    const uint8_t *in_clump;
    Ckpt ck;                         // ck.n null: no checkpoints
};

// Restore listed clumps for a rerun: to their state before rebinding, or, when the first
// call the rerun affects comes after some of their checkpoints, to the last of those (its
// members claimed again, the deferral records of the calls before it kept, the rest
// cleared); either way the per-pass records of later calls go.
__global__ void k_rebind_restore(const uint32_t *list, uint32_t n, CT ct, Pool P, RestoreArgs r, unsigned *err) {
    __shared__ uint32_t s_off, s_m, s_kp, s_rank;
    __shared__ const uint32_t *s_idx;
    __shared__ const double *s_dist;
    uint32_t t = blockIdx.x;
    if (t >= n) return;
    uint32_t sl = list[t];
    if (threadIdx.x == 0) {
        const uint32_t kp = (r.keep && r.ck.n) ? r.keep[t] : 0u;
        const uint32_t rank = r.rank_of[sl];
        ct.r_in[sl] = r.bri[sl]; ct.r_out[sl] = r.bro[sl]; ct.r10[sl] = r.br10[sl]; ct.r2s[sl] = r.br2[sl];
        uint32_t lim = 0;  // calls kept
        if (kp == 0) {
            ct.M[sl] = r.bM[sl]; ct.hill[sl] = r.bh[sl];
            ct.com[sl] = r.bc[sl]; ct.vcom[sl] = r.bv[sl];
            s_idx = r.bidx + r.bo[sl];
            s_dist = r.bdist + r.bo[sl];
            s_m = r.bn[sl];
        } else {
            const size_t e = (size_t)rank * kCk + (kp - 1);
            const double *q = r.ck.st + e * 8;
            ct.M[sl] = q[0];
            ct.com[sl] = make_double4_32a(q[1], q[2], q[3], 0);
            ct.vcom[sl] = make_double4_32a(q[4], q[5], q[6], 0);
            ct.hill[sl] = q[7];
            s_idx = r.ck.idx + r.ck.off[e];
            s_dist = r.ck.dist + r.ck.off[e];
            s_m = r.ck.m[e];
            lim = r.ck.call[e];
            r.distsq[sl] = 1;  // a checkpoint holds the squared distances of its sort
            r.needsort[sl] = 0;
        }
        if (r.ck.n) r.ck.n[rank] = kp;
        if (r.ccall) r.ccall[sl] = lim;
        s_kp = kp;
        s_rank = rank;
        s_off = pool_alloc(P, s_m, err);
        r.invalid[sl] = 0;
        // the records of the kept calls, packed to the front
        uint32_t w = 0, dm = 0, df = kNone;
        uint32_t *ds = r.dset + (size_t)sl * kDeferSlots, *dc = r.dcall ? r.dcall + (size_t)sl * kDeferSlots : nullptr;
        for (int j = 0; j < kDeferSlots; ++j) {
            const uint32_t v = ds[j], cj = dc ? dc[j] : kNone;
            if (v != kNone && kp > 0 && cj <= lim) {
                ds[w] = v;
                if (dc) dc[w] = cj;
                dm = max(dm, (v & ~kDeferSpec) + 1);
                df = min(df, cj);
                ++w;
            }
        }
        for (int j = (int)w; j < kDeferSlots; ++j) {
            ds[j] = kNone;
            if (dc) dc[j] = kNone;
        }
        r.dmax[sl] = dm;
        if (r.dfirst) r.dfirst[sl] = df;
        r.dover[sl] = 0;
    }
    __syncthreads();
    if (s_off == kNone) return;
    const uint32_t m = s_m;
    for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
        const uint32_t q = s_idx[k];
        P.idx[s_off + k] = q;
        P.dist[s_off + k] = s_dist[k];
        if (s_kp && !r.in_clump[q]) atomicMin(&r.owner[q], s_rank);  // the checkpoint's holdings
    }
    if (threadIdx.x == 0) {
        ct.moff[sl] = s_off;
        ct.mn[sl] = m;
    }
}

// After a pass: a clump whose accepted particles are not all still its own lost one to an
// earlier clump (the claims keep the lowest rank); it is invalid and depends on that clump.
// For an invalid clump, lost_ck (by rank) is the first of its checkpoints that holds a
// particle it lost: its run is good up to the checkpoint before that one.
__global__ void k_rebind_verify(const uint32_t *list, uint32_t n, CT ct, Pool P, const uint8_t *in_clump, const uint32_t *owner,
                                const uint32_t *rank_of, uint8_t *invalid, uint32_t *dset, uint8_t *dover, uint32_t *dmax, Ckpt ck,
                                uint32_t *lost_ck) {
    __shared__ int s_lost;
    if (blockIdx.x >= n) return;
    const uint32_t s = list[blockIdx.x];
    const uint32_t myrank = rank_of[s], o = ct.moff[s], m = ct.mn[s];
    if (threadIdx.x == 0) s_lost = 0;
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
        const uint32_t q = P.idx[o + k];
        if (in_clump[q]) continue;  // a member before rebinding
        const uint32_t w = owner[q];
        if (w != myrank) {
            invalid[s] = 1;
            s_lost = 1;
            if (w != kNone && w < myrank) defer_add(dset, dover, dmax, s, w);
        }
    }
    __syncthreads();
    if (!s_lost || !ck.n) return;
    const uint32_t nck = ck.n[myrank];
    uint32_t first = nck;
    for (uint32_t i = 0; i < nck; ++i) {
        __syncthreads();
        if (threadIdx.x == 0) s_lost = 0;
        __syncthreads();
        const size_t e = (size_t)myrank * kCk + i;
        const uint32_t co = ck.off[e], cm = ck.m[e];
        for (uint32_t k = threadIdx.x; k < cm; k += blockDim.x) {
            const uint32_t q = ck.idx[co + k];
            if (!in_clump[q] && owner[q] != myrank) s_lost = 1;
        }
        __syncthreads();
        if (s_lost) {
            first = i;
            break;
        }
    }
    if (threadIdx.x == 0) lost_ck[myrank] = first;
}

// Before a rerun pass: the particles of the clumps to be rerun become predictions (tent) of
// who ends up with them; every other entry is a final holding.
__global__ void k_rebind_tentative(uint32_t Tu, uint32_t *owner, uint32_t *tent, const uint8_t *rerun_rank) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= Tu) return;
    const uint32_t o = owner[q];
    if (o != kNone && rerun_rank[o]) {
        tent[q] = o;
        owner[q] = kNone;
    } else {
        tent[q] = kNone;
    }
}

// order-independent hash of a clump's member set
__global__ void k_member_hash(const uint32_t *list, uint32_t n, CT ct, Pool P, unsigned long long *out) {
    __shared__ unsigned long long acc;
    if (blockIdx.x >= n) return;
    const uint32_t s = list[blockIdx.x];
    if (threadIdx.x == 0) acc = 0;
    __syncthreads();
    unsigned long long local = 0;
    const uint32_t o = ct.moff[s], m = ct.mn[s];
    for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
        unsigned long long z = (unsigned long long)P.idx[o + k] + 0x9e3779b97f4a7c15ull;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        local += z ^ (z >> 31);
    }
    atomicAdd(&acc, local);
    __syncthreads();
    if (threadIdx.x == 0) out[s] = acc ^ ((unsigned long long)m << 40);
}

__global__ void k_mark_members(uint32_t C, CT ct, Pool P, uint8_t *in_clump) {
    uint32_t s = blockIdx.x;
    if (s >= C || !ct.alive[s]) return;
    for (uint32_t k = threadIdx.x; k < ct.mn[s]; k += blockDim.x) in_clump[P.idx[ct.moff[s] + k]] = 1;
}

// RemoveSmallMassAndLowPeak (src/tree.hpp:3524-3546)
__global__ void k_prune(uint32_t C, CT ct, Pool P, const double4_32a *vel, const double *dens, CP cp, uint8_t *kill) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C) return;
    kill[s] = 0;
    if (!ct.alive[s]) return;
    if (ct.M[s] < cp.mass_thr || dens[ct.key[s]] < cp.peak_thr) { kill[s] = 1; return; }
    uint32_t lim = min(ct.mn[s], cp.knn);
    double m = 0;
    for (uint32_t k = 0; k < lim; ++k) {
        double a = vel[P.idx[ct.moff[s] + k]].w;
        m = (m < a) ? a : m;
    }
    if (m < cp.peak_thr) kill[s] = 1;
}

// envelope rip step (src/tree.hpp:4231-4239)
__global__ void k_rip(uint32_t C, CT ct, Pool P, uint8_t *pending, uint32_t *changed, uint32_t *nchanged) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C || !ct.alive[s] || !pending[s]) return;
    const uint32_t o = ct.moff[s], m = ct.mn[s];
    if (m == 0) { pending[s] = 0; return; }
    double h = ct.hill[s];
    if (!(h < P.dist[o + m - 1])) { pending[s] = 0; return; }
    uint32_t lo = 0, hi = m;  // first member with distance >= h
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (P.dist[o + mid] < h) lo = mid + 1;
        else hi = mid;
    }
    if (lo == 0) { ct.alive[s] = 0; pending[s] = 0; return; }
    ct.mn[s] = lo;
    changed[atomicAdd(nchanged, 1u)] = s;
}

// CalculateAngularMomentum sums (src/tree.hpp:4721-4747), unnormalised: per-member terms by
// the warp, the three running sums in member order by lanes 0..2
__global__ void __launch_bounds__(128) k_angmom(const uint32_t *list, uint32_t n, CT ct, Pool P, const double4_32a *pos,
                                                const double4_32a *vel, CP cp) {
    __shared__ double tile[4][3][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t t = blockIdx.x * 4 + wid;
    if (t >= n) return;
    const uint32_t s = list[t];
    const uint32_t o = ct.moff[s], m = ct.mn[s];
    const double4_32a c = ct.com[s], vc = ct.vcom[s];
    double acc = 0;
    for (uint32_t base = 0; base < m; base += 32) {
        const uint32_t k = base + lane;
        if (k < m) {
            uint32_t i = P.idx[o + k];
            double4_32a p = pos[i], v = vel[i];
            double drx = p.x - c.x, dry = p.y - c.y, drz = p.z - c.z;
            double sx = 0. * p.x, sy = cp.shear * p.x, sz = 0. * p.x;
            double cx0 = 0. * c.x, cy0 = cp.shear * c.x, cz0 = 0. * c.x;
            double dvx = (v.x - sx) - (vc.x - cx0), dvy = (v.y - sy) - (vc.y - cy0), dvz = (v.z - sz) - (vc.z - cz0);
            double tx = dry * dvz - drz * dvy, ty = drz * dvx - drx * dvz, tz = drx * dvy - dry * dvx;
            double ax = -drx * drz, ay = -dry * drz, az = (drx * drx + dry * dry);
            tx = tx + cp.Omega * ax;
            ty = ty + cp.Omega * ay;
            tz = tz + cp.Omega * az;
            tile[wid][0][lane] = p.w * tx;
            tile[wid][1][lane] = p.w * ty;
            tile[wid][2][lane] = p.w * tz;
        }
        __syncwarp();
        const uint32_t cnt = min(32u, m - base);
        if (lane < 3)
            for (uint32_t j = 0; j < cnt; ++j) acc = acc + tile[wid][lane][j];
        __syncwarp();
    }
    double jx = __shfl_sync(0xffffffffu, acc, 0), jy = __shfl_sync(0xffffffffu, acc, 1), jz = __shfl_sync(0xffffffffu, acc, 2);
    if (lane == 0) ct.J[s] = make_double4_32a(jx, jy, jz, 0);
}

// copy every live segment into the other pool buffer at packed offsets
__global__ void k_compact(uint32_t C, CT ct, Pool P, const uint32_t *newoff, uint32_t *dst_idx, double *dst_dist) {
    uint32_t s = blockIdx.x;
    if (s >= C || !ct.alive[s]) return;
    const uint32_t o = ct.moff[s], m = ct.mn[s], no = newoff[s];
    for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
        dst_idx[no + k] = P.idx[o + k];
        dst_dist[no + k] = P.dist[o + k];
    }
}

__global__ void k_set_offsets(uint32_t C, CT ct, const uint32_t *newoff) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < C && ct.alive[s]) ct.moff[s] = newoff[s];
}

// output gather: per final clump member (particles order): tree index -> pos/vel/orig,
// and the number of offset sources (sink particles expand)
__global__ void k_out_counts(const uint32_t *list, uint32_t nl, const uint32_t *base, CT ct, Pool P, const uint32_t *sink_n,
                             uint32_t *ocnt) {
    uint32_t t = blockIdx.x;
    if (t >= nl) return;
    uint32_t s = list[t];
    for (uint32_t k = threadIdx.x; k < ct.mn[s]; k += blockDim.x) ocnt[base[t] + k] = sink_n[P.idx[ct.moff[s] + k]];
}

__global__ void k_out_fill(const uint32_t *list, uint32_t nl, const uint32_t *base, CT ct, Pool P, const double4_32a *pos, const double4_32a *vel,
                           const uint32_t *orig, const uint32_t *sink_n, const uint32_t *sink_first, const uint32_t *sorted_src,
                           const double4_32a *in_pos, const uint32_t *obase, double *mpos, double *mvel, double *mmass, uint32_t *morig,
                           double *opos) {
    uint32_t t = blockIdx.x;
    if (t >= nl) return;
    uint32_t s = list[t];
    for (uint32_t k = threadIdx.x; k < ct.mn[s]; k += blockDim.x) {
        uint32_t i = P.idx[ct.moff[s] + k];
        size_t g = base[t] + k;
        double4_32a p = pos[i], v = vel[i];
        mpos[3 * g] = p.x; mpos[3 * g + 1] = p.y; mpos[3 * g + 2] = p.z;
        mvel[3 * g] = v.x; mvel[3 * g + 1] = v.y; mvel[3 * g + 2] = v.z;
        mmass[g] = p.w;
        morig[g] = orig[i];
        uint32_t ob = obase[g], n = sink_n[i];
        if (n <= 1) {
            opos[3 * (size_t)ob] = p.x; opos[3 * (size_t)ob + 1] = p.y; opos[3 * (size_t)ob + 2] = p.z;
        } else {
            for (uint32_t j = 0; j < n; ++j) {
                double4_32a q = in_pos[sorted_src[sink_first[i] + j]];
                opos[3 * (size_t)(ob + j)] = q.x; opos[3 * (size_t)(ob + j) + 1] = q.y; opos[3 * (size_t)(ob + j) + 2] = q.z;
            }
        }
    }
}

}  // namespace

// ====================================================================== host orchestration
namespace {

struct Stage {
    Context &c;
    cudaStream_t s;
    CT ct;
    Pool P;
    CP cp;
    uint32_t C = 0;
    uint32_t *slot_of_key = nullptr;
    uint32_t *alt_idx = nullptr;  // second pool buffer for compaction
    double *alt_dist = nullptr;
    uint32_t *d_off = nullptr;
    uint32_t *d_list = nullptr;   // scratch slot list (capacity C)
    uint32_t *d_list2 = nullptr;
    uint8_t *d_flag8 = nullptr;
    uint8_t *d_tie = nullptr;  // per slot: the last member sort met a tie (k_sort_small, k_lib_order)
    uint32_t *d_u = nullptr;      // small device counters
    const DevTree &tr;

    Stage(Context &cc, cudaStream_t ss) : c(cc), s(ss), tr(cc.tree) {}

    int sync() {
        PLAN_CUDA(cudaStreamSynchronize(s));
        return kOk;
    }
    template <class T> int down(std::vector<T> &h, const T *d, size_t n) {
        h.resize(n);
        if (n) PLAN_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, s));
        return sync();
    }
    int up_list(const std::vector<uint32_t> &h, uint32_t *d) {
        if (!h.empty()) PLAN_CUDA(cudaMemcpyAsync(d, h.data(), h.size() * 4, cudaMemcpyHostToDevice, s));
        return kOk;
    }
    // alive slots in key order
    int live_order(std::vector<uint32_t> &order, bool need_mask = false) {
        std::vector<uint32_t> key;
        std::vector<uint8_t> alive, mask;
        int rc = down(key, ct.key, C);
        if (!rc) rc = down(alive, ct.alive, C);
        if (!rc && need_mask) rc = down(mask, ct.mask, C);
        if (rc) return rc;
        order.clear();
        for (uint32_t i = 0; i < C; ++i)
            if (alive[i] && (!need_mask || mask[i])) order.push_back(i);
        std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
        return kOk;
    }

    int kinematics(const std::vector<uint32_t> &list, bool with_hill = false) {
        if (list.empty()) return kOk;
        int rc = up_list(list, d_list);
        if (rc) return rc;
        k_kinematics<<<(unsigned)((list.size() + 3) / 4), 128, 0, s>>>(d_list, (uint32_t)list.size(), ct, P, tr.pos, tr.vel, with_hill ? 1 : 0,
                                                                        cp.G, cp.Omega);
        k_kinematics_big<<<(unsigned)list.size(), 256, 0, s>>>(d_list, ct, P, tr.pos, tr.vel, with_hill ? 1 : 0, cp.G, cp.Omega);
        c.launches += 2;
        PLAN_CUDA(cudaGetLastError());
        return kOk;
    }

    // distances, sort, radii for the listed clumps (the tail of SortParticles / Merge)
    // known_mn: sizes of the listed clumps when the caller has them (saves a download)
    int resort(const std::vector<uint32_t> &list, bool radii = true, const std::vector<uint32_t> *known_mn = nullptr) {
        if (list.empty()) return kOk;
        int rc = up_list(list, d_list);
        if (rc) return rc;
        const uint32_t n = (uint32_t)list.size();
        std::vector<uint32_t> mn_all, mn_list;
        if (known_mn) {
            mn_list = *known_mn;
        } else {
            rc = down(mn_all, ct.mn, C);
            if (rc) return rc;
            for (uint32_t sl : list) mn_list.push_back(mn_all[sl]);
        }
        uint32_t mx = 0;
        for (uint32_t v : mn_list) mx = std::max(mx, v);
        const unsigned ny = std::min(64u, std::max(1u, (mx + 8191) / 8192));
        k_dist<<<dim3(n, ny), 256, 0, s>>>(d_list, ct, P, tr.pos);
        k_sort_small<<<n, 1024, 0, s>>>(d_list, ct, P, d_tie);
        c.launches += 2;
        // segments longer than the in-block sort go through the radix sort
        std::vector<uint32_t> large, base;
        uint64_t tot = 0;
        for (size_t k = 0; k < list.size(); ++k)
            if (mn_list[k] > (uint32_t)kSmallSort) { large.push_back(list[k]); base.push_back((uint32_t)tot); tot += mn_list[k]; }
        if (!large.empty()) {
            Arena &S = c.scratch;
            size_t mark = S.used;
            uint32_t *w0 = S.get<uint32_t>(tot), *w1 = S.get<uint32_t>(tot), *w2 = S.get<uint32_t>(tot), *pay = S.get<uint32_t>(tot);
            uint32_t *dl = S.get<uint32_t>(large.size()), *db = S.get<uint32_t>(large.size());
            size_t sb = radix_sort96_scratch_bytes(tot);
            void *scr = S.take(sb);
            if (S.failed || !scr) { S.used = mark; return kErrOutOfMemory; }
            PLAN_CUDA(cudaMemcpyAsync(dl, large.data(), large.size() * 4, cudaMemcpyHostToDevice, s));
            PLAN_CUDA(cudaMemcpyAsync(db, base.data(), base.size() * 4, cudaMemcpyHostToDevice, s));
            k_large_gather<<<(unsigned)large.size(), 256, 0, s>>>(dl, (uint32_t)large.size(), db, ct, P, w0, w1, w2, pay);
            rc = radix_sort96(w0, w1, w2, pay, tot, scr, sb, s);
            if (rc) { S.used = mark; return rc; }
            k_large_scatter<<<(unsigned)large.size(), 256, 0, s>>>(dl, (uint32_t)large.size(), db, ct, P, w0, w1, pay, d_tie);
            c.launches += 2 + 36;
            PLAN_CUDA(cudaGetLastError());
            rc = sync();
            S.used = mark;
            if (rc) return rc;
            rc = up_list(list, d_list);
            if (rc) return rc;
        }
        k_lib_order<<<(n + 63) / 64, 64, 0, s>>>(d_list, n, ct, P, d_tie);
        c.launches++;
        if (radii) {
            k_one10th<<<n, 256, 0, s>>>(d_list, ct, P, tr.pos, tr.dens);
            c.launches++;
        }
        PLAN_CUDA(cudaGetLastError());
        return kOk;
    }

    // SortParticles; the one-tenth radii are only read by the merge sweeps, and with_hill
    // folds the CalculateHillRadius that follows every later SortParticles into the sums
    int sort_particles(const std::vector<uint32_t> &list, bool radii = true, bool with_hill = false,
                       const std::vector<uint32_t> *known_mn = nullptr) {
        int rc = kinematics(list, with_hill);
        if (!rc) rc = resort(list, radii, known_mn);
        return rc;
    }

    int dispersion(const std::vector<uint32_t> &list, double tol, std::vector<uint8_t> &res) {
        res.clear();
        if (list.empty()) return kOk;
        int rc = up_list(list, d_list);
        if (rc) return rc;
        k_dispersion<<<(unsigned)((list.size() + 3) / 4), 128, 0, s>>>(d_list, (uint32_t)list.size(), ct, P, tol, d_flag8);
        c.launches++;
        return down(res, d_flag8, list.size());
    }

    int hill(const std::vector<uint32_t> &list) {
        if (list.empty()) return kOk;
        int rc = up_list(list, d_list);
        if (rc) return rc;
        k_hill<<<grid_for(list.size(), 128), 128, 0, s>>>(d_list, (uint32_t)list.size(), ct, cp.G, cp.Omega);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        return kOk;
    }

    // Pack the live segments into the other buffer once the bump allocator has used half
    // of the pool (merges and rebinding write fresh segments and abandon the old ones).
    int maybe_compact(bool force = false) {
        uint32_t top = 0;
        PLAN_CUDA(cudaMemcpyAsync(&top, P.top, 4, cudaMemcpyDeviceToHost, s));
        int rc = sync();
        if (rc) return rc;
        if (!force && top < P.cap / 2) return kOk;
        std::vector<uint32_t> mn;
        std::vector<uint8_t> alive;
        rc = down(mn, ct.mn, C);
        if (!rc) rc = down(alive, ct.alive, C);
        if (rc) return rc;
        std::vector<uint32_t> off(C + 1, 0);
        uint64_t run = 0;
        for (uint32_t i = 0; i < C; ++i) { off[i] = (uint32_t)run; if (alive[i]) run += mn[i]; }
        if (run > P.cap) return kErrDeviceLimit;
        PLAN_CUDA(cudaMemcpyAsync(d_off, off.data(), (size_t)C * 4, cudaMemcpyHostToDevice, s));
        k_compact<<<C, 256, 0, s>>>(C, ct, P, d_off, alt_idx, alt_dist);
        k_set_offsets<<<grid_for(C, 256), 256, 0, s>>>(C, ct, d_off);
        c.launches += 2;
        std::swap(P.idx, alt_idx);
        std::swap(P.dist, alt_dist);
        uint32_t t32 = (uint32_t)run;
        PLAN_CUDA(cudaMemcpyAsync(P.top, &t32, 4, cudaMemcpyHostToDevice, s));
        ++compactions;
        return sync();
    }
    uint32_t compactions = 0;

    int unbind(const std::vector<uint32_t> &list) {
        if (list.empty()) return kOk;
        int rc = up_list(list, d_list);
        if (rc) return rc;
        k_unbind<<<(unsigned)list.size(), 256, 0, s>>>(d_list, ct, P, tr.pos, tr.vel, cp);
        c.launches++;
        PLAN_CUDA(cudaGetLastError());
        // RemoveUnboundParticles ends with SortParticles; every caller computes the Hill
        // radius right after it (src/tree.hpp:4190-4191, 4241-4242)
        return sort_particles(list, false, true);
    }
};

}  // namespace

static double wall_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// PLAN_TRACE=1 in the environment prints the progress of FindPlanetesimals to stderr (the
// stream is synchronised at every mark, so traced runs are slower; off by default).
struct Trace {
    bool on = false, fine_on = false;  // PLAN_TRACE=1: stages; 2: also the steps inside a merge sweep
    cudaStream_t s = nullptr;
    double t0 = 0, last = 0;
    Trace(cudaStream_t st) : s(st) {
        const char *e = std::getenv("PLAN_TRACE");
        on = e && *e && *e != '0';
        fine_on = on && *e == '2';
        t0 = last = wall_ms();
    }
    void fine(const char *what, long long a = -1, long long b = -1) {
        if (fine_on) mark(what, a, b);
    }
    void mark(const char *what, long long a = -1, long long b = -1, long long c = -1, long long d = -1) {
        if (!on) return;
        cudaStreamSynchronize(s);
        double t = wall_ms();
        std::fprintf(stderr, "[plan] %10.1f ms  +%9.1f ms  %s", t - t0, t - last, what);
        if (a >= 0) std::fprintf(stderr, " %lld", a);
        if (b >= 0) std::fprintf(stderr, " %lld", b);
        if (c >= 0) std::fprintf(stderr, " %lld", c);
        if (d >= 0) std::fprintf(stderr, " %lld", d);
        std::fprintf(stderr, "\n");
        last = t;
    }
};

int find_planetesimals(Context &c, plan_params &p, cudaStream_t s, plan_catalogue **out) {
    cudaEvent_t ev[6];
    for (auto &e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], s);
    Trace trace(s);
    c.counters[27] = 0;  // saddle queries of the merge sweeps left to the exact heap path (ties)
    const DevTree &tr = c.tree;
    const uint32_t Tu = tr.Tu, N = c.n_input;
    // kernel choice and thresholds (src/tree.hpp:3576-3660), host scalars
    uint32_t horiz = p.box_resolution[0] * p.box_resolution[1];
    if (tr.box.half_width < p.max_half_width + p.max_ghost_zone_width - 1e-16)
        horiz = (uint32_t)std::pow(tr.box.half_width / p.cell_length[0] * ((tr.box.half_width - p.max_ghost_zone_width) / tr.box.half_width), 2.0);
    // at least 4 particles per horizontal cell: median-sphere density; otherwise the spline
    // kernel, and groups are pruned right after HOP (src/tree.hpp:3583-3610, 3834-3836)
    const bool median = N >= 4 * horiz;
    if (median && !p.fixed_hop && N >= 1.67e7) p.hop = 64;
    const double PI = 3.14159265358979323846;
    double thr = std::pow(p.Omega, 2.) / PI / p.grav_constant * 2.;
    if (p.mass_total_code_units / N / p.cell_volume > thr / 4) thr *= 9. / 8.;
    double rmin = std::min(std::min((double)p.box_resolution[0] / p.box_length[0], (double)p.box_resolution[1] / p.box_length[1]),
                           (double)p.box_resolution[2] / p.box_length[2]);
    unsigned hydro = (unsigned)rmin;
    double diffuse = 0.55, hillf = 0.25;
    if (hydro <= 1024) { diffuse = 0.35; hillf = 0.75; }
    else if (hydro <= 1536) { diffuse = 0.4; hillf = 0.5; }
    else if (hydro <= 2048) { diffuse = 0.5; hillf = 0.35; }
    if (p.clump_diffuse_threshold > 0) diffuse = p.clump_diffuse_threshold;
    if (p.Hill_fraction_for_merge > 0) hillf = p.Hill_fraction_for_merge;
    if (p.knn < 1 || p.knn > 128 || p.hop < 1 || p.hop > 128 || p.knn > Tu || p.hop > Tu) {
        c.last_error = "knn and hop must lie in [1, 128] and not exceed the number of tree points";
        return kErrUnsupported;
    }
    c.fs = FindScalars{thr, 3 * thr, p.min_trusted_mass, diffuse, hillf, p.knn, p.hop, median ? 1 : 0,
                       spline_cells(p.cell_length, p.cell_volume)};

    // 1-2. densities and densest neighbours
    int rc = launch_density(c, p, p.knn, s);
    if (rc) return rc;
    cudaEventRecord(ev[1], s);
    uint32_t *densest = c.arena.get<uint32_t>(Tu);
    if (!densest) return kErrOutOfMemory;
    c.densest = densest;
    trace.mark("density", c.counters[17]);
    rc = launch_densest(c, p, p.hop, thr, densest, s);
    if (rc) return rc;
    cudaEventRecord(ev[2], s);
    trace.mark("densest", c.counters[18]);
    // 3. HOP groups
    HopGroups hg;
    rc = hop_groups(c, densest, thr, hg, s);
    if (rc) return rc;
    c.peak = hg.peak;
    cudaEventRecord(ev[3], s);
    trace.mark("hop groups", hg.n_groups, hg.n_members);

    // ------------------------------------------------------------------ clump stage
    Stage st(c, s);
    const uint32_t C = hg.n_groups;
    st.C = C;
    Arena &A = c.arena;
    CT &ct = st.ct;
    ct.C = C;
    ct.key = A.get<uint32_t>(C + 1); ct.peak = A.get<uint32_t>(C + 1);
    ct.mask = A.get<uint8_t>(C + 1); ct.alive = A.get<uint8_t>(C + 1);
    ct.M = A.get<double>(C + 1);
    ct.com = A.get<double4_32a>(C + 1); ct.vcom = A.get<double4_32a>(C + 1); ct.J = A.get<double4_32a>(C + 1);
    ct.r_in = A.get<double>(C + 1); ct.r_out = A.get<double>(C + 1); ct.r10 = A.get<double>(C + 1);
    ct.r2s = A.get<double>(C + 1); ct.hill = A.get<double>(C + 1);
    ct.moff = A.get<uint32_t>(C + 1); ct.mn = A.get<uint32_t>(C + 1);
    ct.sub_head = A.get<uint32_t>(C + 1); ct.sub_tail = A.get<uint32_t>(C + 1);
    Pool &P = st.P;
    const uint32_t m0 = hg.n_members;
    {
        // the member pool: generous (40 x the HOP members + 6 x the tree points) where the
        // arena has room, keeping ~256 B per tree point for what the clump stage allocates
        // after it; never below the former 6 x members + tree points
        const uint64_t want = 40ull * m0 + 6ull * Tu + 4096, floor_cap = 6ull * m0 + Tu + 4096;
        const uint64_t used = (A.used + 255) & ~uint64_t(255), reserve = 256ull * Tu + (64ull << 20);
        const uint64_t room = A.cap > used + reserve ? (A.cap - used - reserve) / 24 : 0;
        P.cap = (uint32_t)std::min<uint64_t>(0xfffffff0ull, std::max(floor_cap, std::min(want, room)));
    }
    P.idx = A.get<uint32_t>(P.cap);
    P.dist = A.get<double>(P.cap);
    st.alt_idx = A.get<uint32_t>(P.cap);
    st.alt_dist = A.get<double>(P.cap);
    st.d_off = A.get<uint32_t>(C + 1);
    P.top = A.get<uint32_t>(4);
    P.sub_cap = C + 16;
    P.sub_peak = A.get<uint32_t>(P.sub_cap);
    P.sub_next = A.get<uint32_t>(P.sub_cap);
    P.sub_top = A.get<uint32_t>(4);
    st.slot_of_key = A.get<uint32_t>(Tu);
    st.d_list = A.get<uint32_t>(C + 1);
    st.d_list2 = A.get<uint32_t>(C + 1);
    st.d_flag8 = A.get<uint8_t>(C + 1);
    st.d_tie = A.get<uint8_t>(C + 1);
    st.d_u = A.get<uint32_t>(64);
    uint8_t *in_clump = A.get<uint8_t>(Tu);
    if (A.failed) return kErrOutOfMemory;
    st.cp = CP{p.grav_constant, p.q * p.Omega, p.Omega, thr, 3 * thr, p.min_trusted_mass, diffuse, hillf, p.knn, Tu};
    PLAN_CUDA(cudaMemsetAsync(st.slot_of_key, 0xff, (size_t)Tu * 4, s));
    PLAN_CUDA(cudaMemsetAsync(st.d_u, 0, 64 * 4, s));
    PLAN_CUDA(cudaMemsetAsync(P.sub_top, 0, 4, s));
    PLAN_CUDA(cudaMemcpyAsync(P.idx, hg.members, (size_t)m0 * 4, cudaMemcpyDeviceToDevice, s));
    PLAN_CUDA(cudaMemcpyAsync(P.top, &m0, 4, cudaMemcpyHostToDevice, s));
    if (C) {
        k_init<<<grid_for(C, 256), 256, 0, s>>>(C, hg.key, hg.off, ct, st.slot_of_key);
        c.launches++;
    }
    c.counters[5] = m0;
    c.counters[6] = C;
    PLAN_CUDA(cudaStreamSynchronize(s));
    double tw0 = wall_ms();
    for (int k = 15; k < 32; ++k)
        if (k != 20 && k != 21) c.stage_ms[k] = 0;  // 20, 21: the density kernels, timed before
    std::vector<uint32_t> all(C);
    std::iota(all.begin(), all.end(), 0u);
    // SortParticles + the diffuse cut after HOP (src/tree.hpp:3816-3829)
    rc = st.sort_particles(all);
    if (rc) return rc;
    trace.mark("sort particles of all groups", C);
    std::vector<uint8_t> too;
    std::vector<uint32_t> del_keys_host;
    if (diffuse < 0.525) {
        rc = st.dispersion(all, diffuse, too);
        if (rc) return rc;
        std::vector<uint8_t> alive(C, 1);
        for (uint32_t i = 0; i < C; ++i) if (too[i]) alive[i] = 0;
        PLAN_CUDA(cudaMemcpyAsync(ct.alive, alive.data(), C, cudaMemcpyHostToDevice, s));
    }
    if (!median && C) {  // RemoveSmallMassAndLowPeak (src/tree.hpp:3834-3836)
        k_prune<<<grid_for(C, 128), 128, 0, s>>>(C, ct, P, tr.vel, tr.dens, st.cp, st.d_flag8);
        c.launches++;
        std::vector<uint8_t> kill, alive;
        rc = st.down(kill, st.d_flag8, C);
        if (!rc) rc = st.down(alive, ct.alive, C);
        if (rc) return rc;
        for (uint32_t i = 0; i < C; ++i) if (kill[i]) alive[i] = 0;
        PLAN_CUDA(cudaMemcpyAsync(ct.alive, alive.data(), C, cudaMemcpyHostToDevice, s));
        trace.mark("small-mass and low-peak groups removed");
    }
    std::vector<uint32_t> live;
    rc = st.live_order(live);
    if (rc) return rc;
    uint32_t num_planetesimals = (uint32_t)live.size();

    // 4. merge sweeps (src/tree.hpp:3863-4152)
    uint32_t *d_cnt = A.get<uint32_t>(C + 1), *d_off = A.get<uint32_t>(C + 1);
    uint32_t *d_rank = A.get<uint32_t>(C + 1), *d_ctslot = A.get<uint32_t>(C + 1);
    uint32_t *d_pairs = A.get<uint32_t>(2 * (size_t)C + 2), *d_del = A.get<uint32_t>(2 * (size_t)C + 2);
    uint32_t *d_wave = A.get<uint32_t>(C + 1), *d_pl = A.get<uint32_t>(C + 1), *d_pf = A.get<uint32_t>(C + 1);
    uint32_t *d_pc = A.get<uint32_t>(C + 1), *d_pw = A.get<uint32_t>(C + 1), *d_merged = A.get<uint32_t>(C + 1);
    double4_32a *ct_pos = A.get<double4_32a>(C + 1), *ct_vel = A.get<double4_32a>(C + 1);
    double *d_maxr = A.get<double>(2);
    if (A.failed) return kErrOutOfMemory;
    const size_t arena_mark = A.used;
    uint32_t nunknown_total = 0, quirk = 0;
    for (int kind = 0; kind < 2 && C; ++kind) {
        const bool hill_mode = kind == 1;
        if (hill_mode) {
            rc = st.hill(live);
            if (rc) return rc;
            trace.fine("  Hill radii (clumps)", (long long)live.size());
        }
        double max_radius = 0.;
        const uint32_t start_num = num_planetesimals;
        uint32_t delete_count = 0;
        PLAN_CUDA(cudaMemsetAsync(st.d_u, 0, 64 * 4, s));  // [0] ndel, [1] npairs, [2] nunknown, ...
        bool merged_any = true;
        for (int sweep = 0; merged_any && sweep < 100000; ++sweep) {
            A.used = arena_mark;  // per-sweep buffers (clump tree, candidates) are rebuilt
            // BuildClumpTree over live clumps in key order (src/tree.hpp:5251-5284)
            k_mark_live<<<grid_for(C, 256), 256, 0, s>>>(C, ct, d_cnt);
            uint32_t *d_tot = st.d_u + 8;
            size_t sb = scan_u32_scratch_bytes(C + 1);
            const size_t smark = c.scratch.used;
            void *scr = c.scratch.take(sb);
            if (!scr) return kErrOutOfMemory;
            rc = scan_u32(d_cnt, d_rank, C, d_tot, scr, sb, s);
            c.scratch.used = smark;
            if (rc) return rc;
            k_ct_points<<<grid_for(C, 256), 256, 0, s>>>(C, ct, d_cnt, d_rank, p.mass_per_particle[0], ct_pos, ct_vel, d_ctslot);
            k_max_radius<<<1, 1024, 0, s>>>(C, ct, hill_mode, hillf, d_maxr);
            c.launches += 3;
            uint32_t nct = 0;
            double mr = 0;
            PLAN_CUDA(cudaMemcpyAsync(&nct, d_tot, 4, cudaMemcpyDeviceToHost, s));
            PLAN_CUDA(cudaMemcpyAsync(&mr, d_maxr, 8, cudaMemcpyDeviceToHost, s));
            rc = st.sync();
            if (rc) return rc;
            if (nct != num_planetesimals) ++quirk;  // the reference sizes the clump set by this count
            max_radius = std::max(mr, max_radius);
            DevTree ctree;
            if (nct) {
                TreeBox box = make_box(tr.box.root_center, tr.box.half_width);
                rc = build_octree(c, ct_pos, ct_vel, nullptr, nct, box, p.mass_per_particle, 1, ctree, s, nullptr);
                if (rc) return rc;
            }
            KTree kct = ktree_of(ctree);
            trace.fine("  clump tree (clumps)", nct);
            // candidates
            uint32_t ncand = 0;
            if (nct) {
                k_ball_clumps<<<grid_for(C, 128), 128, 0, s>>>(0, C, ct, kct, hill_mode, hillf, max_radius, d_cnt, nullptr, nullptr, c.d_err);
                const size_t sm2 = c.scratch.used;
                void *scr2 = c.scratch.take(sb);
                rc = scan_u32(d_cnt, d_off, C, d_tot, scr2, sb, s);
                c.scratch.used = sm2;
                if (rc) return rc;
                PLAN_CUDA(cudaMemcpyAsync(&ncand, d_tot, 4, cudaMemcpyDeviceToHost, s));
                rc = st.sync();
                if (rc) return rc;
                c.launches++;
            }
            uint32_t *d_cand = A.get<uint32_t>(ncand + 1), *d_cp1 = A.get<uint32_t>(ncand + 1), *d_p2 = A.get<uint32_t>(ncand + 1);
            uint8_t *d_code = A.get<uint8_t>(ncand + 1);
            double *d_sq = A.get<double>(3 * (size_t)ncand + 3), *d_sest = A.get<double>(ncand + 1), *d_sden = A.get<double>(ncand + 1);
            uint32_t *d_sof = A.get<uint32_t>(ncand + 1);
            uint32_t *d_rfl = A.get<uint32_t>(ncand + 1), *d_rpos = A.get<uint32_t>(ncand + 1), *d_rlist = A.get<uint32_t>(ncand + 1);
            uint32_t *d_nrl = st.d_u + 12;  // candidates the resolution acts on
            if (A.failed) return kErrOutOfMemory;
            PLAN_CUDA(cudaMemsetAsync(d_nrl, 0, 4, s));
            uint32_t nsaddle = 0;
            if (ncand) {
                k_ball_clumps<<<grid_for(C, 128), 128, 0, s>>>(1, C, ct, kct, hill_mode, hillf, max_radius, d_cnt, d_off, d_cand, c.d_err);
                k_cand_owner<<<grid_for(C, 256), 256, 0, s>>>(C, d_cnt, d_off, d_cp1);
                PLAN_CUDA(cudaMemsetAsync(st.d_u + 16, 0, 4, s));
                k_pair_eval<<<grid_for(ncand, 128), 128, 0, s>>>(ncand, d_cp1, d_cand, ctree.vel, ct, st.slot_of_key, st.cp, hill_mode,
                                                                 d_code, d_p2, d_sq, d_sest, d_sof, st.d_u + 16);
                PLAN_CUDA(cudaMemcpyAsync(&nsaddle, st.d_u + 16, 4, cudaMemcpyDeviceToHost, s));
                rc = st.sync();
                if (rc) return rc;
                c.launches += 3;
                if (nsaddle) {
                    rc = launch_density_at(c, d_sq, d_sest, nsaddle, p.knn, d_sden, s);
                    if (rc) return rc;
                    k_saddle_apply<<<grid_for(nsaddle, 128), 128, 0, s>>>(nsaddle, d_sof, d_sden, 2.5 * thr, d_code);
                    c.launches++;
                }
                k_flag_resolve<<<grid_for(ncand, 256), 256, 0, s>>>(ncand, d_code, d_rfl);
                const size_t sb3 = scan_u32_scratch_bytes(ncand + 1), sm3 = c.scratch.used;
                void *scr3 = c.scratch.take(sb3);
                if (!scr3) return kErrOutOfMemory;
                rc = scan_u32(d_rfl, d_rpos, ncand, d_nrl, scr3, sb3, s);
                c.scratch.used = sm3;
                if (rc) return rc;
                k_scatter_flagged<<<grid_for(ncand, 256), 256, 0, s>>>(ncand, d_rfl, d_rpos, d_rlist);
                c.launches += 4;
            }
            trace.fine("  candidate pairs evaluated (candidates, saddles)", ncand, nsaddle);
            trace.fine("  saddle queries with distance ties so far", (long long)c.counters[27]);
            // serial resolution
            PLAN_CUDA(cudaMemsetAsync(st.d_u + 1, 0, 4, s));
            k_resolve<<<1, 32, 0, s>>>(d_rlist, d_nrl, d_cp1, ct, d_code, d_p2, d_pairs, st.d_u + 1, d_del, st.d_u + 0, st.d_u + 2);
            c.launches++;
            uint32_t h_u[3];
            PLAN_CUDA(cudaMemcpyAsync(h_u, st.d_u, 12, cudaMemcpyDeviceToHost, s));
            rc = st.sync();
            if (rc) return rc;
            const uint32_t npairs = h_u[1];
            delete_count = h_u[0];
            if (std::getenv("PLAN_DEBUG_MERGES") && npairs) {
                std::vector<uint32_t> hp, hk;
                rc = st.down(hp, d_pairs, 2 * (size_t)npairs);
                if (!rc) rc = st.down(hk, ct.key, C);
                if (rc) return rc;
                for (uint32_t k = 0; k < npairs; ++k) std::fprintf(stderr, "merge kind %d pred %u prey %u\n", kind, hk[hp[2 * k]], hk[hp[2 * k + 1]]);
            }
            merged_any = npairs > 0;
            trace.fine("  resolved (pairs)", npairs);
            if (npairs) {
                PLAN_CUDA(cudaMemsetAsync(d_wave, 0xff, (size_t)(C + 1) * 4, s));
                k_waves<<<1, 1, 0, s>>>(npairs, d_pairs, C, d_wave, d_pl, d_pf, d_pc, d_pw, st.d_u + 20, st.d_u + 21);
                uint32_t hw[2];
                PLAN_CUDA(cudaMemcpyAsync(hw, st.d_u + 20, 8, cudaMemcpyDeviceToHost, s));
                rc = st.sync();
                if (rc) return rc;
                c.launches++;
                const uint32_t npred = hw[0], nwaves = hw[1];
                for (uint32_t w = 0; w < nwaves; ++w) {
                    rc = st.maybe_compact();
                    if (rc) return rc;
                    PLAN_CUDA(cudaMemsetAsync(st.d_u + 24, 0, 4, s));
                    k_merge<<<npred, 256, 0, s>>>(npred, d_pl, d_pf, d_pc, d_pw, w, d_pairs, ct, P, tr.dens, d_merged, st.d_u + 24, c.d_err);
                    c.launches++;
                    std::vector<uint32_t> nm;
                    rc = st.down(nm, st.d_u + 24, 1);
                    if (rc) return rc;
                    std::vector<uint32_t> merged;
                    rc = st.down(merged, d_merged, nm[0]);
                    if (rc) return rc;
                    rc = st.resort(merged);
                    if (rc) return rc;
                    if (hill_mode) {
                        rc = st.hill(merged);
                        if (rc) return rc;
                    }
                }
            }
            trace.fine("  merged");
            // post-sweep diffuse test with the default tolerance (src/tree.hpp:3984-3992)
            std::vector<uint32_t> masked;
            rc = st.live_order(masked, true);
            if (rc) return rc;
            rc = st.dispersion(masked, 0.55, too);
            if (rc) return rc;
            std::vector<uint8_t> mask_now;
            rc = st.down(mask_now, ct.mask, C);
            if (rc) return rc;
            std::vector<uint32_t> keys_now;
            rc = st.down(keys_now, ct.key, C);
            if (rc) return rc;
            std::vector<uint32_t> extra_del;
            for (size_t k = 0; k < masked.size(); ++k)
                if (too[k]) { mask_now[masked[k]] = 0; extra_del.push_back(keys_now[masked[k]]); }
            if (!extra_del.empty()) {
                PLAN_CUDA(cudaMemcpyAsync(ct.mask, mask_now.data(), C, cudaMemcpyHostToDevice, s));
                PLAN_CUDA(cudaMemcpyAsync(d_del + delete_count, extra_del.data(), extra_del.size() * 4, cudaMemcpyHostToDevice, s));
                delete_count += (uint32_t)extra_del.size();
                PLAN_CUDA(cudaMemcpyAsync(st.d_u + 0, &delete_count, 4, cudaMemcpyHostToDevice, s));
            }
            num_planetesimals = (uint32_t)live.size() - delete_count;
            (hill_mode ? c.counters[12] : c.counters[11])++;
            trace.mark(hill_mode ? "hill merge sweep (sweep, pairs, deleted)" : "merge sweep (sweep, pairs, deleted)", sweep, npairs,
                       delete_count);
            rc = st.maybe_compact();
            if (rc) return rc;
        }
        // erase the deleted clumps (and a clump keyed 0 when the zero-filled list has room,
        // src/tree.hpp:3874, 4000-4002)
        std::vector<uint32_t> dk;
        rc = st.down(dk, d_del, delete_count);
        if (rc) return rc;
        std::vector<uint8_t> alive;
        rc = st.down(alive, ct.alive, C);
        if (rc) return rc;
        std::vector<uint32_t> keys_now;
        rc = st.down(keys_now, ct.key, C);
        if (rc) return rc;
        std::vector<uint32_t> sok(Tu, kNone);
        for (uint32_t i = 0; i < C; ++i) if (alive[i]) sok[keys_now[i]] = i;
        for (uint32_t k : dk) if (sok[k] != kNone) { alive[sok[k]] = 0; }
        if (delete_count < start_num && sok[0] != kNone && alive[sok[0]]) { alive[sok[0]] = 0; ++quirk; }
        std::vector<uint32_t> sok_dev(Tu, kNone);
        for (uint32_t i = 0; i < C; ++i) if (alive[i]) sok_dev[keys_now[i]] = i;
        PLAN_CUDA(cudaMemcpyAsync(ct.alive, alive.data(), C, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(st.slot_of_key, sok_dev.data(), (size_t)Tu * 4, cudaMemcpyHostToDevice, s));
        rc = st.live_order(live);
        if (rc) return rc;
        num_planetesimals = (uint32_t)live.size() + ((delete_count < start_num && quirk) ? 0 : 0);
        // all survivors are masked again by construction (every unmasked clump was deleted)
    }
    A.used = arena_mark;
    double tw1 = wall_ms();
    c.counters[13] = quirk;
    c.counters[14] = nunknown_total;
    cudaEventRecord(ev[4], s);

    // re-key (src/tree.hpp:4156-4182)
    if (std::getenv("PLAN_DEBUG_MERGES")) {
        std::vector<uint32_t> hk, hpk, hh, hsp, hsn;
        rc = st.down(hk, ct.key, C);
        if (!rc) rc = st.down(hpk, ct.peak, C);
        if (!rc) rc = st.down(hh, ct.sub_head, C);
        if (!rc) rc = st.down(hsp, P.sub_peak, P.sub_cap);
        if (!rc) rc = st.down(hsn, P.sub_next, P.sub_cap);
        if (rc) return rc;
        for (uint32_t sl : live) {
            std::fprintf(stderr, "clump %u peak %u subs", hk[sl], hpk[sl]);
            for (uint32_t e = hh[sl]; e != kNone; e = hsn[e]) std::fprintf(stderr, " %u", hsp[e]);
            std::fprintf(stderr, "\n");
        }
    }
    if (!live.empty()) {
        int rc2 = st.up_list(live, st.d_list2);
        if (rc2) return rc2;
        k_rekey<<<1, 1, 0, s>>>(C, ct, st.d_list2, (uint32_t)live.size(), P, tr.dens, st.slot_of_key, st.d_u + 30);
        c.launches++;
        rc = st.live_order(live);
        if (rc) return rc;
    }
    // 5. unbind, mark, rebind (src/tree.hpp:4189-4208)
    trace.mark("re-key", live.size());
    rc = st.unbind(live);  // includes SortParticles and the Hill radius
    if (rc) return rc;
    trace.mark("unbind");
    PLAN_CUDA(cudaStreamSynchronize(s));
    double tw2 = wall_ms();
    PLAN_CUDA(cudaMemsetAsync(in_clump, 0, Tu, s));
    if (C) {
        k_mark_members<<<C, 256, 0, s>>>(C, ct, P, in_clump);
        c.launches++;
    }
    {
        // the call-independent candidate list E and its prefix counts
        uint32_t *epos = A.get<uint32_t>((size_t)Tu + 1), *E = A.get<uint32_t>((size_t)Tu + 1);
        if (A.failed) return kErrOutOfMemory;
        {
            Arena &S = c.scratch;
            size_t mark = S.used;
            size_t sb = scan_u32_scratch_bytes((size_t)Tu + 1);
            void *scr = S.take(sb);
            if (S.failed || !scr) { S.used = mark; return kErrOutOfMemory; }
            PLAN_CUDA(cudaMemsetAsync(epos + Tu, 0, 4, s));
            k_elig_flags<<<grid_for(Tu, 256), 256, 0, s>>>(Tu, in_clump, tr.dens, st.cp.thr, epos);
            rc = scan_u32(epos, epos, (size_t)Tu + 1, nullptr, scr, sb, s);
            S.used = mark;
            if (rc) return rc;
            k_elig_compact<<<grid_for(Tu, 256), 256, 0, s>>>(Tu, in_clump, tr.dens, st.cp.thr, epos, E);
            c.launches += 4;
            PLAN_CUDA(cudaGetLastError());
        }
        // Clumps rebind concurrently (one SearchBound call per clump per round) under the
        // ordered-claim rule of k_rebind_round; passes rerun invalid clumps from their saved
        // state until the result equals the reference's clump-by-clump run in key order.
        const size_t nb = (size_t)C + 1;
        double *bM = A.get<double>(nb), *bh = A.get<double>(nb), *bri = A.get<double>(nb), *bro = A.get<double>(nb);
        double *br10 = A.get<double>(nb), *br2 = A.get<double>(nb);
        double4_32a *bc = A.get<double4_32a>(nb), *bv = A.get<double4_32a>(nb);
        uint32_t *bo = A.get<uint32_t>(nb), *bn = A.get<uint32_t>(nb), *owner = A.get<uint32_t>(Tu);
        uint32_t *rank_of = A.get<uint32_t>(nb), *slot_of_rank = A.get<uint32_t>(nb), *dmax = A.get<uint32_t>(nb);
        uint32_t *dset = A.get<uint32_t>(nb * kDeferSlots);
        uint8_t *dover = A.get<uint8_t>(nb);
        uint8_t *d_grew = A.get<uint8_t>(nb), *invalid = A.get<uint8_t>(nb), *rerun_rank = A.get<uint8_t>(nb);
        uint32_t *d_mnout = A.get<uint32_t>(nb);
        unsigned long long *d_prof = trace.on ? A.get<unsigned long long>(8 * nb) : nullptr;
        unsigned long long *reach = A.get<unsigned long long>(nb);
        uint32_t *tent = A.get<uint32_t>(Tu);
        unsigned long long *mhash = A.get<unsigned long long>(nb);
        if (A.failed) return kErrOutOfMemory;
        const uint32_t nlive = (uint32_t)live.size();
        // save the state (the member pool is packed first, then copied aside)
        uint32_t saved_top = 0;
        uint32_t *bidx = nullptr;
        double *bdist = nullptr;
        if (nlive) {
            rc = st.maybe_compact(true);
            if (rc) return rc;
            auto cp8 = [&](void *dst, const void *src, size_t b) -> int {
                PLAN_CUDA(cudaMemcpyAsync(dst, src, b, cudaMemcpyDeviceToDevice, s));
                return kOk;
            };
            rc = cp8(bM, ct.M, C * 8) | cp8(bh, ct.hill, C * 8) | cp8(bri, ct.r_in, C * 8) | cp8(bro, ct.r_out, C * 8) |
                 cp8(br10, ct.r10, C * 8) | cp8(br2, ct.r2s, C * 8) | cp8(bc, ct.com, C * 32) | cp8(bv, ct.vcom, C * 32) |
                 cp8(bo, ct.moff, C * 4) | cp8(bn, ct.mn, C * 4);
            if (rc) return kErrDevice;
            PLAN_CUDA(cudaMemcpyAsync(&saved_top, P.top, 4, cudaMemcpyDeviceToHost, s));
            rc = st.sync();
            if (rc) return rc;
            bidx = A.get<uint32_t>(saved_top + 1);
            bdist = A.get<double>(saved_top + 1);
            if (A.failed) return kErrOutOfMemory;
            PLAN_CUDA(cudaMemcpyAsync(bidx, P.idx, (size_t)saved_top * 4, cudaMemcpyDeviceToDevice, s));
            PLAN_CUDA(cudaMemcpyAsync(bdist, P.dist, (size_t)saved_top * 8, cudaMemcpyDeviceToDevice, s));
        }
        std::vector<uint32_t> h_rank(C, kNone);
        for (uint32_t r = 0; r < nlive; ++r) h_rank[live[r]] = r;
        PLAN_CUDA(cudaMemcpyAsync(rank_of, h_rank.data(), (size_t)C * 4, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(slot_of_rank, live.data(), (size_t)nlive * 4, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemsetAsync(owner, 0xff, (size_t)Tu * 4, s));
        PLAN_CUDA(cudaMemsetAsync(invalid, 0, nb, s));
        PLAN_CUDA(cudaMemsetAsync(dmax, 0, nb * 4, s));
        PLAN_CUDA(cudaMemsetAsync(dset, 0xff, nb * kDeferSlots * 4, s));
        PLAN_CUDA(cudaMemsetAsync(dover, 0, nb, s));
        PLAN_CUDA(cudaMemsetAsync(reach, 0, nb * 8, s));
        PLAN_CUDA(cudaMemsetAsync(tent, 0xff, (size_t)Tu * 4, s));
        KTree kt = ktree_of(tr);
        const FTree ftr{tr.phi, tr.plo, tr.nhi, tr.nlo};
        if (!tr.phi) return kErrDevice;  // the FP32 copies are made by the density stage
        // speculative acceptance windows (exact by verification; PLAN_ACCEPT_SPECULATE=1)
        const char *spec_env = std::getenv("PLAN_ACCEPT_SPECULATE");
        const bool speculate = spec_env && *spec_env == '1';
        // the default loop with the reciprocal taken during the test (PLAN_ACCEPT_RCP=1)
        const char *rcp_env = std::getenv("PLAN_ACCEPT_RCP");
        const bool rcp = rcp_env && *rcp_env == '1';
        auto rebind_kernel = speculate ? k_rebind_round<1> : rcp ? k_rebind_round<2> : k_rebind_round<0>;
        uint64_t rounds = 0, passes = 0, reruns = 0;
        // Each clump's calls run on the device (k_rebind_loop), one launch per pass; the
        // round-by-round host loop (one launch and one host round trip per call) stays
        // available with PLAN_REBIND_ROUNDS=1 for comparison.
        const char *rounds_env = std::getenv("PLAN_REBIND_ROUNDS");
        const bool use_rounds = rounds_env && *rounds_env == '1';
        uint8_t *d_fin = A.get<uint8_t>(nb), *d_susp = A.get<uint8_t>(nb), *d_needsort = A.get<uint8_t>(nb), *d_distsq = A.get<uint8_t>(nb);
        uint32_t *d_head = A.get<uint32_t>(4), *d_blkoff = A.get<uint32_t>(nb + 1);
        unsigned long long *d_rstats = trace.on ? A.get<unsigned long long>((size_t)kRbStats * nb) : nullptr;
        double4_32a *tm0 = use_rounds ? nullptr : A.get<double4_32a>(Tu), *tm1 = use_rounds ? nullptr : A.get<double4_32a>(Tu);
        if (A.failed) return kErrOutOfMemory;
        int rb_grid = 1;
        if (!use_rounds) {
            k_member_terms<<<grid_for(Tu, 256), 256, 0, s>>>(Tu, tr.pos, tr.vel, tm0, tm1);
            c.launches++;
            PLAN_CUDA(cudaMemsetAsync(d_needsort, 0, nb, s));
            PLAN_CUDA(cudaMemsetAsync(d_distsq, 0, nb, s));
            PLAN_CUDA(cudaFuncSetAttribute(k_rebind_loop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRbSmem));
            int dev = 0, nsm = 0, per = 0;
            PLAN_CUDA(cudaGetDevice(&dev));
            PLAN_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
            PLAN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rebind_loop, kRB, kRbSmem));
            rb_grid = std::max(1, nsm * std::max(1, per));
        }
        // Checkpoints of the clumps' runs (loop path, PLAN_REBIND_CHECKPOINTS=1): tables by key
        // rank and a store for their member lists from what the arena has left; a rerun then
        // resumes from the last checkpoint before its first affected call. Off by default: the
        // kept calls may hold particles that an earlier clump rerunning in the same pass takes
        // in its new run, which costs another pass (measured: 1M snapshot 2 -> 3 passes, 16.7M
        // no better), where a rerun from the start would have waited for that clump.
        uint32_t *d_ccall = nullptr, *d_dcall = nullptr, *d_dfirst = nullptr, *d_lostck = nullptr, *d_keep = nullptr;
        Ckpt ck{};
        if (!use_rounds) {  // the calls of each run and of each deferral record: with or without checkpoints
            d_ccall = A.get<uint32_t>(nb);
            d_dcall = A.get<uint32_t>(nb * kDeferSlots);
            d_dfirst = A.get<uint32_t>(nb);
            if (A.failed) return kErrOutOfMemory;
            PLAN_CUDA(cudaMemsetAsync(d_ccall, 0, nb * 4, s));
            PLAN_CUDA(cudaMemsetAsync(d_dcall, 0xff, nb * kDeferSlots * 4, s));
            PLAN_CUDA(cudaMemsetAsync(d_dfirst, 0xff, nb * 4, s));
        }
        {
            const char *ck_env = std::getenv("PLAN_REBIND_CHECKPOINTS");
            if (!use_rounds && ck_env && *ck_env == '1') {
                const size_t nr = (size_t)nlive + 1;
                d_lostck = A.get<uint32_t>(nr);
                d_keep = A.get<uint32_t>(nb);
                ck.n = A.get<uint32_t>(nr);
                ck.call = A.get<uint32_t>(nr * kCk);
                ck.off = A.get<uint32_t>(nr * kCk);
                ck.m = A.get<uint32_t>(nr * kCk);
                ck.st = A.get<double>(nr * kCk * 8);
                ck.top = A.get<uint32_t>(4);
                if (A.failed) return kErrOutOfMemory;
                const uint64_t used = (A.used + 255) & ~uint64_t(255), margin = 64ull * Tu + (256ull << 20);
                const uint64_t ent = std::min<uint64_t>({A.cap > used + margin ? (A.cap - used - margin) / 12 : 0, 16ull * Tu, 0xfffffff0ull});
                if (ent >= 4096) {
                    ck.cap = (uint32_t)ent;
                    ck.idx = A.get<uint32_t>(ent);
                    ck.dist = A.get<double>(ent);
                    if (A.failed) return kErrOutOfMemory;
                    PLAN_CUDA(cudaMemsetAsync(ck.n, 0, nr * 4, s));
                    PLAN_CUDA(cudaMemsetAsync(ck.top, 0, 4, s));
                } else {
                    ck = Ckpt{};
                }
            }
        }
        uint64_t loop_launches = 0, suspensions = 0, resumed = 0, calls_kept = 0;
        c.counters[24] = 0;  // members of the clumps each rebinding pass ran, summed over the passes
        // One pass of the device loop over `list` (key-rank order). Clumps that found the
        // member pool full stop with a consistent state; the pool is compacted and they
        // continue in another launch.
        auto run_loop = [&](const std::vector<uint32_t> &list, const std::vector<std::vector<uint32_t>> *blk) -> int {
            std::vector<uint32_t> todo = list;
            int stuck = 0;
            for (int attempt = 0; !todo.empty(); ++attempt) {
                if (attempt > 4096 || stuck > 3) return kErrOutOfMemory;
                std::vector<uint8_t> fin(nb, 1);
                for (uint32_t sl : todo) fin[sl] = 0;
                PLAN_CUDA(cudaMemcpyAsync(d_fin, fin.data(), nb, cudaMemcpyHostToDevice, s));
                PLAN_CUDA(cudaMemsetAsync(d_head, 0, 4, s));
                int r = st.up_list(todo, st.d_list);
                if (r) return r;
                Arena &S = c.scratch;
                const size_t mark = S.used;
                uint32_t *d_blk = nullptr;
                const bool with_blk = blk != nullptr && attempt == 0;
                std::vector<uint32_t> off, lst;  // kept alive until the launch has read them
                if (with_blk) {
                    off.assign(todo.size() + 1, 0);
                    for (size_t i = 0; i < todo.size(); ++i) {
                        for (uint32_t b : (*blk)[todo[i]]) lst.push_back(b);
                        off[i + 1] = (uint32_t)lst.size();
                    }
                    d_blk = S.get<uint32_t>(lst.size() + 1);
                    if (S.failed || !d_blk) { S.used = mark; return kErrOutOfMemory; }
                    PLAN_CUDA(cudaMemcpyAsync(d_blkoff, off.data(), off.size() * 4, cudaMemcpyHostToDevice, s));
                    if (!lst.empty()) PLAN_CUDA(cudaMemcpyAsync(d_blk, lst.data(), lst.size() * 4, cudaMemcpyHostToDevice, s));
                }
                RbArgs ra;
                ra.list = st.d_list;
                ra.n = (uint32_t)todo.size();
                ra.head = d_head;
                ra.blk_off = with_blk ? d_blkoff : nullptr;
                ra.blk = d_blk;
                ra.finished = d_fin;
                ra.suspended = d_susp;
                ra.needsort = d_needsort;
                ra.distsq = d_distsq;
                ra.stats = d_rstats;
                ra.ct = ct;
                ra.P = P;
                ra.t = kt;
                ra.ft = ftr;
                ra.vel = tr.vel;
                ra.tm0 = tm0;
                ra.tm1 = tm1;
                ra.E = E;
                ra.epos = epos;
                ra.owner = owner;
                ra.rank_of = rank_of;
                ra.slot_of_rank = slot_of_rank;
                ra.tent = tent;
                ra.dmax = dmax;
                ra.dset = dset;
                ra.dover = dover;
                ra.com0 = bc;
                ra.reach = reach;
                ra.cp = st.cp;
                ra.err = c.d_err;
                // a blocker's calls take longer on larger snapshots: the bound grows with them
                ra.wait_limit = (uint32_t)std::min<uint64_t>(0xffffffffull, (uint64_t)kWaitLimit * std::max<uint64_t>(1, (Tu + (1u << 24) - 1) >> 24));
                ra.ccall = d_ccall;
                ra.dcall = d_dcall;
                ra.dfirst = d_dfirst;
                ra.ck = ck;
                const unsigned grid = (unsigned)std::min<size_t>(todo.size(), (size_t)rb_grid);
                double t_a = wall_ms();
                if (c.kev[0]) cudaEventRecord(c.kev[0], s);
                k_rebind_loop<<<grid, kRB, kRbSmem, s>>>(ra);
                c.launches++;
                ++loop_launches;
                PLAN_CUDA(cudaGetLastError());
                if (c.kev[1]) cudaEventRecord(c.kev[1], s);
                std::vector<uint8_t> sus;
                std::vector<uint32_t> mn_after;
                r = st.down(sus, d_susp, nb);
                if (!r) r = st.down(mn_after, ct.mn, C);
                S.used = mark;
                if (r) return r;
                c.stage_ms[16] += wall_ms() - t_a;
                float kms = 0.f;
                if (c.kev[0] && c.kev[1] && cudaEventElapsedTime(&kms, c.kev[0], c.kev[1]) == cudaSuccess) c.stage_ms[19] += kms;
                uint64_t launch_members = 0;
                for (uint32_t sl : todo) launch_members += mn_after[sl];
                if (trace.on)
                    std::fprintf(stderr, "[plan]   rebinding launch: %zu clumps, %llu members, %.3f ms\n", todo.size(),
                                 (unsigned long long)launch_members, (double)kms);
                std::vector<uint32_t> next;
                for (uint32_t sl : todo)
                    if (sus[sl]) next.push_back(sl);
                if (!next.empty()) {
                    suspensions += next.size();
                    stuck = next.size() == todo.size() ? stuck + 1 : 0;
                    r = st.maybe_compact(true);
                    if (r) return r;
                }
                todo.swap(next);
            }
            // the pass's work in the algorithmic model: the members of the clumps it ran, each
            // once however many launches (after member-pool compactions) it took
            std::vector<uint32_t> mn_end;
            int r = st.down(mn_end, ct.mn, C);
            if (r) return r;
            for (uint32_t sl : list) c.counters[24] += mn_end[sl];
            return kOk;
        };
        // Rounds until no clump grows. Clumps in `waiting` start once every clump listed as
        // their blocker has finished (reruns in key order where their balls may meet).
        std::vector<uint8_t> finished(C, 0);
        std::vector<uint32_t> rounds_of(C, 0);  // rounds a clump grew in during the last pass
        auto run_rounds = [&](std::vector<uint32_t> active, int seq_mode, std::vector<uint32_t> waiting,
                              const std::vector<std::vector<uint32_t>> &blockers) -> int {
            for (uint32_t sl : active) finished[sl] = 0;
            for (uint32_t sl : waiting) finished[sl] = 0;
            auto admit = [&](std::vector<uint32_t> &to) {
                std::vector<uint32_t> keep;
                for (uint32_t w : waiting) {
                    bool ready = true;
                    for (uint32_t b : blockers[w]) ready = ready && finished[b];
                    if (ready) to.push_back(w);
                    else keep.push_back(w);
                }
                waiting.swap(keep);
            };
            admit(active);
            for (int round = 0; !active.empty() || !waiting.empty(); ++round) {
                if (round > 200000) return kErrDeviceLimit;
                if (active.empty()) {  // cannot happen with blockers of lower rank; start the first waiting clump
                    active.push_back(waiting.front());
                    waiting.erase(waiting.begin());
                }
                ++rounds;
                int r = st.up_list(active, st.d_list);
                if (r) return r;
                double t_a = wall_ms();
                rebind_kernel<<<(unsigned)active.size(), kRebindThreads, 0, s>>>(st.d_list, ct, P, kt, tr.vel, E, epos, in_clump, owner,
                                                                                  rank_of, slot_of_rank, invalid, dmax, dset, dover, seq_mode,
                                                                                  st.cp, d_grew,
                                                                                  d_mnout, c.d_err, trace.on ? d_prof : nullptr, bc, reach, tent, ftr);
                c.launches++;
                PLAN_CUDA(cudaGetLastError());
                std::vector<uint8_t> g;
                std::vector<uint32_t> mo;
                r = st.down(g, d_grew, active.size());
                if (!r) r = st.down(mo, d_mnout, active.size());
                if (r) return r;
                // calls that found the member pool full (grew = 2) changed nothing: compact the
                // pool and repeat them
                for (int attempt = 0;; ++attempt) {
                    std::vector<uint32_t> retry;
                    std::vector<size_t> at_k;
                    for (size_t k = 0; k < active.size(); ++k)
                        if (g[k] == 2) { retry.push_back(active[k]); at_k.push_back(k); }
                    if (retry.empty()) break;
                    if (attempt > 0 && retry.size() == g.size()) return kErrOutOfMemory;
                    r = st.maybe_compact(true);
                    if (!r) r = st.up_list(retry, st.d_list);
                    if (r) return r;
                    rebind_kernel<<<(unsigned)retry.size(), kRebindThreads, 0, s>>>(st.d_list, ct, P, kt, tr.vel, E, epos, in_clump, owner,
                                                                                     rank_of, slot_of_rank, invalid, dmax, dset, dover, seq_mode,
                                                                                     st.cp, d_grew, d_mnout, c.d_err, nullptr, bc, reach, tent, ftr);
                    c.launches++;
                    PLAN_CUDA(cudaGetLastError());
                    std::vector<uint8_t> g2;
                    std::vector<uint32_t> mo2;
                    r = st.down(g2, d_grew, retry.size());
                    if (!r) r = st.down(mo2, d_mnout, retry.size());
                    if (r) return r;
                    size_t still = 0;
                    for (size_t q = 0; q < retry.size(); ++q) {
                        g[at_k[q]] = g2[q];
                        mo[at_k[q]] = mo2[q];
                        still += g2[q] == 2;
                    }
                    if (still == retry.size()) return kErrOutOfMemory;  // no progress after compaction
                    c.counters[22] += retry.size();
                }
                double t_b = wall_ms();
                c.stage_ms[16] += t_b - t_a;
                if (trace.on && (round % 25 == 0 || t_b - t_a > 20)) {
                    std::vector<unsigned long long> pr;
                    r = st.down(pr, d_prof, 8 * active.size());
                    if (r) return r;
                    unsigned long long mx[4] = {0, 0, 0, 0}, sum[4] = {0, 0, 0, 0};
                    size_t worst = 0;
                    unsigned long long worst_t = 0;
                    for (size_t k = 0; k < active.size(); ++k) {
                        unsigned long long tot = 0;
                        for (int q = 0; q < 4; ++q) {
                            mx[q] = std::max(mx[q], pr[8 * k + q]);
                            sum[q] += pr[8 * k + q];
                            tot += pr[8 * k + q];
                        }
                        if (tot > worst_t) { worst_t = tot; worst = k; }
                    }
                    const unsigned long long *w = &pr[8 * worst];
                    std::fprintf(stderr,
                                 "[plan]   rebind kernel %.1f ms, %zu blocks; max kcycles front %llu count %llu fill %llu accept %llu; "
                                 "worst block: front %llu count %llu fill %llu accept %llu kcycles, nf %llu nel %llu nacc %llu iters %llu m0 %llu\n",
                                 t_b - t_a, active.size(), mx[0] / 1000, mx[1] / 1000, mx[2] / 1000, mx[3] / 1000, w[0] / 1000, w[1] / 1000,
                                 w[2] / 1000, w[3] / 1000, w[4], w[5], w[6], w[7] >> 32, w[7] & 0xffffffffull);
                }
                std::vector<uint32_t> grown, grown_mn;
                for (size_t k = 0; k < active.size(); ++k)
                    if (g[k] == 1) { grown.push_back(active[k]); grown_mn.push_back(mo[k]); }
                // SortParticles when the clump grew, then CalculateHillRadius (unchanged mass
                // gives an unchanged radius for the others)
                r = st.sort_particles(grown, false, true, &grown_mn);
                if (!r) r = st.sync();
                double t_c = wall_ms();
                c.stage_ms[17] += t_c - t_b;
                if (trace.on && (round % 25 == 0 || t_c - t_b > 20))
                    std::fprintf(stderr, "[plan]   sort particles %.1f ms for %zu grown\n", t_c - t_b, grown.size());
                if (!r) r = st.maybe_compact();
                if (r) return r;
                c.stage_ms[18] += wall_ms() - t_c;
                uint64_t mx = 0;
                for (uint32_t v : grown_mn) mx = std::max<uint64_t>(mx, v);
                c.counters[16] = std::max<uint64_t>(c.counters[16], mx);
                if (round % 25 == 0) trace.mark("rebinding round (round, grown, largest, waiting)", round, grown.size(), mx, waiting.size());
                for (size_t k = 0; k < active.size(); ++k) {
                    if (g[k] != 1) finished[active[k]] = 1;
                    else rounds_of[active[k]] = round + 1;
                }
                admit(grown);
                active.swap(grown);
            }
            return kOk;
        };
        const std::vector<std::vector<uint32_t>> no_blockers(C);
        // reruns either start together (speculatively, as the first pass) or wait for the
        // reruns they met in the previous pass (PLAN_RERUN_SCHEDULE=1)
        const char *sched_env = std::getenv("PLAN_RERUN_SCHEDULE");
        const bool schedule_reruns = sched_env && *sched_env == '1';
        const char *front_env = std::getenv("PLAN_RERUN_FRONT");  // rerun only clumps without pending partners
        const bool front_only = front_env && *front_env == '1';
        std::vector<std::vector<uint32_t>> blockers(C);
        std::vector<unsigned long long> pred_hash(C, 0);
        std::vector<uint32_t> keep_of(C, 0);  // per slot: checkpoints its next rerun keeps
        std::vector<uint32_t> active = live;
        for (uint32_t pass = 0; !active.empty(); ++pass) {
            if (pass > nlive + 2) return kErrDeviceLimit;
            ++passes;
            const std::vector<uint32_t> active_all = active;
            std::vector<uint32_t> waiting;
            if (pass > 0 && schedule_reruns) {  // the reruns start once the reruns they met in the last pass are done
                std::vector<uint32_t> first;
                for (uint32_t sa : active) {
                    if (blockers[sa].empty()) first.push_back(sa);
                    else waiting.push_back(sa);
                }
                trace.mark("rerun schedule (rerun, start now, wait)", active.size(), first.size(), waiting.size());
                active.swap(first);
            }
            const std::vector<uint32_t> ran = pass > 0 ? active_all : live;
            if (use_rounds) {
                rc = run_rounds(active, 0, waiting, (pass > 0 && schedule_reruns) ? blockers : no_blockers);
            } else {
                // reruns wait on the device for the lower-ranked reruns they met in the last
                // pass (PLAN_RERUN_SCHEDULE=0: all start at once)
                if (d_rstats) PLAN_CUDA(cudaMemsetAsync(d_rstats, 0, (size_t)kRbStats * nb * 8, s));
                rc = run_loop(active_all, (pass > 0 && !(sched_env && *sched_env == '0')) ? &blockers : nullptr);
                if (!rc && trace.on) {
                    std::vector<unsigned long long> rs;
                    rc = st.down(rs, d_rstats, (size_t)kRbStats * nb);
                    if (!rc) {
                        size_t worst = 0;
                        unsigned long long wt = 0, calls = 0, acc = 0;
                        for (uint32_t sl : active_all) {
                            const unsigned long long *q = &rs[(size_t)kRbStats * sl];
                            calls += q[0];
                            acc += q[2];
                            if (q[3] + q[4] + q[5] > wt) { wt = q[3] + q[4] + q[5]; worst = sl; }
                        }
                        const unsigned long long *w = &rs[(size_t)kRbStats * worst];
                        std::fprintf(stderr,
                                     "[plan]   loop pass %u: %zu clumps, %llu calls, %llu accepted; worst clump: calls %llu scanned %llu cand %llu acc %llu "
                                     "rounds %llu unsure %llu | kcycles search %llu accept %llu (warp-0 updates %llu: table %llu chain %llu) sort %llu (sums %llu; dist %llu "
                                     "order %llu) sorts %llu members %llu | sum steps/kcycles:",
                                     (unsigned)pass, active_all.size(), calls, acc, w[0], w[13], w[1], w[2], w[12], w[10], w[3] / 1000, w[4] / 1000,
                                     w[14] / 1000, w[15] / 1000, w[16] / 1000, w[5] / 1000, w[6] / 1000, w[8] / 1000, w[9] / 1000, w[7], w[11]);
                        for (int q = 0; q < 7; ++q) std::fprintf(stderr, " %llu/%llu", w[17 + q], w[24 + q] / 1000);
                        std::fprintf(stderr, " | tiles %llu set-up kcycles %llu; predicted %llu held %llu taken %llu\n", w[32], w[31] / 1000, w[33],
                                     w[34], w[35]);
                    }
                }
            }
            if (rc) return rc;
            if (!live.empty()) {  // every clump: a running one may have taken a particle from any later one
                rc = st.up_list(live, st.d_list2);
                if (rc) return rc;
                k_rebind_verify<<<(unsigned)live.size(), 256, 0, s>>>(st.d_list2, (uint32_t)live.size(), ct, P, in_clump, owner, rank_of,
                                                                      invalid, dset, dover, dmax, ck, d_lostck);
                c.launches++;
                PLAN_CUDA(cudaGetLastError());
            }
            std::vector<uint8_t> inv, dov;
            std::vector<uint32_t> dm, ds, hdc, hdf, hckn, hckc, hlost;
            rc = st.down(inv, invalid, C);
            if (!rc) rc = st.down(dm, dmax, C);
            if (!rc) rc = st.down(ds, dset, (size_t)C * kDeferSlots);
            if (!rc) rc = st.down(dov, dover, C);
            if (!rc && ck.n) {
                rc = st.down(hdc, d_dcall, (size_t)C * kDeferSlots);
                if (!rc) rc = st.down(hdf, d_dfirst, C);
                if (!rc) rc = st.down(hckn, ck.n, nlive);
                if (!rc) rc = st.down(hckc, ck.call, (size_t)nlive * kCk);
                if (!rc) rc = st.down(hlost, d_lostck, nlive);
            }
            if (rc) return rc;
            // checkpoints of rank r made after calls before j0
            auto ck_before = [&](uint32_t r, uint32_t j0) -> uint32_t {
                uint32_t k = 0;
                while (k < hckn[r] && hckc[(size_t)r * kCk + k] < j0) ++k;
                return k;
            };
            // clumps of this pass whose members differ from the prediction the others used
            std::vector<uint8_t> changed(nlive + 1, 0);
            if (pass > 0) {
                rc = st.up_list(ran, st.d_list2);
                if (rc) return rc;
                k_member_hash<<<(unsigned)ran.size(), 256, 0, s>>>(st.d_list2, (uint32_t)ran.size(), ct, P, mhash);
                c.launches++;
                std::vector<unsigned long long> hnow;
                rc = st.down(hnow, mhash, C);
                if (rc) return rc;
                for (uint32_t sl : ran) changed[h_rank[sl]] = hnow[sl] != pred_hash[sl];
            }
            // rerun the invalid clumps and, in rank order, every clump that skipped particles
            // of a clump that is rerun or ended up with other members than predicted; the
            // rest keep their result
            std::vector<uint32_t> rerun;
            std::vector<uint8_t> rr(nlive + 1, 0);
            uint32_t low = kNone;  // lowest rank rerun or changed so far
            uint64_t why_inv = 0, why_dov = 0, why_rerun = 0, why_changed = 0;
            for (uint32_t r = 0; r < nlive; ++r) {
                const uint32_t sl = live[r];
                // checkpoints the rerun keeps: none before the first call it affects
                uint32_t kp = ck.n ? hckn[r] : 0;
                bool again = inv[sl] != 0;
                why_inv += again;
                if (again && ck.n) kp = std::min(kp, hlost[r]);
                if (dov[sl]) {  // the records overflowed: any deferral may be the first affected call
                    const bool dep = low != kNone && dm[sl] && dm[sl] - 1 >= low;
                    why_dov += dep && !again;
                    if (dep && ck.n) kp = std::min(kp, ck_before(r, hdf[sl]));
                    again = again || dep;
                } else {
                    for (int j = 0; j < kDeferSlots; ++j) {
                        const uint32_t d0 = ds[(size_t)sl * kDeferSlots + j];
                        if (d0 == kNone) continue;
                        // a partner that reruns; or one whose members differ from what this clump
                        // assumed (it saw a holding that could still change)
                        const uint32_t d = d0 & ~kDeferSpec;
                        const bool spec = use_rounds || (d0 & kDeferSpec) != 0;
                        const bool dep = d < nlive && (rr[d] || (spec && changed[d]));
                        if (!dep) continue;
                        if (!again) {
                            why_rerun += rr[d];
                            why_changed += !rr[d];
                        }
                        again = true;
                        if (ck.n) kp = std::min(kp, ck_before(r, hdc[(size_t)sl * kDeferSlots + j]));
                    }
                }
                if (again) {
                    rerun.push_back(sl);
                    rr[r] = 1;
                    keep_of[sl] = kp;
                }
                if ((again || changed[r]) && low == kNone) low = r;
            }
            if (rerun.empty()) break;
            // Run only the front of the reruns: clumps none of whose recorded lower partners is
            // itself pending. The others keep their state (and stay pending: invalid, or
            // deferring to a pending clump) until their partners are settled; the closure above
            // decides again after every pass, so this only avoids work that would be redone.
            if (front_only) {
                std::vector<uint32_t> front;
                for (uint32_t sl : rerun) {
                    bool ready = true;
                    if (!dov[sl]) {
                        for (int j = 0; j < kDeferSlots && ready; ++j) {
                            const uint32_t d0 = ds[(size_t)sl * kDeferSlots + j], d = d0 & ~kDeferSpec;
                            ready = !(d0 != kNone && d < nlive && rr[d] && live[d] != sl);
                        }
                    }
                    if (ready) front.push_back(sl);
                }
                std::fill(rr.begin(), rr.end(), 0);
                for (uint32_t sl : front) rr[h_rank[sl]] = 1;
                trace.mark("rerun front (pending, run now)", rerun.size(), front.size());
                rerun.swap(front);
            }
            // their present members are the prediction of the next pass
            {
                rc = st.up_list(rerun, st.d_list2);
                if (rc) return rc;
                k_member_hash<<<(unsigned)rerun.size(), 256, 0, s>>>(st.d_list2, (uint32_t)rerun.size(), ct, P, mhash);
                c.launches++;
                std::vector<unsigned long long> hnow;
                rc = st.down(hnow, mhash, C);
                if (rc) return rc;
                for (uint32_t sl : rerun) pred_hash[sl] = hnow[sl];
            }
            trace.mark("rerun closure (invalid+deferred, changed)", rerun.size(), std::count(changed.begin(), changed.end(), 1));
            trace.mark("  rerun reasons (lost a particle, overflowed record, partner reruns, partner changed)", why_inv, why_dov, why_rerun,
                       why_changed);

            // blockers of each rerun clump: the rerun clumps of lower rank it met (skipped a
            // particle of, lost one to, or had one taken by); when its record overflowed, every
            // lower rerun clump whose balls came within reach
            std::vector<unsigned long long> rb;
            std::vector<double4_32a> c0;
            rc = st.down(rb, reach, C);
            if (!rc) rc = st.down(c0, bc, C);
            if (rc) return rc;
            for (size_t a = 0; a < rerun.size(); ++a) {
                const uint32_t sa = rerun[a];
                blockers[sa].clear();
                if (!dov[sa]) {
                    for (int j = 0; j < kDeferSlots; ++j) {
                        const uint32_t d0 = ds[(size_t)sa * kDeferSlots + j], d = d0 & ~kDeferSpec;
                        if (d0 != kNone && d < nlive && rr[d] && live[d] != sa) blockers[sa].push_back(live[d]);
                    }
                } else {
                    const double ra = __builtin_bit_cast(double, rb[sa]);
                    for (size_t b = 0; b < a; ++b) {  // rerun is in key order
                        const uint32_t sb = rerun[b];
                        const double r2 = __builtin_bit_cast(double, rb[sb]);
                        const double dx = c0[sa].x - c0[sb].x, dy = c0[sa].y - c0[sb].y, dz = c0[sa].z - c0[sb].z;
                        const double lim = 1.25 * (ra + r2) + 1e-12;
                        if (dx * dx + dy * dy + dz * dz <= lim * lim) blockers[sa].push_back(sb);
                    }
                }
            }
            reruns += rerun.size();
            std::vector<uint32_t> keep(rerun.size(), 0);
            uint32_t from_ck = 0;
            for (size_t k = 0; k < rerun.size(); ++k) {
                keep[k] = ck.n ? keep_of[rerun[k]] : 0;
                if (keep[k]) {
                    ++from_ck;
                    calls_kept += hckc[(size_t)h_rank[rerun[k]] * kCk + keep[k] - 1];
                }
            }
            resumed += from_ck;
            trace.mark("  rerun starts (from the beginning, from a checkpoint)", (long long)(rerun.size() - from_ck), from_ck);
            if (trace.fine_on && ck.n) {  // the largest reruns: where they resume, and why
                std::vector<uint32_t> mnow;
                rc = st.down(mnow, ct.mn, C);
                if (rc) return rc;
                std::vector<size_t> ord(rerun.size());
                std::iota(ord.begin(), ord.end(), size_t(0));
                std::sort(ord.begin(), ord.end(), [&](size_t x, size_t y) { return mnow[rerun[x]] > mnow[rerun[y]]; });
                for (size_t q = 0; q < std::min<size_t>(6, ord.size()); ++q) {
                    const uint32_t sl = rerun[ord[q]], r = h_rank[sl], kp = keep[ord[q]];
                    std::fprintf(stderr, "[plan]     rerun rank %u members %u: checkpoints %u (last after call %u), keeps %u (to call %u); lost %d first-lost ck %u%s\n",
                                 r, mnow[sl], hckn[r], hckn[r] ? hckc[(size_t)r * kCk + hckn[r] - 1] : 0, kp, kp ? hckc[(size_t)r * kCk + kp - 1] : 0,
                                 (int)inv[sl], inv[sl] ? hlost[r] : 0, dov[sl] ? " (records overflowed)" : "");
                    for (int j = 0; j < kDeferSlots; ++j) {
                        const uint32_t d0 = ds[(size_t)sl * kDeferSlots + j];
                        if (d0 == kNone) continue;
                        const uint32_t d = d0 & ~kDeferSpec;
                        std::fprintf(stderr, "[plan]       record rank %u%s call %u: %s\n", d, (d0 & kDeferSpec) ? " spec" : "", hdc[(size_t)sl * kDeferSlots + j],
                                     d < nlive && rr[d] ? "reruns" : (d < nlive && changed[d]) ? "changed" : "-");
                    }
                }
            }
            PLAN_CUDA(cudaMemcpyAsync(rerun_rank, rr.data(), nlive, cudaMemcpyHostToDevice, s));
            k_rebind_tentative<<<grid_for(Tu, 256), 256, 0, s>>>(Tu, owner, tent, rerun_rank);
            rc = st.maybe_compact();  // room for the restored segments
            if (rc) return rc;
            rc = st.up_list(rerun, st.d_list2);
            if (rc) return rc;
            if (ck.n) PLAN_CUDA(cudaMemcpyAsync(d_keep, keep.data(), keep.size() * 4, cudaMemcpyHostToDevice, s));
            RestoreArgs ra{bM, bh, bri, bro, br10, br2, bc, bv, bo, bn, bidx, bdist, invalid, dover, d_distsq, d_needsort, dmax, dset,
                           d_dcall, d_dfirst, d_ccall, owner, ck.n ? d_keep : nullptr, rank_of, in_clump, ck};
            k_rebind_restore<<<(unsigned)rerun.size(), 256, 0, s>>>(st.d_list2, (uint32_t)rerun.size(), ct, P, ra, c.d_err);
            c.launches += 2;
            PLAN_CUDA(cudaGetLastError());
            active = rerun;
        }
        // final ownership = the reference's in-clump marks of rebinding
        c.stage_ms[14] = (double)(use_rounds ? rounds : loop_launches);
        c.counters[14] = reruns;
        c.counters[12] = passes;
        c.counters[23] = suspensions;
        c.counters[28] = resumed;     // reruns that resumed from a checkpoint
        c.counters[29] = calls_kept;  // calls those resumptions did not redo
    }
    PLAN_CUDA(cudaStreamSynchronize(s));
    double tw3 = wall_ms();
    trace.mark("rebinding done (rounds, passes, reruns)", c.stage_ms[14], c.counters[12], c.counters[14]);
    // 6. prune and loose streams (src/tree.hpp:4213-4224)
    auto prune = [&]() -> int {
        if (!C) return kOk;
        k_prune<<<grid_for(C, 128), 128, 0, s>>>(C, ct, P, tr.vel, tr.dens, st.cp, st.d_flag8);
        c.launches++;
        std::vector<uint8_t> kill, alive;
        int r = st.down(kill, st.d_flag8, C);
        if (!r) r = st.down(alive, ct.alive, C);
        if (r) return r;
        for (uint32_t i = 0; i < C; ++i) if (kill[i]) alive[i] = 0;
        PLAN_CUDA(cudaMemcpyAsync(ct.alive, alive.data(), C, cudaMemcpyHostToDevice, s));
        return st.live_order(live);
    };
    rc = prune();
    if (rc) return rc;
    {
        rc = st.dispersion(live, std::min(diffuse + 0.1, 0.475), too);
        if (rc) return rc;
        std::vector<uint8_t> alive;
        rc = st.down(alive, ct.alive, C);
        if (rc) return rc;
        for (size_t k = 0; k < live.size(); ++k) if (too[k]) alive[live[k]] = 0;
        PLAN_CUDA(cudaMemcpyAsync(ct.alive, alive.data(), C, cudaMemcpyHostToDevice, s));
        rc = st.live_order(live);
        if (rc) return rc;
    }
    // 7. rip the envelope (src/tree.hpp:4229-4248)
    {
        uint8_t *pending = A.get<uint8_t>(C + 1);
        if (!pending) return kErrOutOfMemory;
        PLAN_CUDA(cudaMemsetAsync(pending, 1, C + 1, s));
        for (int round = 0; round < 100000 && C; ++round) {
            PLAN_CUDA(cudaMemsetAsync(st.d_u + 50, 0, 4, s));
            k_rip<<<grid_for(C, 128), 128, 0, s>>>(C, ct, P, pending, st.d_list2, st.d_u + 50);
            c.launches++;
            std::vector<uint32_t> nch;
            rc = st.down(nch, st.d_u + 50, 1);
            if (rc) return rc;
            if (!nch[0]) break;
            std::vector<uint32_t> changed;
            rc = st.down(changed, st.d_list2, nch[0]);
            if (rc) return rc;
            rc = st.kinematics(changed);
            if (!rc) rc = st.unbind(changed);  // includes SortParticles and the Hill radius
            if (rc) return rc;
        }
        rc = st.live_order(live);
        if (rc) return rc;
    }
    // 8-9. prune again; ghost clumps (src/tree.hpp:4253-4266)
    rc = prune();
    if (rc) return rc;
    {
        std::vector<double4_32a> com;
        std::vector<uint8_t> alive;
        rc = st.down(com, ct.com, C);
        if (!rc) rc = st.down(alive, ct.alive, C);
        if (rc) return rc;
        for (uint32_t sl : live) {
            double x[3] = {com[sl].x, com[sl].y, com[sl].z};
            bool in = true;
            for (int d = 0; d < 3; ++d) in = in && (x[d] >= p.box_min[d] && x[d] <= p.box_max[d]);
            if (!in) alive[sl] = 0;
        }
        PLAN_CUDA(cudaMemcpyAsync(ct.alive, alive.data(), C, cudaMemcpyHostToDevice, s));
        rc = st.live_order(live);
        if (rc) return rc;
    }
    // 10. angular momentum (src/tree.hpp:4273-4275)
    if (!live.empty()) {
        rc = st.up_list(live, st.d_list);
        if (rc) return rc;
        k_angmom<<<(unsigned)((live.size() + 3) / 4), 128, 0, s>>>(st.d_list, (uint32_t)live.size(), ct, P, tr.pos, tr.vel, st.cp);
        c.launches++;
    }
    cudaEventRecord(ev[5], s);
    PLAN_CUDA(cudaStreamSynchronize(s));
    double tw4 = wall_ms();
    trace.mark("prune, rip, ghost cut, J");
    c.stage_ms[10] = tw1 - tw0;  // HOP-group sort + both merge sweeps
    c.stage_ms[11] = tw2 - tw1;  // re-key + unbinding
    c.stage_ms[12] = tw3 - tw2;  // Hill rebinding
    c.stage_ms[13] = tw4 - tw3;  // prune, rip, ghost cut, J
    c.counters[15] = st.compactions;

    // ------------------------------------------------------------------ catalogue
    plan_catalogue *cat = new plan_catalogue();
    cat->time = c.time;
    cat->mass_total_code_units = p.mass_total_code_units;
    cat->mass_physical = p.mass_physical;
    cat->grav_constant = p.grav_constant;
    cat->Omega = p.Omega;
    const uint32_t nl = (uint32_t)live.size();
    std::vector<uint32_t> keys, mn;
    std::vector<double> M;
    std::vector<double4_32a> com, vcom, J;
    rc = st.down(keys, ct.key, C);
    if (!rc) rc = st.down(mn, ct.mn, C);
    if (!rc) rc = st.down(M, ct.M, C);
    if (!rc) rc = st.down(com, ct.com, C);
    if (!rc) rc = st.down(vcom, ct.vcom, C);
    if (!rc) rc = st.down(J, ct.J, C);
    if (rc) { delete cat; return rc; }
    std::vector<uint32_t> base(nl + 1, 0);
    for (uint32_t t = 0; t < nl; ++t) base[t + 1] = base[t] + mn[live[t]];
    const uint32_t tot = base[nl];
    uint64_t d2h = (uint64_t)C * (4 + 4 + 8 + 3 * 32);  // catalogue bytes read back: clump table ...
    if (nl) {
        uint32_t *dl = A.get<uint32_t>(nl), *db = A.get<uint32_t>(nl + 1), *ocnt = A.get<uint32_t>(tot + 1), *obase = A.get<uint32_t>(tot + 1);
        uint32_t *d_otot = A.get<uint32_t>(2);
        if (A.failed) { delete cat; return kErrOutOfMemory; }
        PLAN_CUDA(cudaMemcpyAsync(dl, live.data(), nl * 4, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(db, base.data(), (nl + 1) * 4, cudaMemcpyHostToDevice, s));
        k_out_counts<<<nl, 256, 0, s>>>(dl, nl, db, ct, P, tr.sink_n, ocnt);
        const size_t sm3 = c.scratch.used;
        size_t sb = scan_u32_scratch_bytes(tot + 1);
        void *scr = c.scratch.take(sb);
        if (!scr) { delete cat; return kErrOutOfMemory; }
        rc = scan_u32(ocnt, obase, tot, d_otot, scr, sb, s);
        c.scratch.used = sm3;
        if (rc) { delete cat; return rc; }
        uint32_t otot = 0;
        PLAN_CUDA(cudaMemcpyAsync(&otot, d_otot, 4, cudaMemcpyDeviceToHost, s));
        rc = st.sync();
        if (rc) { delete cat; return rc; }
        double *mpos = A.get<double>(3 * (size_t)tot + 3), *mvel = A.get<double>(3 * (size_t)tot + 3), *mmass = A.get<double>(tot + 1);
        uint32_t *morig = A.get<uint32_t>(tot + 1);
        double *opos = A.get<double>(3 * (size_t)otot + 3);
        if (A.failed) { delete cat; return kErrOutOfMemory; }
        k_out_fill<<<nl, 256, 0, s>>>(dl, nl, db, ct, P, tr.pos, tr.vel, tr.orig, tr.sink_n, tr.sink_first, tr.sorted_src, tr.in_pos, obase,
                                      mpos, mvel, mmass, morig, opos);
        c.launches += 3;
        std::vector<double> hpos, hvel, hmass, hopos;
        std::vector<uint32_t> horig, hob;
        rc = st.down(hpos, mpos, 3 * (size_t)tot);
        if (!rc) rc = st.down(hvel, mvel, 3 * (size_t)tot);
        if (!rc) rc = st.down(hmass, mmass, tot);
        if (!rc) rc = st.down(horig, morig, tot);
        if (!rc) rc = st.down(hopos, opos, 3 * (size_t)otot);
        if (!rc) rc = st.down(hob, obase, tot);
        if (rc) { delete cat; return rc; }
        d2h += 4 + (uint64_t)tot * (24 + 24 + 8 + 4 + 4) + (uint64_t)otot * 24;  // ... and member records
        cat->clumps.resize(nl);
        for (uint32_t t = 0; t < nl; ++t) {
            uint32_t sl = live[t];
            auto &k = cat->clumps[t];
            k.key = keys[sl];
            k.M = M[sl];
            k.com[0] = com[sl].x; k.com[1] = com[sl].y; k.com[2] = com[sl].z;
            k.vcom[0] = vcom[sl].x; k.vcom[1] = vcom[sl].y; k.vcom[2] = vcom[sl].z;
            k.Jsum[0] = J[sl].x; k.Jsum[1] = J[sl].y; k.Jsum[2] = J[sl].z;
            uint32_t b = base[t], n = mn[sl];
            k.orig.assign(horig.begin() + b, horig.begin() + b + n);
            k.pos.assign(hpos.begin() + 3 * (size_t)b, hpos.begin() + 3 * (size_t)(b + n));
            k.vel.assign(hvel.begin() + 3 * (size_t)b, hvel.begin() + 3 * (size_t)(b + n));
            k.mass.assign(hmass.begin() + b, hmass.begin() + b + n);
            uint32_t ob = hob[b], oe = (t + 1 < nl) ? hob[base[t + 1]] : otot;
            k.opos.assign(hopos.begin() + 3 * (size_t)ob, hopos.begin() + 3 * (size_t)oe);
            k.npar = oe - ob;
        }
        cat->have_members = true;
    }
    trace.mark("catalogue download");
    finish_catalogue(*cat, p.num_peaks);  // ranking, cap, host-libm values, summary
    rc = st.sync();
    if (rc) { delete cat; return rc; }
    float ms;
    cudaEventElapsedTime(&ms, ev[0], ev[1]); c.stage_ms[4] = ms;
    cudaEventElapsedTime(&ms, ev[1], ev[2]); c.stage_ms[5] = ms;
    cudaEventElapsedTime(&ms, ev[2], ev[3]); c.stage_ms[6] = ms;
    cudaEventElapsedTime(&ms, ev[3], ev[5]); c.stage_ms[7] = ms;
    c.stage_ms[8] = wall_ms() - tw4;  // catalogue download and host finishing
    for (auto &e : ev) cudaEventDestroy(e);
    c.counters[7] = cat->clumps.size();
    c.counters[21] = d2h;
    c.counters[25] = c.arena.peak;  // bytes of the snapshot arena used at most, and its size
    c.counters[26] = c.arena.cap;
    if (out) *out = cat;
    else delete cat;
    return kOk;
}

}  // namespace plan
