// FP32-filtered KNN with the reference's exact results.
//
// On this GPU a dependent FP64 add takes ~63 cycles and FP64 issue is ~1/72 of FP32, so the
// reference's FP64 traversal is recast: points and node centres are held as exact float
// hi/lo pairs (every coordinate is a float32 or a float32 shifted by the box length, so two
// floats represent it exactly; node centres are dyadic), differences are formed as
// (a_hi - b_hi) + (a_lo - b_lo), and every comparison the reference makes in FP64 is
// decided in FP32 when the FP32 value is outside a proven error bound of the threshold.
// The bound used is relative 2^-17 plus a small absolute term, against a worst-case FP32
// error near 2^-20 relative, so a decided comparison always agrees with the FP64 one.
// Coordinates that are not float sums (ghost images shifted by the shear at t != 0) are held
// to 2^-48 relative, an absolute error below 1e-15 per difference for |x| < 0.25; squared
// distances then err by at most 2*sqrt(3)*d*1e-15, which 2^-17*d^2 + 1e-24 covers for every d.
// When a comparison falls inside its bound the query is redone on the exact FP64 path, and
// exact FP64 distances are computed for every candidate that could belong to the k
// nearest; a tie at the k-boundary also sends the query to the exact heap path.
#pragma once

#include "tree_walk.cuh"

namespace plan {

struct FTree {
    const float4 *phi, *plo;  // points: x, y, z (hi / lo)
    const float4 *nhi, *nlo;  // nodes: cx, cy, cz, hw (hi / lo)
};

constexpr float kRel = 7.62939453125e-06f;  // 2^-17
constexpr float kAbs = 1e-30f;
constexpr float kSqrt3f = 1.7320508075688772f;

// a < b decided with relative/absolute error bounds on both sides (any signs): 1 true,
// 0 false, -1 unsure
__device__ __forceinline__ int f_less(float a, float b, float abs_a = kAbs) {
    float ea = fabsf(a) * kRel + abs_a, eb = fabsf(b) * kRel;
    if (a + ea < b - eb) return 1;
    if (a - ea > b + eb) return 0;
    return -1;
}

__device__ __forceinline__ float f_diff(float ah, float al, float bh, float bl) { return (ah - bh) + (al - bl); }

// SphereContainNode in FP32: 1 contained, 0 not, -1 unsure
__device__ __forceinline__ int f_contained(const float4 nh, const float4 nl, const float4 qh, const float4 ql, float r) {
    float t = nh.w * kSqrt3f;
    float a = fabsf(f_diff(nh.x, nl.x, qh.x, ql.x)) + t;
    float b = fabsf(f_diff(nh.y, nl.y, qh.y, ql.y)) + t;
    float c = fabsf(f_diff(nh.z, nl.z, qh.z, ql.z)) + t;
    float s = a * a + b * b + c * c;
    return f_less(s, r * r, 1e-24f);
}

// SphereNodeIntersect in FP32: 1 intersects, 0 not, -1 unsure
__device__ __forceinline__ int f_intersects(const float4 nh, const float4 nl, const float4 qh, const float4 ql, float r) {
    float dx = f_diff(nh.x, nl.x, qh.x, ql.x), dy = f_diff(nh.y, nl.y, qh.y, ql.y), dz = f_diff(nh.z, nl.z, qh.z, ql.z);
    float c2c = dx * dx + dy * dy + dz * dz;
    float t = nh.w * kSqrt3f + r;
    int outside = f_less(t * t, c2c, 1e-24f);  // c2c > t^2
    if (outside == 1) return 0;
    if (outside == -1) return -1;
    int a = f_less(c2c, r, 1e-24f), b = f_less(c2c, nh.w, 1e-24f);
    if (a == 1 || b == 1) return 1;
    if (a == -1 || b == -1) return -1;
    // exact box distance: q below, inside or above each face (differences q - c vs +-hw)
    float m2 = 0.f;
    float d3[3] = {-dx, -dy, -dz};  // q - c
    for (int k = 0; k < 3; ++k) {
        float u = d3[k];
        int below = f_less(u, -nh.w, 1e-14f), above = f_less(nh.w, u, 1e-14f);
        if (below == -1 || above == -1) return -1;
        if (below == 1) { float e = u + nh.w; m2 += e * e; }
        else if (above == 1) { float e = u - nh.w; m2 += e * e; }
    }
    int in = f_less(r * r, m2, 1e-24f);  // m2 > r^2 means no intersection
    if (in == -1) return -1;
    return in == 1 ? 0 : 1;
}

// The reference's recursion with FP32 node classification; returns false if any
// classification was unsure (the caller then takes the FP64 path).
template <class Visit>
__device__ __forceinline__ bool f_traverse(const KTree &t, const FTree &f, const float4 qh, const float4 ql, float r, Visit visit,
                                           unsigned *err) {
    uint32_t node = 0;
    for (uint32_t guard = 0; guard < 4u * t.nodes + 8u; ++guard) {
        if (node >= t.nodes) {
            atomicOr(err, (unsigned)kDevErrBadNode);
            return false;
        }
        const float4 nh = f.nhi[node], nl = f.nlo[node];
        bool down = false;
        int cont = f_contained(nh, nl, qh, ql, r);
        if (cont < 0) return false;
        if (cont) {
            if (!visit(t.nbeg[node], t.nend[node])) return true;
        } else {
            int inter = f_intersects(nh, nl, qh, ql, r);
            if (inter < 0) return false;
            if (inter) {
                if (t.nnd[node] == 0) {
                    if (!visit(t.nbeg[node], t.nend[node])) return true;
                } else {
                    down = true;
                }
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

// Max-heap of FP32 keys (approximate distances) with candidate indices, strided slab.
struct FHeap {
    float *k;
    uint32_t *ix;
    int stride;
    __device__ float kget(int j) const { return k[j * stride]; }
    __device__ void put(int j, float v, uint32_t i) { k[j * stride] = v; ix[j * stride] = i; }
    __device__ void sift_up(int j) {
        float v = kget(j);
        uint32_t vi = ix[j * stride];
        while (j > 0) {
            int p = (j - 1) / 2;
            if (!(kget(p) < v)) break;
            put(j, kget(p), ix[p * stride]);
            j = p;
        }
        put(j, v, vi);
    }
    __device__ void sift_down(int j, int len) {
        float v = kget(j);
        uint32_t vi = ix[j * stride];
        for (;;) {
            int c = 2 * j + 1;
            if (c >= len) break;
            if (c + 1 < len && kget(c) < kget(c + 1)) ++c;
            if (!(v < kget(c))) break;
            put(j, kget(c), ix[c * stride]);
            j = c;
        }
        put(j, v, vi);
    }
    // keep the `cap` smallest keys
    __device__ void add(int &size, int cap, float v, uint32_t i) {
        if (size < cap) {
            put(size, v, i);
            sift_up(size);
            ++size;
        } else if (v < kget(0)) {
            put(0, v, i);
            sift_down(0, size);
        }
    }
};

__device__ __forceinline__ float f_dr2(const float4 qh, const float4 ql, const float4 ph, const float4 pl) {
    float dx = f_diff(qh.x, ql.x, ph.x, pl.x), dy = f_diff(qh.y, ql.y, ph.y, pl.y), dz = f_diff(qh.z, ql.z, ph.z, pl.z);
    return dx * dx + dy * dy + dz * dz;
}

// Upper/lower bounds of the FP64 distance given the FP32 one.
__device__ __forceinline__ float f_hi(float v) { return v * (1.f + kRel) + 1e-24f; }
__device__ __forceinline__ float f_lo(float v) { return v * (1.f - kRel) - 1e-24f; }

// Exact k-nearest of the reference for one query through the FP32 filter, in two parts.
// knn_collect_f32 walks the tree in FP32 and leaves the candidates in ascending FP32 order in
// the heap slab; it returns how many of them could belong to the k nearest (z), or -1 when
// the query must take the exact FP64 path. knn_exact_f32 then takes their exact FP64
// distances. The callers let the warp reconverge between the two (the walks of a warp's
// queries diverge; the FP64 part, whose instructions cost the same for one lane as for 32,
// then runs for all lanes at once).
// Slab layout per thread: cap = k + slack entries of (float key, u32 idx) and of (double, u32).
__device__ inline int knn_collect_f32(const KTree &t, const FTree &f, uint32_t qi, double r, uint32_t k, int cap, FHeap &fh, unsigned *err) {
    const float4 qh = f.phi[qi], ql = f.plo[qi];
    // radius doubling with count-only passes
    for (int it = 0; it < 200; ++it) {
        uint32_t cnt = 0;
        bool ok = f_traverse(t, f, qh, ql, (float)r, [&](uint32_t b, uint32_t e) { cnt += e - b; return cnt < k; }, err);
        if (!ok) return -1;
        if ((float)r != (float)r || r > 1e30) return -1;
        if (cnt >= k) break;
        r = r * 2;
        if (it == 199) return -1;
    }
    // the float radius must order exactly like the double one in every test above; tests
    // carry their own margins, but a radius that is not representable to 2^-24 is fine
    // because kRel covers its rounding
    int size = 0;
    uint32_t visited = 0;
    bool ok = f_traverse(t, f, qh, ql, (float)r,
                         [&](uint32_t b, uint32_t e) {
                             for (uint32_t p = b; p < e; ++p) fh.add(size, cap, f_dr2(qh, ql, f.phi[p], f.plo[p]), p);
                             visited += e - b;
                             return true;
                         },
                         err);
    if (!ok || visited < k) return -1;
    // heap -> ascending FP32 order
    for (int len = size; len > 1; --len) {
        float v = fh.kget(0);
        uint32_t vi = fh.ix[0];
        fh.put(0, fh.kget(len - 1), fh.ix[(len - 1) * fh.stride]);
        fh.put(len - 1, v, vi);
        fh.sift_down(0, len - 1);
    }
    const float thr = f_hi(fh.kget(k - 1));  // >= the k-th smallest exact distance
    if ((int)visited > size && !(f_lo(fh.kget(size - 1)) > thr)) return -1;  // buffer might miss candidates
    int z = 0;
    while (z < size && !(f_lo(fh.kget(z)) > thr)) ++z;
    return z;
}

// The second part: fills d64/i64 (ascending exact dr2, the reference's k-set) from the z
// candidates and returns k, or -1 on a tie the library heap order decides.
__device__ inline int knn_exact_f32(const KTree &t, double qx, double qy, double qz, uint32_t k, int z, const FHeap &fh, double *d64,
                                    uint32_t *i64) {
    const int dstride = 1;
    // exact FP64 distances for every possible member, insertion-sorted by (dr2, index)
    for (int j = 0; j < z; ++j) {
        uint32_t p = fh.ix[j * fh.stride];
        double v = point_dr2(qx, qy, qz, t.pos[p]);
        int m = j;
        while (m > 0) {
            double pv = d64[(m - 1) * dstride];
            uint32_t pi = i64[(m - 1) * dstride];
            if (pv < v || (pv == v && pi < p)) break;
            d64[m * dstride] = pv;
            i64[m * dstride] = pi;
            --m;
        }
        d64[m * dstride] = v;
        i64[m * dstride] = p;
    }
    // a tie at the k-boundary or inside the k-set is resolved by the library heap order of
    // the reference: leave those queries to the exact path
    for (int j = 1; j < (int)k + (z > (int)k ? 1 : 0); ++j)
        if (d64[(j - 1) * dstride] == d64[j * dstride]) return -1;
    return (int)k;
}

}  // namespace plan
