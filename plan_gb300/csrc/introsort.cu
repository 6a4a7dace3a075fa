// The order std::sort gives the Morton keys (src/tree.hpp:2831) when keys repeat.
//
// BHtree::BuildTree sorts 128-bit Morton values with a comparator that looks at the low 96
// bits only (AscendingMorton, src/tree.hpp:2269-2273), so particles that share a key (the
// future sink particles) end up in the order libstdc++'s introsort happens to leave them,
// and that order decides which particle represents a sink and in which order its
// velocities are summed (src/tree.hpp:2591-2630). Without repeated keys any correct sort
// gives the same array; with them, this file reproduces the library's algorithm.
//
// libstdc++ (GCC 13, bits/stl_algo.h) sorts by an introsort loop (median-of-three pivot
// moved to the front, an unguarded Hoare partition of the rest, recursion on the right part
// and a loop on the left part, ranges of at most 16 left alone, a heap sort once the depth
// budget of 2*floor(log2 n) is spent), then a final insertion sort. The insertion sort moves
// an element only past strictly greater ones, so it keeps the relative order of equal keys:
// the final array is the array after the introsort loop, stably sorted. This file runs the
// loop level by level over all live ranges at once, then the stable radix sort finishes.
//
// One Hoare partition of [f+1, l) around the pivot P at f, in parallel: with L_1 < L_2 < ...
// the positions holding a key >= P and R_1 > R_2 > ... those holding a key <= P, the
// partition swaps L_k with R_k for k = 1..m, m the largest k with L_k < R_k (equivalently
// m = max over x of min(#{L_k < x}, #{R_k >= x})), and returns min(L_{m+1}, R_m) (L_1 when
// m = 0). Both counts come from prefix sums over the ranges.
#include <algorithm>
#include <vector>

#include "pipeline.h"
#include "sort.h"

namespace plan {

namespace {

constexpr uint32_t kThreshold = 16;  // _S_threshold

struct Keys {
    uint32_t *w0, *w1, *w2, *ix;
};

__device__ __forceinline__ bool kless(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t b0, uint32_t b1, uint32_t b2) {
    if (a2 != b2) return a2 < b2;
    if (a1 != b1) return a1 < b1;
    return a0 < b0;
}

__device__ __forceinline__ bool kless_at(const Keys &k, uint32_t i, uint32_t j) {
    return kless(k.w0[i], k.w1[i], k.w2[i], k.w0[j], k.w1[j], k.w2[j]);
}

__device__ __forceinline__ void kswap(const Keys &k, uint32_t i, uint32_t j) {
    uint32_t t;
    t = k.w0[i]; k.w0[i] = k.w0[j]; k.w0[j] = t;
    t = k.w1[i]; k.w1[i] = k.w1[j]; k.w1[j] = t;
    t = k.w2[i]; k.w2[i] = k.w2[j]; k.w2[j] = t;
    t = k.ix[i]; k.ix[i] = k.ix[j]; k.ix[j] = t;
}

// Ranges whose depth budget is spent go to the heap-sort list; the others get their pivot
// (__move_median_to_first on first+1, mid, last-1) and take part in this level.
__global__ void k_pivot(uint32_t ns, const uint32_t *sf, const uint32_t *sl, const uint32_t *sd, Keys k, uint32_t *size,
                        uint32_t *pk, uint32_t *hf, uint32_t *hl, uint32_t *nheap) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ns) return;
    const uint32_t f = sf[g], l = sl[g];
    if (sd[g] == 0) {
        uint32_t h = atomicAdd(nheap, 1u);
        hf[h] = f;
        hl[h] = l;
        size[g] = 0;
        return;
    }
    const uint32_t a = f + 1, b = f + (l - f) / 2, c = l - 1;
    uint32_t pick;
    if (kless_at(k, a, b)) {
        if (kless_at(k, b, c)) pick = b;
        else if (kless_at(k, a, c)) pick = c;
        else pick = a;
    } else if (kless_at(k, a, c)) {
        pick = a;
    } else if (kless_at(k, b, c)) {
        pick = c;
    } else {
        pick = b;
    }
    kswap(k, f, pick);
    pk[3 * g] = k.w0[f];
    pk[3 * g + 1] = k.w1[f];
    pk[3 * g + 2] = k.w2[f];
    size[g] = l - f;
}

__device__ __forceinline__ uint32_t seg_of(const uint32_t *off, uint32_t ns, uint32_t j) {
    uint32_t lo = 0, hi = ns;  // last g with off[g] <= j
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) / 2;
        if (off[mid] <= j) lo = mid;
        else hi = mid;
    }
    return lo;
}

// flags of every element of the live ranges (>= pivot, <= pivot) and a copy of it
__global__ void k_flags(uint32_t total, uint32_t ns, const uint32_t *off, const uint32_t *sf, const uint32_t *pk, Keys k, Keys tmp,
                        uint32_t *ge, uint32_t *le) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= total) return;
    const uint32_t g = seg_of(off, ns, j);
    const uint32_t p = sf[g] + (j - off[g]);
    const uint32_t a0 = k.w0[p], a1 = k.w1[p], a2 = k.w2[p];
    tmp.w0[j] = a0; tmp.w1[j] = a1; tmp.w2[j] = a2; tmp.ix[j] = k.ix[p];
    if (p == sf[g]) {  // the pivot itself is outside the partitioned range
        ge[j] = 0;
        le[j] = 0;
        return;
    }
    const uint32_t p0 = pk[3 * g], p1 = pk[3 * g + 1], p2 = pk[3 * g + 2];
    ge[j] = kless(a0, a1, a2, p0, p1, p2) ? 0u : 1u;
    le[j] = kless(p0, p1, p2, a0, a1, a2) ? 0u : 1u;
}

// A(x) = #ge in local [1, x), B(x) = #le in local [x, sz); pge/ple are exclusive prefix sums
// over the live elements with one extra entry at the end.
struct Counts {
    const uint32_t *pge, *ple;
    uint32_t j0, sz;
    __device__ uint32_t A(uint32_t x) const { return pge[j0 + x] - pge[j0 + 1]; }
    __device__ uint32_t B(uint32_t x) const { return ple[j0 + sz] - ple[j0 + x]; }
    // local position of the k-th (1-based) element >= pivot from the left, or sz
    __device__ uint32_t left(uint32_t kk) const {
        if (A(sz) < kk) return sz;
        uint32_t lo = 1, hi = sz;  // smallest x with A(x) >= kk, then x - 1
        while (lo < hi) {
            uint32_t mid = (lo + hi) / 2;
            if (A(mid) >= kk) hi = mid;
            else lo = mid + 1;
        }
        return lo - 1;
    }
    // local position of the k-th (1-based) element <= pivot from the right
    __device__ uint32_t right(uint32_t kk) const {
        uint32_t lo = 1, hi = sz - 1;  // largest x with B(x) >= kk
        while (lo < hi) {
            uint32_t mid = (lo + hi + 1) / 2;
            if (B(mid) >= kk) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    }
};

// number of swaps and the cut of every live range
__global__ void k_cut(uint32_t ns, const uint32_t *off, const uint32_t *sf, const uint32_t *size, const uint32_t *pge, const uint32_t *ple,
                      uint32_t *mswap, uint32_t *cut, unsigned *err) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ns) return;
    const uint32_t sz = size[g];
    if (sz == 0) return;
    Counts cn{pge, ple, off[g], sz};
    // largest x in [1, sz] with A(x) <= B(x) (A - B is nondecreasing)
    uint32_t lo = 1, hi = sz;
    if (cn.A(1) > cn.B(1)) {
        hi = 1;
    } else {
        while (lo < hi) {
            uint32_t mid = (lo + hi + 1) / 2;
            if (cn.A(mid) <= cn.B(mid)) lo = mid;
            else hi = mid - 1;
        }
    }
    uint32_t m = min(cn.A(lo), cn.B(lo));
    if (lo + 1 <= sz) m = max(m, min(cn.A(lo + 1), cn.B(lo + 1)));
    uint32_t c;
    if (m == 0) {
        c = cn.left(1);
    } else {
        c = min(cn.left(m + 1), cn.right(m));
    }
    if (c == 0 || c >= sz) {  // the median-of-three guarantees an inner cut
        atomicOr(err, (unsigned)kDevErrLoopLimit);
        c = min(max(c, 1u), sz - 1);
    }
    mswap[g] = m;
    cut[g] = sf[g] + c;
}

// the swaps of every live range: L_k <-> R_k for k <= m
__global__ void k_swap(uint32_t total, uint32_t ns, const uint32_t *off, const uint32_t *sf, const uint32_t *size, const uint32_t *pge,
                       const uint32_t *ple, const uint32_t *ge, const uint32_t *le, const uint32_t *mswap, Keys tmp, Keys k) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= total) return;
    const uint32_t g = seg_of(off, ns, j);
    const uint32_t sz = size[g];
    if (sz == 0) return;
    const uint32_t x = j - off[g], m = mswap[g];
    Counts cn{pge, ple, off[g], sz};
    uint32_t dest = x;
    if (ge[j] && cn.A(x) + 1 <= m) dest = cn.right(cn.A(x) + 1);
    else if (le[j] && cn.B(x + 1) + 1 <= m) dest = cn.left(cn.B(x + 1) + 1);
    if (dest == x) return;
    const uint32_t p = sf[g] + dest;
    k.w0[p] = tmp.w0[j]; k.w1[p] = tmp.w1[j]; k.w2[p] = tmp.w2[j]; k.ix[p] = tmp.ix[j];
}

// children [first, cut) and [cut, last) with one less depth; ranges of <= 16 are final
__global__ void k_children(uint32_t ns, const uint32_t *sf, const uint32_t *sl, const uint32_t *sd, const uint32_t *size,
                           const uint32_t *cut, uint32_t *nf, uint32_t *nl, uint32_t *nd, uint32_t *nn) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ns || size[g] == 0) return;
    const uint32_t f = sf[g], l = sl[g], c = cut[g], d = sd[g] - 1;
    if (l - c > kThreshold) {
        uint32_t o = atomicAdd(nn, 1u);
        nf[o] = c; nl[o] = l; nd[o] = d;
    }
    if (c - f > kThreshold) {
        uint32_t o = atomicAdd(nn, 1u);
        nf[o] = f; nl[o] = c; nd[o] = d;
    }
}

// __partial_sort(first, last, last) = __make_heap + __sort_heap, one thread per range
__device__ void heap_adjust(const Keys &k, uint32_t f, uint32_t hole, uint32_t len, uint32_t v0, uint32_t v1, uint32_t v2, uint32_t vi) {
    const uint32_t top = hole;
    uint32_t child = hole;
    auto mv = [&](uint32_t dst, uint32_t src) {
        k.w0[f + dst] = k.w0[f + src]; k.w1[f + dst] = k.w1[f + src]; k.w2[f + dst] = k.w2[f + src]; k.ix[f + dst] = k.ix[f + src];
    };
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (kless_at(k, f + child, f + child - 1)) child--;
        mv(hole, child);
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        mv(hole, child - 1);
        hole = child - 1;
    }
    // __push_heap(first, hole, top, value)
    uint32_t parent = (hole - 1) / 2;
    while (hole > top && kless(k.w0[f + parent], k.w1[f + parent], k.w2[f + parent], v0, v1, v2)) {
        mv(hole, parent);
        hole = parent;
        parent = (hole - 1) / 2;
    }
    k.w0[f + hole] = v0; k.w1[f + hole] = v1; k.w2[f + hole] = v2; k.ix[f + hole] = vi;
}

__global__ void k_heapsort(uint32_t nh, const uint32_t *hf, const uint32_t *hl, Keys k) {
    uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    const uint32_t f = hf[h], len = hl[h] - f;
    if (len < 2) return;
    for (uint32_t parent = (len - 2) / 2;; --parent) {  // __make_heap
        heap_adjust(k, f, parent, len, k.w0[f + parent], k.w1[f + parent], k.w2[f + parent], k.ix[f + parent]);
        if (parent == 0) break;
    }
    for (uint32_t last = len; last > 1;) {  // __sort_heap: __pop_heap(first, last-1, last-1)
        --last;
        uint32_t v0 = k.w0[f + last], v1 = k.w1[f + last], v2 = k.w2[f + last], vi = k.ix[f + last];
        k.w0[f + last] = k.w0[f]; k.w1[f + last] = k.w1[f]; k.w2[f + last] = k.w2[f]; k.ix[f + last] = k.ix[f];
        heap_adjust(k, f, 0, last, v0, v1, v2, vi);
    }
}

uint32_t floor_log2(uint32_t n) { return 31u - (uint32_t)__builtin_clz(n); }

}  // namespace

size_t morton_sort_scratch_bytes(size_t n) {
    const size_t segs = n / kThreshold + 4;
    size_t b = 0;
    auto add = [&](size_t bytes) { b += (bytes + 255) & ~size_t(255); };
    for (int i = 0; i < 4; ++i) add(n * 4);             // tmp keys
    for (int i = 0; i < 4; ++i) add((n + 1) * 4);       // ge, le, pge, ple
    for (int i = 0; i < 8; ++i) add(segs * 4);          // two range tables (first, last, depth) + size/off
    for (int i = 0; i < 4; ++i) add(segs * 4);          // pivots (3) , cut, m
    add(segs * 12);
    for (int i = 0; i < 2; ++i) add(segs * 4);          // heap list
    add(64);
    b += std::max(scan_u32_scratch_bytes(n + 1), radix_sort96_scratch_bytes(n));
    return b + 4096;
}

int morton_sort_std(Context &c, uint32_t *w0, uint32_t *w1, uint32_t *w2, uint32_t *ix, uint32_t n, void *scratch, size_t bytes,
                    cudaStream_t s) {
    if (n <= 1) return kOk;
    if (bytes < morton_sort_scratch_bytes(n)) return kErrOutOfMemory;
    unsigned char *p = static_cast<unsigned char *>(scratch);
    auto take = [&](size_t b) {
        void *r = p;
        p += (b + 255) & ~size_t(255);
        return r;
    };
    const size_t segs = n / kThreshold + 4;
    Keys k{w0, w1, w2, ix};
    Keys tmp{(uint32_t *)take(n * 4), (uint32_t *)take(n * 4), (uint32_t *)take(n * 4), (uint32_t *)take(n * 4)};
    uint32_t *ge = (uint32_t *)take((n + 1) * 4), *le = (uint32_t *)take((n + 1) * 4);
    uint32_t *pge = (uint32_t *)take((n + 1) * 4), *ple = (uint32_t *)take((n + 1) * 4);
    uint32_t *sf[2], *sl[2], *sd[2];
    for (int t = 0; t < 2; ++t) {
        sf[t] = (uint32_t *)take(segs * 4);
        sl[t] = (uint32_t *)take(segs * 4);
        sd[t] = (uint32_t *)take(segs * 4);
    }
    uint32_t *size = (uint32_t *)take(segs * 4), *off = (uint32_t *)take(segs * 4);
    uint32_t *cut = (uint32_t *)take(segs * 4), *mswap = (uint32_t *)take(segs * 4);
    uint32_t *pk = (uint32_t *)take(segs * 12);
    uint32_t *hf = (uint32_t *)take(segs * 4), *hl = (uint32_t *)take(segs * 4);
    uint32_t *cnt = (uint32_t *)take(64);  // [0] next ranges, [1] heap ranges, [2] total, [3] scratch total
    const size_t sb = std::max(scan_u32_scratch_bytes(n + 1), radix_sort96_scratch_bytes(n));
    void *scr = take(sb);

    PLAN_CUDA(cudaMemsetAsync(cnt, 0, 64, s));
    uint32_t ns = 0;
    if (n > kThreshold) {
        uint32_t h3[3] = {0, n, 2 * floor_log2(n)};
        PLAN_CUDA(cudaMemcpyAsync(sf[0], &h3[0], 4, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(sl[0], &h3[1], 4, cudaMemcpyHostToDevice, s));
        PLAN_CUDA(cudaMemcpyAsync(sd[0], &h3[2], 4, cudaMemcpyHostToDevice, s));
        ns = 1;
    }
    int cur = 0;
    for (uint32_t level = 0; ns > 0; ++level) {
        if (level > 2 * 32 + 2) return kErrDeviceLimit;  // the depth budget bounds the levels
        const int nx = 1 - cur;
        const unsigned gs = (ns + 255) / 256;
        k_pivot<<<gs, 256, 0, s>>>(ns, sf[cur], sl[cur], sd[cur], k, size, pk, hf, hl, cnt + 1);
        int rc = scan_u32(size, off, ns, cnt + 2, scr, sb, s);
        if (rc) return rc;
        uint32_t total = 0;
        PLAN_CUDA(cudaMemcpyAsync(&total, cnt + 2, 4, cudaMemcpyDeviceToHost, s));
        PLAN_CUDA(cudaStreamSynchronize(s));
        c.launches += 4;
        if (total) {
            const unsigned ge_blocks = (total + 255) / 256;
            k_flags<<<ge_blocks, 256, 0, s>>>(total, ns, off, sf[cur], pk, k, tmp, ge, le);
            PLAN_CUDA(cudaMemsetAsync(ge + total, 0, 4, s));
            PLAN_CUDA(cudaMemsetAsync(le + total, 0, 4, s));
            rc = scan_u32(ge, pge, total + 1, nullptr, scr, sb, s);
            if (!rc) rc = scan_u32(le, ple, total + 1, nullptr, scr, sb, s);
            if (rc) return rc;
            k_cut<<<gs, 256, 0, s>>>(ns, off, sf[cur], size, pge, ple, mswap, cut, c.d_err);
            k_swap<<<ge_blocks, 256, 0, s>>>(total, ns, off, sf[cur], size, pge, ple, ge, le, mswap, tmp, k);
            PLAN_CUDA(cudaMemsetAsync(cnt, 0, 4, s));
            k_children<<<gs, 256, 0, s>>>(ns, sf[cur], sl[cur], sd[cur], size, cut, sf[nx], sl[nx], sd[nx], cnt);
            c.launches += 10;
            PLAN_CUDA(cudaGetLastError());
            PLAN_CUDA(cudaMemcpyAsync(&ns, cnt, 4, cudaMemcpyDeviceToHost, s));
            PLAN_CUDA(cudaStreamSynchronize(s));
        } else {
            ns = 0;
        }
        cur = nx;
    }
    uint32_t nh = 0;
    PLAN_CUDA(cudaMemcpyAsync(&nh, cnt + 1, 4, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    if (nh) {
        k_heapsort<<<(nh + 127) / 128, 128, 0, s>>>(nh, hf, hl, k);
        c.launches++;
    }
    // the final insertion sort keeps equal keys in place: a stable sort finishes
    int rc = radix_sort96(w0, w1, w2, ix, n, scr, sb, s);
    if (rc) return rc;
    c.launches += 36;
    PLAN_CUDA(cudaGetLastError());
    return kOk;
}

}  // namespace plan
