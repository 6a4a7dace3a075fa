// The order std::sort (GCC's libstdc++) leaves a sequence of (distance, member) pairs in, when
// pairs compare by distance alone: one thread, sequential, in place.
//
// The reference sorts clump members by their distance from the centre of mass with an
// unstable std::sort (src/tree.hpp:4451-4453, 4548-4550). Where two members of one clump lie at
// exactly the same distance, their final order is whatever the library's introsort leaves, and
// that order reaches the catalogue (member lists, the median member, swap-with-back
// removals). Clumps of at most 16 members are insertion-sorted by the library, which keeps
// ties in order, so a stable sort agrees there; longer ones with a tie are re-sorted here.
//
// The steps restate the library's documented algorithm (introsort: median-of-three pivot
// moved to the front, unguarded Hoare partition, depth limit 2 floor(log2 n), heap sort when
// the limit is reached, final insertion sort with a threshold of 16), in our own code; the
// parity tests compare it with std::sort on the CPU, ties included.
//
// Host-compilable for those tests.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define PLAN_LS_HD __host__ __device__
#else
#define PLAN_LS_HD
#endif

namespace plan {

struct LibSortSeq {
    double *key;
    uint32_t *val;
    PLAN_LS_HD bool less(int64_t a, int64_t b) const { return key[a] < key[b]; }
    PLAN_LS_HD void swap(int64_t a, int64_t b) const {
        const double k = key[a];
        key[a] = key[b];
        key[b] = k;
        const uint32_t v = val[a];
        val[a] = val[b];
        val[b] = v;
    }
    PLAN_LS_HD void move(int64_t to, int64_t from) const {
        key[to] = key[from];
        val[to] = val[from];
    }
};

namespace libsort_detail {

constexpr int64_t kThreshold = 16;

// sift the hole at `hole` down to a leaf, then push (vk, vv) up from there, not above `top`
PLAN_LS_HD inline void adjust_heap(const LibSortSeq &s, int64_t first, int64_t hole, int64_t len, double vk, uint32_t vv) {
    const int64_t top = hole;
    int64_t child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (s.key[first + child] < s.key[first + child - 1]) child--;
        s.move(first + hole, first + child);
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        s.move(first + hole, first + child - 1);
        hole = child - 1;
    }
    int64_t parent = (hole - 1) / 2;
    while (hole > top && s.key[first + parent] < vk) {
        s.move(first + hole, first + parent);
        hole = parent;
        parent = (hole - 1) / 2;
    }
    s.key[first + hole] = vk;
    s.val[first + hole] = vv;
}

// heap sort of [first, last): build a max-heap, then pop to the back
PLAN_LS_HD inline void heap_sort(const LibSortSeq &s, int64_t first, int64_t last) {
    const int64_t len = last - first;
    if (len >= 2) {
        for (int64_t parent = (len - 2) / 2;; --parent) {
            adjust_heap(s, first, parent, len, s.key[first + parent], s.val[first + parent]);
            if (parent == 0) break;
        }
    }
    while (last - first > 1) {
        --last;
        const double vk = s.key[last];
        const uint32_t vv = s.val[last];
        s.move(last, first);
        adjust_heap(s, first, 0, last - first, vk, vv);
    }
}

// put the median of a, b, c at `result`
PLAN_LS_HD inline void median_to_first(const LibSortSeq &s, int64_t result, int64_t a, int64_t b, int64_t c) {
    if (s.less(a, b)) {
        if (s.less(b, c)) s.swap(result, b);
        else if (s.less(a, c)) s.swap(result, c);
        else s.swap(result, a);
    } else if (s.less(a, c)) {
        s.swap(result, a);
    } else if (s.less(b, c)) {
        s.swap(result, c);
    } else {
        s.swap(result, b);
    }
}

PLAN_LS_HD inline int64_t partition_pivot(const LibSortSeq &s, int64_t first, int64_t last) {
    const int64_t mid = first + (last - first) / 2;
    median_to_first(s, first, first + 1, mid, last - 1);
    int64_t lo = first + 1, hi = last;
    const int64_t pivot = first;
    // the library's scans are unguarded (the median-of-three leaves a sentinel at each end);
    // the range checks here never stop a scan early on a strict weak order and keep a NaN
    // key from walking outside the range
    while (true) {
        while (lo < last && s.less(lo, pivot)) ++lo;
        --hi;
        while (hi > first && s.less(pivot, hi)) --hi;
        if (!(lo < hi)) return lo;
        s.swap(lo, hi);
        ++lo;
    }
}

PLAN_LS_HD inline void linear_insert(const LibSortSeq &s, int64_t at) {
    const double vk = s.key[at];
    const uint32_t vv = s.val[at];
    int64_t next = at - 1;
    while (next >= 0 && vk < s.key[next]) {  // unguarded in the library: key[0] is the minimum
        s.move(at, next);
        at = next;
        --next;
    }
    s.key[at] = vk;
    s.val[at] = vv;
}

PLAN_LS_HD inline void insertion_sort(const LibSortSeq &s, int64_t first, int64_t last) {
    if (first == last) return;
    for (int64_t i = first + 1; i != last; ++i) {
        if (s.key[i] < s.key[first]) {
            const double vk = s.key[i];
            const uint32_t vv = s.val[i];
            for (int64_t j = i; j > first; --j) s.move(j, j - 1);
            s.key[first] = vk;
            s.val[first] = vv;
        } else {
            linear_insert(s, i);
        }
    }
}

PLAN_LS_HD inline int floor_log2(int64_t n) {
    int k = 0;
    while (n > 1) {
        n >>= 1;
        ++k;
    }
    return k;
}

}  // namespace libsort_detail

// std::sort of key[0, n) (payload val moves with it), comparing keys with <; n < 2^32
PLAN_LS_HD inline void lib_sort(double *key, uint32_t *val, int64_t n) {
    using namespace libsort_detail;
    if (n < 2) return;
    const LibSortSeq s{key, val};
    // The introsort loop. The library recurses into the right part of each partition and
    // continues with the left one; the two parts are disjoint and each one's result depends
    // only on its own elements and depth, so the right parts can wait on a stack. Entries
    // are pushed with strictly decreasing depths above any entry below them, so the stack
    // never holds more than 2 floor(log2 n) + 1 <= 64 ranges.
    struct Range {
        uint32_t first, last;  // n < 2^32
        int32_t depth;
    };
    Range stack[66];
    int top = 0;
    stack[top++] = Range{0u, (uint32_t)n, 2 * floor_log2(n)};
    while (top > 0) {
        const Range r = stack[--top];
        int64_t first = r.first, last = r.last;
        int depth = r.depth;
        while (last - first > kThreshold) {
            if (depth == 0) {
                heap_sort(s, first, last);
                break;
            }
            --depth;
            const int64_t cut = partition_pivot(s, first, last);
            stack[top++] = Range{(uint32_t)cut, (uint32_t)last, depth};
            last = cut;
        }
    }
    // final insertion sort
    if (n > kThreshold) {
        insertion_sort(s, 0, kThreshold);
        for (int64_t i = kThreshold; i < n; ++i) linear_insert(s, i);
    } else {
        insertion_sort(s, 0, n);
    }
}

}  // namespace plan
