// Per-point rules of the octree built from sorted Morton keys, host+device (front.cu builds
// the tree on the GPU with them; the parity tests run them on the CPU against the oracle's
// tree, with both leaf sizes).
//
// BuildTree (src/tree.hpp:2655-2755) splits a node while it holds more than max_leaf_size
// points and is above the last level. With the points in key order, the node at digit level
// L containing point i is internal iff some run of max_leaf_size + 1 consecutive keys around
// i shares L digits; point i starts a node at level L iff it shares fewer than L digits with
// the point before it and L is not below its leaf level.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace plan {

// digits shared with the previous key (0 for the first point), at most 31
__host__ __device__ inline uint8_t octree_prev_lcp(const uint32_t *k0, const uint32_t *k1, const uint32_t *k2, uint32_t i) {
    int a = 0;
    if (i > 0) a = key_lcp_digits(k0[i - 1], k1[i - 1], k2[i - 1], k0[i], k1[i], k2[i]);
    return (uint8_t)(a < 31 ? a : 31);
}

// digits shared by the (LEAF + 1)-key window starting at i (its first and last key), at most
// 31; 255 when the window runs past the end
template <uint32_t LEAF>
__host__ __device__ inline uint8_t octree_window_lcp(const uint32_t *k0, const uint32_t *k1, const uint32_t *k2, uint32_t n, uint32_t i) {
    if (i + LEAF >= n) return 255;
    const int w = key_lcp_digits(k0[i], k1[i], k2[i], k0[i + LEAF], k1[i + LEAF], k2[i + LEAF]);
    return (uint8_t)(w < 31 ? w : 31);
}

// the leaf's digit level for point i: one below the deepest level some window holding i shares
template <uint32_t LEAF>
__host__ __device__ inline uint8_t octree_leaf_level(const uint8_t *win, uint32_t i) {
    int M = 0;
    const uint32_t j0 = i >= LEAF ? i - LEAF : 0;
    for (uint32_t j = j0; j <= i; ++j) {
        const uint8_t w = win[j];
        if (w != 255 && w > M) M = w;
    }
    return (uint8_t)(M + 1 < 31 ? M + 1 : 31);
}

// point i (shared prefix a with its predecessor, leaf level l) starts a node at level L
__host__ __device__ inline bool starts_level(int L, int a, int l) { return L > a && L <= l; }

}  // namespace plan
