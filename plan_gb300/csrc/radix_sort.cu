// Stable LSD radix sort of 96-bit keys (three u32 words) with a u32 payload.
//
// One sort primitive serves three uses: Morton keys (src/tree.hpp:2831), the HOP group
// order (root, first-visit index, chain position) and per-clump distance orders
// (clump slot, distance bits). 8-bit digits, 12 passes at most; a pre-pass computes all
// twelve digit histograms in one read and passes whose digit is constant are skipped.
// Each pass is reduce-then-scan: per-tile digit counts, a per-digit scan over tiles, and a
// stable scatter that ranks keys within a tile with warp match masks.
#include "sort.h"

#include <cstdio>

namespace plan {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;  // 2048 keys per tile
constexpr int kRadix = 256;

__device__ __forceinline__ uint32_t digit_of(const uint32_t *w0, const uint32_t *w1, const uint32_t *w2, size_t i, int pass) {
    int word = pass >> 2, shift = (pass & 3) * 8;
    uint32_t v = word == 0 ? w0[i] : (word == 1 ? w1[i] : w2[i]);
    return (v >> shift) & 0xffu;
}

// All 12 digit histograms in one pass over the keys.
__global__ void k_hist_all(const uint32_t *w0, const uint32_t *w1, const uint32_t *w2, size_t n, unsigned long long *hist /*12*256*/) {
    __shared__ unsigned int s[12 * kRadix];
    for (int j = threadIdx.x; j < 12 * kRadix; j += blockDim.x) s[j] = 0;
    __syncthreads();
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t a = w0[i], b = w1[i], c = w2[i];
        for (int k = 0; k < 4; ++k) {
            atomicAdd(&s[(0 + k) * kRadix + ((a >> (8 * k)) & 0xff)], 1u);
            atomicAdd(&s[(4 + k) * kRadix + ((b >> (8 * k)) & 0xff)], 1u);
            atomicAdd(&s[(8 + k) * kRadix + ((c >> (8 * k)) & 0xff)], 1u);
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < 12 * kRadix; j += blockDim.x)
        if (s[j]) atomicAdd(&hist[j], (unsigned long long)s[j]);
}

// Per-tile digit counts: counts[digit * ntiles + tile].
__global__ void k_tile_counts(const uint32_t *w0, const uint32_t *w1, const uint32_t *w2, size_t n, int pass, uint32_t *counts, int ntiles) {
    __shared__ unsigned int s[kRadix];
    for (int j = threadIdx.x; j < kRadix; j += blockDim.x) s[j] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * kTile;
    for (int r = 0; r < kItems; ++r) {
        size_t i = base + (size_t)r * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&s[digit_of(w0, w1, w2, i, pass)], 1u);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kRadix; j += blockDim.x) counts[(size_t)j * ntiles + blockIdx.x] = s[j];
}

// Exclusive scan of counts[digit][*] over tiles plus the digit's global base.
// One block per digit.
__global__ void k_scan_tiles(uint32_t *counts, int ntiles, const unsigned long long *digit_base) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    int d = blockIdx.x;
    uint32_t *row = counts + (size_t)d * ntiles;
    if (threadIdx.x == 0) carry = (uint32_t)digit_base[d];
    __syncthreads();
    for (int start = 0; start < ntiles; start += blockDim.x) {
        int t = start + threadIdx.x;
        uint32_t v = t < ntiles ? row[t] : 0;
        // inclusive warp scan
        uint32_t x = v;
        int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int nw = blockDim.x / 32;
            uint32_t w = lane < nw ? warp_sums[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            if (lane < nw) warp_sums[lane] = w;
        }
        __syncthreads();
        uint32_t prefix = x - v + (warp > 0 ? warp_sums[warp - 1] : 0) + carry;
        if (t < ntiles) row[t] = prefix;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = prefix + v;
        __syncthreads();
    }
}

// Stable scatter of one tile. Items are taken round-major (item r*256 + t), and within a
// round ranks follow lane then warp order, so the tile's input order is preserved.
__global__ void k_scatter(const uint32_t *w0, const uint32_t *w1, const uint32_t *w2, const uint32_t *pay, uint32_t *o0, uint32_t *o1,
                          uint32_t *o2, uint32_t *op, size_t n, int pass, const uint32_t *counts, int ntiles) {
    __shared__ uint32_t s_off[kRadix];          // running position per digit for this tile
    __shared__ uint32_t s_w[kThreads / 32][kRadix];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j = threadIdx.x; j < kRadix; j += blockDim.x) s_off[j] = counts[(size_t)j * ntiles + blockIdx.x];
    size_t base = (size_t)blockIdx.x * kTile;
    for (int r = 0; r < kItems; ++r) {
        for (int j = threadIdx.x; j < (kThreads / 32) * kRadix; j += blockDim.x) (&s_w[0][0])[j] = 0;
        __syncthreads();
        size_t i = base + (size_t)r * kThreads + threadIdx.x;
        bool valid = i < n;
        uint32_t dg = valid ? digit_of(w0, w1, w2, i, pass) : 0xffffffffu;
        unsigned peers = __match_any_sync(0xffffffffu, dg);
        unsigned lt = (1u << lane) - 1u;
        int rank_in_warp = __popc(peers & lt);
        int leader = __ffs(peers) - 1;
        if (valid && lane == leader) s_w[warp][dg] = __popc(peers);
        __syncthreads();
        // per digit: exclusive scan over warps, seeded with the running tile offset
        for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
            uint32_t run = s_off[d];
            for (int w = 0; w < kThreads / 32; ++w) {
                uint32_t c = s_w[w][d];
                s_w[w][d] = run;
                run += c;
            }
            s_off[d] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = s_w[warp][dg] + rank_in_warp;
            o0[pos] = w0[i];
            o1[pos] = w1[i];
            o2[pos] = w2[i];
            op[pos] = pay[i];
        }
        __syncthreads();
    }
}

}  // namespace

size_t radix_sort96_scratch_bytes(size_t n) {
    size_t ntiles = (n + kTile - 1) / kTile;
    size_t b = 4 * n * sizeof(uint32_t);                 // ping-pong buffers
    b += (size_t)kRadix * ntiles * sizeof(uint32_t);    // tile counts
    b += 12 * kRadix * sizeof(unsigned long long);       // histograms
    return b + 4096;
}

int radix_sort96(uint32_t *w0, uint32_t *w1, uint32_t *w2, uint32_t *payload, size_t n, void *scratch, size_t scratch_bytes,
                 cudaStream_t stream, unsigned pass_mask) {
    if (n <= 1) return kOk;
    if (scratch_bytes < radix_sort96_scratch_bytes(n)) return kErrArgument;
    size_t ntiles = (n + kTile - 1) / kTile;
    char *p = static_cast<char *>(scratch);
    uint32_t *b0 = reinterpret_cast<uint32_t *>(p); p += n * 4;
    uint32_t *b1 = reinterpret_cast<uint32_t *>(p); p += n * 4;
    uint32_t *b2 = reinterpret_cast<uint32_t *>(p); p += n * 4;
    uint32_t *bp = reinterpret_cast<uint32_t *>(p); p += n * 4;
    uint32_t *counts = reinterpret_cast<uint32_t *>(p); p += (size_t)kRadix * ntiles * 4;
    p = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
    unsigned long long *hist = reinterpret_cast<unsigned long long *>(p);

    PLAN_CUDA(cudaMemsetAsync(hist, 0, 12 * kRadix * sizeof(unsigned long long), stream));
    int hblocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_hist_all<<<hblocks, 256, 0, stream>>>(w0, w1, w2, n, hist);
    PLAN_CUDA(cudaGetLastError());
    unsigned long long h_hist[12 * kRadix];
    PLAN_CUDA(cudaMemcpyAsync(h_hist, hist, sizeof(h_hist), cudaMemcpyDeviceToHost, stream));
    PLAN_CUDA(cudaStreamSynchronize(stream));
    // digit bases (exclusive prefix per pass), uploaded in place of the histogram
    unsigned long long h_base[12 * kRadix];
    bool skip[12];
    for (int pass = 0; pass < 12; ++pass) {
        unsigned long long run = 0;
        skip[pass] = !((pass_mask >> pass) & 1u);
        for (int d = 0; d < kRadix; ++d) {
            unsigned long long c = h_hist[pass * kRadix + d];
            if (c == n) skip[pass] = true;
            h_base[pass * kRadix + d] = run;
            run += c;
        }
    }
    PLAN_CUDA(cudaMemcpyAsync(hist, h_base, sizeof(h_base), cudaMemcpyHostToDevice, stream));
    uint32_t *src[4] = {w0, w1, w2, payload}, *dst[4] = {b0, b1, b2, bp};
    int done = 0;
    for (int pass = 0; pass < 12; ++pass) {
        if (skip[pass]) continue;
        k_tile_counts<<<(int)ntiles, kThreads, 0, stream>>>(src[0], src[1], src[2], n, pass, counts, (int)ntiles);
        k_scan_tiles<<<kRadix, 1024, 0, stream>>>(counts, (int)ntiles, hist + pass * kRadix);
        k_scatter<<<(int)ntiles, kThreads, 0, stream>>>(src[0], src[1], src[2], src[3], dst[0], dst[1], dst[2], dst[3], n, pass, counts, (int)ntiles);
        PLAN_CUDA(cudaGetLastError());
        for (int k = 0; k < 4; ++k) std::swap(src[k], dst[k]);
        ++done;
    }
    if (src[0] != w0) {  // odd number of passes: copy back
        PLAN_CUDA(cudaMemcpyAsync(w0, src[0], n * 4, cudaMemcpyDeviceToDevice, stream));
        PLAN_CUDA(cudaMemcpyAsync(w1, src[1], n * 4, cudaMemcpyDeviceToDevice, stream));
        PLAN_CUDA(cudaMemcpyAsync(w2, src[2], n * 4, cudaMemcpyDeviceToDevice, stream));
        PLAN_CUDA(cudaMemcpyAsync(payload, src[3], n * 4, cudaMemcpyDeviceToDevice, stream));
    }
    (void)done;
    return kOk;
}

}  // namespace plan
