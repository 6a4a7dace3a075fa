// Exclusive prefix sum of u32 values: block sums, a scan of the block sums, then a
// block-local scan with the block's carry added.
#include "sort.h"

namespace plan {

namespace {

constexpr int kT = 1024;
constexpr int kPer = 4;
constexpr int kChunk = kT * kPer;

__device__ uint32_t block_exclusive(uint32_t v, uint32_t *s_warp, uint32_t &total) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (int)(blockDim.x / 32) ? s_warp[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t excl = x - v + (warp > 0 ? s_warp[warp - 1] : 0);
    total = s_warp[blockDim.x / 32 - 1];
    __syncthreads();
    return excl;
}

__global__ void k_chunk_sums(const uint32_t *in, size_t n, uint32_t *sums) {
    __shared__ uint32_t s_warp[32];
    size_t base = (size_t)blockIdx.x * kChunk + (size_t)threadIdx.x * kPer;
    uint32_t v = 0;
    for (int k = 0; k < kPer; ++k) if (base + k < n) v += in[base + k];
    uint32_t tot;
    block_exclusive(v, s_warp, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// single block: exclusive scan of the chunk sums, grand total to d_total
__global__ void k_scan_sums(uint32_t *sums, size_t m, uint32_t *d_total) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (size_t start = 0; start < m; start += blockDim.x) {
        size_t t = start + threadIdx.x;
        uint32_t v = t < m ? sums[t] : 0;
        uint32_t tot;
        uint32_t e = block_exclusive(v, s_warp, tot);
        uint32_t c = carry;
        if (t < m) sums[t] = e + c;
        __syncthreads();
        if (threadIdx.x == 0) carry = c + tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && d_total) *d_total = carry;
}

__global__ void k_chunk_scan(const uint32_t *in, uint32_t *out, size_t n, const uint32_t *sums) {
    __shared__ uint32_t s_warp[32];
    size_t base = (size_t)blockIdx.x * kChunk + (size_t)threadIdx.x * kPer;
    uint32_t v[kPer], s = 0;
    for (int k = 0; k < kPer; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    uint32_t tot;
    uint32_t e = block_exclusive(s, s_warp, tot) + sums[blockIdx.x];
    for (int k = 0; k < kPer; ++k) {
        if (base + k < n) out[base + k] = e;
        e += v[k];
    }
}

}  // namespace

size_t scan_u32_scratch_bytes(size_t n) { return ((n + kChunk - 1) / kChunk + 1) * sizeof(uint32_t) + 256; }

int scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *d_total, void *scratch, size_t scratch_bytes, cudaStream_t stream) {
    if (scratch_bytes < scan_u32_scratch_bytes(n)) return kErrArgument;
    if (n == 0) {
        if (d_total) PLAN_CUDA(cudaMemsetAsync(d_total, 0, 4, stream));
        return kOk;
    }
    size_t m = (n + kChunk - 1) / kChunk;
    uint32_t *sums = static_cast<uint32_t *>(scratch);
    k_chunk_sums<<<(unsigned)m, kT, 0, stream>>>(in, n, sums);
    k_scan_sums<<<1, kT, 0, stream>>>(sums, m, d_total);
    k_chunk_scan<<<(unsigned)m, kT, 0, stream>>>(in, out, n, sums);
    PLAN_CUDA(cudaGetLastError());
    return kOk;
}

}  // namespace plan
