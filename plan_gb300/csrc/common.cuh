// Shared device helpers for the GB300 clump finder.
//
// Floating point: every translation unit is compiled with --fmad=false, so a*b+c is two
// IEEE roundings exactly as in the reference's x86-64 SSE2 build; fused operations appear
// only where written explicitly (fma()). Double division and sqrt are IEEE-rounded on the
// GPU, matching the host.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace plan {

// ------------------------------------------------------------------ status codes
enum Status : int {
    kOk = 0,
    kErrArgument = 2,     // bad call (maps to the reference's exit(2))
    kErrIo = 3,           // unreadable file (exit(3))
    kErrParameter = 4,    // bad parameter (exit(4))
    kErrDevice = 5,       // CUDA error
    kErrOutOfMemory = 6,  // device allocation failed / admission refused
    kErrUnsupported = 7,  // input outside what this library handles (reported, never faked)
    kErrDeviceLimit = 8,  // a bounded device loop ran out (error flag set by a kernel)
};

#define PLAN_CUDA(call)                                                     \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) return ::plan::set_cuda_error(e_, #call, __FILE__, __LINE__); \
    } while (0)

int set_cuda_error(cudaError_t e, const char *what, const char *file, int line);

// A stream-ordered device allocation, freed on its stream when it leaves scope (so an early
// return on an error does not leak it).
template <class T>
struct StreamBuf {
    T *p = nullptr;
    cudaStream_t s;
    explicit StreamBuf(cudaStream_t st) : s(st) {}
    StreamBuf(const StreamBuf &) = delete;
    StreamBuf &operator=(const StreamBuf &) = delete;
    ~StreamBuf() {
        if (p) cudaFreeAsync(p, s);
    }
    cudaError_t alloc(size_t count) { return cudaMallocAsync(reinterpret_cast<void **>(&p), (count ? count : 1) * sizeof(T), s); }
};

// ------------------------------------------------------------------ device error flags
// Kernels never trap: a bounded loop that runs out, or an index that would leave its
// buffer, sets a bit here and returns; the host checks after the stage.
enum DevErr : unsigned {
    kDevErrStackOverflow = 1u << 0,
    kDevErrBadNode = 1u << 1,
    kDevErrHeapBound = 1u << 2,
    kDevErrLoopLimit = 1u << 3,
    kDevErrCapacity = 1u << 4,
    kDevErrKey2Leaf = 1u << 5,
};

// ------------------------------------------------------------------ Morton keys
// 96-bit key in three 32-bit words, w0 = bits 0..31. Digit at tree level L (1..32) is the
// 3-bit group at bit 93-3(L-1) (src/tree.hpp:2242-2245); bit 0 of a digit is x.
struct Key96 {
    uint32_t w0, w1, w2;
};

__host__ __device__ inline int key_digit(uint32_t w0, uint32_t w1, uint32_t w2, int level) {
    int shift = 93 - 3 * (level - 1);
    // gather 3 bits at `shift` from the 96-bit number
    unsigned __int128 k = ((unsigned __int128)w2 << 64) | ((unsigned __int128)w1 << 32) | w0;
    return (int)((k >> shift) & 7u);
}

// Number of leading equal 3-bit digits of two keys (0..32).
__host__ __device__ inline int key_lcp_digits(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t b0, uint32_t b1, uint32_t b2) {
    uint32_t x2 = a2 ^ b2, x1 = a1 ^ b1, x0 = a0 ^ b0;
    int lz;
#ifdef __CUDA_ARCH__
    if (x2) lz = __clz(x2);
    else if (x1) lz = 32 + __clz(x1);
    else if (x0) lz = 64 + __clz(x0);
    else lz = 96;
#else
    if (x2) lz = __builtin_clz(x2);
    else if (x1) lz = 32 + __builtin_clz(x1);
    else if (x0) lz = 64 + __builtin_clz(x0);
    else lz = 96;
#endif
    return lz / 3;
}

// round-to-nearest-even of d*(2^32-2) via the reference's magic-number trick
// (src/tree.cpp:106-113): two roundings, then the low 32 bits of the double's encoding.
__host__ __device__ inline uint32_t double_to_cell(double d) {
    double t = d * 4294967294.0;
    t = t + 6755399441055744.0;
#ifdef __CUDA_ARCH__
    return (uint32_t)(unsigned long long)__double_as_longlong(t);
#else
    uint64_t b;
    __builtin_memcpy(&b, &t, 8);
    return (uint32_t)b;
#endif
}

// Spread the bits of v three apart (bit b -> bit 3b) into a 96-bit value.
__host__ __device__ inline void dilate3(uint32_t v, uint32_t &o0, uint32_t &o1, uint32_t &o2) {
    uint64_t lo = 0, hi = 0;  // bits 0..63 and 64..95 of the result
    for (int b = 0; b < 32; ++b) {
        if ((v >> b) & 1u) {
            int p = 3 * b;
            if (p < 64) lo |= 1ull << p;
            else hi |= 1ull << (p - 64);
        }
    }
    o0 = (uint32_t)lo;
    o1 = (uint32_t)(lo >> 32);
    o2 = (uint32_t)hi;
}

// ------------------------------------------------------------------ exact-order heap
// Max-heap on dr2 with the hole-sifting order of the C++ library the reference is built
// with (libstdc++ __push_heap/__adjust_heap), so equal distances resolve exactly as in
// src/tree.hpp:3063-3075 and the final sort_heap order is the same. Entries live in a
// strided shared-memory slab: entry j of this thread at base[j*stride].
struct SlabHeap {
    double *d;
    uint32_t *ix;
    int stride;
    __device__ double dget(int j) const { return d[j * stride]; }
    __device__ uint32_t iget(int j) const { return ix[j * stride]; }
    __device__ void put(int j, double v, uint32_t i) { d[j * stride] = v; ix[j * stride] = i; }

    __device__ void push_hole(int hole, int top, double v, uint32_t vi) {
        int parent = (hole - 1) / 2;
        while (hole > top && dget(parent) < v) {
            put(hole, dget(parent), iget(parent));
            hole = parent;
            parent = (hole - 1) / 2;
        }
        put(hole, v, vi);
    }
    __device__ void adjust(int hole, int len, double v, uint32_t vi) {
        const int top = hole;
        int second = hole;
        while (second < (len - 1) / 2) {
            second = 2 * (second + 1);
            if (dget(second) < dget(second - 1)) second--;
            put(hole, dget(second), iget(second));
            hole = second;
        }
        if ((len & 1) == 0 && second == (len - 2) / 2) {
            second = 2 * (second + 1);
            put(hole, dget(second - 1), iget(second - 1));
            hole = second - 1;
        }
        push_hole(hole, top, v, vi);
    }
    // push_heap after appending (v, vi) at position len-1
    __device__ void push(int len, double v, uint32_t vi) { push_hole(len - 1, 0, v, vi); }
    // pop_heap on [0, len): the maximum moves to len-1
    __device__ void pop(int len) {
        if (len > 1) {
            double v = dget(len - 1);
            uint32_t vi = iget(len - 1);
            put(len - 1, dget(0), iget(0));
            adjust(0, len - 1, v, vi);
        }
    }
    // Add2Heaps: keep the k smallest, replacing the maximum only on a strictly smaller dr2
    __device__ void add(int &size, int k, uint32_t i, double dr2) {
        if (size < k) {
            ++size;
            push(size, dr2, i);
        } else if (dr2 < dget(0)) {
            pop(size);
            put(size - 1, dr2, i);  // pop_back + push_back
            push(size, dr2, i);
        }
    }
    __device__ void sort(int len) {
        while (len > 1) {
            pop(len);
            --len;
        }
    }
};

// ------------------------------------------------------------------ correctly rounded powers
// x^1.5 correctly rounded (except in cases within ~2^-104 relative of a rounding midpoint):
// sqrt(x) = s + t with the exact residual x - s^2, then x*s as an exact product plus the
// correction, all in double-double.
__host__ __device__ inline double cr_pow15(double x) {
    double s = sqrt(x);
    double r = fma(-s, s, x);
    double t = r / (2.0 * s);
    double p = x * s;
    double e = fma(x, s, -p);
    return p + (e + x * t);
}

// x^(1/3.) with 1/3. the double nearest 1/3 (as the reference's pow(..., 1./3.)):
// a double-double cube root refined by one Newton step, times x^(-delta) with
// delta = 1/3 - (double)(1/3.) = 2^-54/3, applied as a first-order correction.
__host__ __device__ inline double cr_pow_third(double x) {
    double c0 = cbrt(x);
    double c2 = c0 * c0, e2 = fma(c0, c0, -c2);
    double c3 = c2 * c0, c3l = fma(c2, c0, -c3) + e2 * c0;
    double r = (x - c3) - c3l;
    double clo = r / (3.0 * c2);
    const double delta = 1.8503717077085943e-17;
    double L = log(x);
    return c0 + (clo - c0 * (delta * L));
}

}  // namespace plan
