// Exact FP64 bookkeeping in integer arithmetic.
//
// On this GPU an FP64 instruction occupies the SM's FP64 pipe for about 19 cycles whatever
// the number of active lanes, and a dependent one waits 36-55 cycles (measured with
// dependent chains on one warp). The clump stage's hot loops therefore do in integer
// arithmetic whatever does not need an FP64 rounding: splitting a double into a float
// pair, and rounding a term onto the grid of a running sum's binade. Both functions here
// give exactly what the FP64 expressions they replace give (checked on the CPU against
// those expressions), and report when an argument falls outside the range they handle.
#pragma once

#include <cstdint>
#include <cstring>

namespace plan {

__host__ __device__ inline uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
#endif
}

__host__ __device__ inline double dfrom(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    std::memcpy(&x, &b, 8);
    return x;
#endif
}

__host__ __device__ inline float ffrom(uint32_t b) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float x;
    std::memcpy(&x, &b, 4);
    return x;
#endif
}

// hi = (float)x and lo = (float)(x - (double)hi), both rounded to nearest even, from the
// bits of x. Handles |x| in [2^-74, 2^126) and zero (lo = +0); returns false otherwise.
// x - hi is exact in FP64 and equals rem * 2^(e-1075) with |rem| <= 2^28, so its float
// rounding is the int-to-float rounding of rem scaled by an exact power of two.
__host__ __device__ inline bool split_hilo_bits(double x, float &hi, float &lo) {
    const uint64_t b = dbits(x);
    const uint32_t ex = (uint32_t)(b >> 52) & 0x7ffu;
    const uint32_t sgn = (uint32_t)(b >> 32) & 0x80000000u;
    if ((b << 1) == 0) {
        hi = ffrom(sgn);
        lo = 0.0f;
        return true;
    }
    if (ex < 949u || ex > 1148u) return false;
    const uint64_t mant = (b & 0xfffffffffffffull) | (1ull << 52);
    uint32_t hm = (uint32_t)(mant >> 29);  // 24 bits
    int32_t rem = (int32_t)(mant & 0x1fffffffull);
    uint32_t fe = ex - 1023u + 127u;
    const int32_t half = 1 << 28;
    if (rem > half || (rem == half && (hm & 1u))) {
        hm += 1u;
        rem -= 1 << 29;
        if (hm == (1u << 24)) {
            hm = 1u << 23;
            fe += 1u;
        }
    }
    hi = ffrom(sgn | (fe << 23) | (hm & 0x7fffffu));
    if (rem == 0) {
        lo = 0.0f;
    } else {
        const float scale = ffrom((ex - 1075u + 127u) << 23);  // 2^(e-1075), a normal float
        const float l = (float)rem * scale;
        lo = sgn ? -l : l;
    }
    return true;
}

// The term x on the grid of a running sum whose biased exponent is es (61 <= es <= 1999):
// n = x / 2^(es-1075) rounded to the nearest integer. Returns false when that quotient is
// exactly half way between two integers, is not below 2^53 in magnitude, or x is not
// finite; the caller then adds x as an ordinary FP64 add. Equal to rint(x * 2^(1075-es))
// with the same refusals as the FP64 test (|y| < 2^53, y - floor(y) != 0.5).
__host__ __device__ inline bool grid_term(double x, uint32_t es, long long &n) {
    const uint64_t b = dbits(x);
    const uint32_t ex = (uint32_t)(b >> 52) & 0x7ffu;
    if (ex == 0x7ffu) return false;
    if ((b << 1) == 0) {
        n = 0;
        return true;
    }
    uint64_t mant = b & 0xfffffffffffffull;
    uint32_t eeff = ex;
    if (ex == 0) {
        eeff = 1;
    } else {
        mant |= 1ull << 52;
    }
    if (eeff > es) return false;  // |x / u| >= 2^53
    const uint32_t d = es - eeff;
    uint64_t q;
    if (d == 0) {
        q = mant;
    } else if (d >= 64) {
        q = 0;  // |x / u| < 2^-11: rounds to zero, never a tie
    } else {
        q = mant >> d;
        const uint64_t rem = mant & ((1ull << d) - 1ull);
        const uint64_t half = 1ull << (d - 1);
        if (rem == half) return false;
        if (rem > half) q += 1;
    }
    n = (b >> 63) ? -(long long)q : (long long)q;
    return true;
}

// The double n * 2^(es-1075) for 2^52 < |n| <= 2^53 (a partial sum inside the binade of
// exponent es, or exactly on its upper edge).
__host__ __device__ inline double grid_value(long long n, uint32_t es) {
    const uint64_t sgn = n < 0 ? (1ull << 63) : 0ull;
    const uint64_t a = (uint64_t)(n < 0 ? -n : n);
    if (a == (1ull << 53)) return dfrom(sgn | ((uint64_t)(es + 1) << 52));
    return dfrom(sgn | ((uint64_t)es << 52) | (a - (1ull << 52)));
}

}  // namespace plan
