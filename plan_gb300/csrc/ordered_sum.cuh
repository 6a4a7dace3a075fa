// Sequential FP64 sums, exactly as a loop would round them, thirty-two terms at a time.
//
// The reference accumulates member sums one term at a time (s = s + x[k], round to nearest
// even each time), and the clump catalogue must keep those bits. On this GPU a dependent FP64
// add costs 63 cycles, so a 200,000-member clump costs milliseconds per sum. This evaluates
// the same recurrence with a warp:
//
// While the running sum stays inside one binade [2^e, 2^(e+1)) (same sign), every double it
// can take is a multiple of u = 2^(e-52), and s + x rounds to s + u * round(x / u): the
// rounding of s + x to the u grid only depends on x, except for a tie (x / u exactly half
// way between integers), where the parity of s decides. So the lanes scale their terms by
// 1/u (exact), round them to integers and take an integer prefix sum; the leading run of
// lanes whose partial sums stay strictly inside the binade (or land exactly on 2^(e+1),
// which every rounding of that exact sum also gives) is exact. A tie, a term too large for
// the grid, a sign change or a partial sum leaving the binade ends the run; the term that
// ended it is then added as one ordinary FP64 add, and the next run starts in the new binade.
// Zero, tiny or huge running sums (no usable grid) also take ordinary adds.
#pragma once

#include <cstdint>

#include "exact64.cuh"

namespace plan {

// s + x[0] + x[1] + ... + x[n-1], left to right with rounding after every add. Called by all
// 32 lanes of a warp with the same arguments; every lane returns the same value.
__device__ inline double warp_ordered_sum(const double *x, uint32_t n, double s) {
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    uint32_t k = 0;
    while (k < n) {
        const long long bits = __double_as_longlong(s);
        const int ex = (int)((bits >> 52) & 0x7ff);
        if (ex <= 60 || ex >= 2000) {  // zero, tiny or huge: no grid, one ordinary add
            s = s + x[k];
            ++k;
            continue;
        }
        const long long mag = (bits & 0xfffffffffffffLL) | (1LL << 52);
        const long long n0 = bits < 0 ? -mag : mag;                             // s / u
        const double inv_u = __longlong_as_double((long long)(2098 - ex) << 52);  // 2^(1075-ex)
        const double u = __longlong_as_double((long long)(ex - 52) << 52);        // 2^(ex-1075)
        const uint32_t j = k + lane;
        bool ok = false;
        long long nj = 0;
        if (j < n) {
            const double y = x[j] * inv_u;  // exact: a power-of-two scale
            if (fabs(y) < 9007199254740992.0) {
                const double fl = floor(y);
                if (y - fl != 0.5) {
                    ok = true;
                    nj = (long long)rint(y);
                }
            }
        }
        long long p = nj;
        for (int d = 1; d < 32; d <<= 1) {
            const long long t = __shfl_up_sync(full, p, d);
            if (lane >= d) p += t;
        }
        const long long nn = n0 + p;
        const long long an = nn < 0 ? -nn : nn;
        const bool inside = ok && ((nn < 0) == (n0 < 0)) && an > (1LL << 52) && an <= (1LL << 53);
        const unsigned valid = __ballot_sync(full, j < n);
        const unsigned good = __ballot_sync(full, inside);
        const unsigned top = __ballot_sync(full, inside && an == (1LL << 53));
        const unsigned bad = valid & ~good;
        int a = bad ? __ffs(bad) - 1 : __popc(valid);
        if (top) a = min(a, __ffs(top));  // stop after the first lane that reached 2^(e+1)
        if (a == 0) {
            s = s + x[k];
            ++k;
            continue;
        }
        const long long na = __shfl_sync(full, nn, a - 1);
        s = (double)na * u;  // |na| <= 2^53: exact
        k += (uint32_t)a;
    }
    return s;
}

// The same sum with the grid rounding of the terms and the result done in integer
// arithmetic (grid_term, grid_value): no FP64 instruction except for the ordinary adds
// that start a run or step over a tie, a binade change or an out-of-range running sum.
__device__ inline double warp_ordered_sum_int(const double *x, uint32_t n, double s) {
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    uint32_t k = 0;
    while (k < n) {
        const long long bits = __double_as_longlong(s);
        const uint32_t ex = (uint32_t)((bits >> 52) & 0x7ff);
        if (ex <= 60 || ex >= 2000) {  // zero, tiny or huge: no grid, one ordinary add
            s = s + x[k];
            ++k;
            continue;
        }
        const long long mag = (bits & 0xfffffffffffffLL) | (1LL << 52);
        const long long n0 = bits < 0 ? -mag : mag;  // s / u
        const uint32_t j = k + lane;
        long long nj = 0;
        const bool ok = j < n && grid_term(x[j], ex, nj);
        long long p = ok ? nj : 0;
        for (int d = 1; d < 32; d <<= 1) {
            const long long t = __shfl_up_sync(full, p, d);
            if (lane >= d) p += t;
        }
        const long long nn = n0 + p;
        const long long an = nn < 0 ? -nn : nn;
        const bool inside = ok && ((nn < 0) == (n0 < 0)) && an > (1LL << 52) && an <= (1LL << 53);
        const unsigned valid = __ballot_sync(full, j < n);
        const unsigned good = __ballot_sync(full, inside);
        const unsigned top = __ballot_sync(full, inside && an == (1LL << 53));
        const unsigned bad = valid & ~good;
        int a = bad ? __ffs(bad) - 1 : __popc(valid);
        if (top) a = min(a, __ffs(top));  // stop after the first lane that reached 2^(e+1)
        if (a == 0) {
            s = s + x[k];
            ++k;
            continue;
        }
        const long long na = __shfl_sync(full, nn, a - 1);
        s = grid_value(na, ex);
        k += (uint32_t)a;
    }
    return s;
}

}  // namespace plan
