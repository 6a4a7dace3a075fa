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
__device__ inline double warp_ordered_sum_int(const double *x, uint32_t n, double s, uint32_t *iters = nullptr) {
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    uint32_t k = 0;
    while (k < n) {
        if (iters) ++*iters;
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

// The same sum over a window of 32*K terms held in registers, lane l holding terms
// [l K, l K + K) of the window in order (cnt valid terms). Each step rounds every
// remaining term onto the grid of the running sum's binade, forms the integer prefix
// sums lane by lane and then across the warp, and keeps the longest leading run whose
// partial sums stay inside the binade (or reach its upper edge, which ends the run); the
// first term that does not fit is added as one ordinary FP64 add. The step then continues
// with the remaining terms of the same registers, so a binade change costs one step, not a
// reload. Every lane returns the same value.
template <int K>
__device__ inline double warp_ordered_sum_window(const double (&x)[K], uint32_t cnt, double s, uint32_t *iters = nullptr) {
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    uint32_t pos = 0;  // terms of the window already added
    while (pos < cnt) {
        if (iters) ++*iters;
        const long long bits = __double_as_longlong(s);
        const uint32_t ex = (uint32_t)((bits >> 52) & 0x7ff);
        if (bits == 0) {
            // s = +0: adding a zero of either sign leaves +0, so a run of zero terms (particles
            // at rest, say) is skipped at once; the first nonzero one is an ordinary add below
            int fz = K;
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const uint32_t seq = (uint32_t)(lane * K + j);
                if (fz == K && seq >= pos && seq < cnt && (__double_as_longlong(x[j]) << 1) != 0) fz = j;
            }
            const unsigned nz = __ballot_sync(full, fz < K);
            if (!nz) break;  // only zeros remain
            const int Lz = __ffs(nz) - 1;
            pos = (uint32_t)(Lz * K + __shfl_sync(full, fz, Lz));
        }
        // this lane's remaining terms on the grid, and their prefix sums within the lane
        long long t[K];
        bool ok[K];
        long long tot = 0;
        const bool grid = ex > 60 && ex < 2000;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const uint32_t seq = (uint32_t)(lane * K + j);
            const bool rem = seq >= pos && seq < cnt;
            t[j] = 0;
            ok[j] = true;
            if (rem && grid) ok[j] = grid_term(x[j], ex, t[j]);
            tot += t[j];
        }
        long long before = tot;  // inclusive scan across lanes, then exclusive
        for (int d = 1; d < 32; d <<= 1) {
            const long long v = __shfl_up_sync(full, before, d);
            if (lane >= d) before += v;
        }
        before -= tot;
        const long long mag = (bits & 0xfffffffffffffLL) | (1LL << 52);
        const long long n0 = bits < 0 ? -mag : mag;  // s / u
        // the first remaining term of this lane whose partial sum leaves the binade (stop at
        // it) or lands on its upper edge (stop after it)
        int stop = K;
        bool stopped = false, edge = false;
        long long run = n0 + before;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const uint32_t seq = (uint32_t)(lane * K + j);
            const bool rem = seq >= pos && seq < cnt;
            if (rem && !stopped) {
                run += t[j];
                const long long an = run < 0 ? -run : run;
                const bool inside = grid && ok[j] && ((run < 0) == (n0 < 0)) && an > (1LL << 52) && an <= (1LL << 53);
                if (!inside) {
                    stop = j;
                    stopped = true;
                } else if (an == (1LL << 53)) {
                    stop = j + 1;
                    stopped = true;
                    edge = true;
                }
            }
        }
        const unsigned hit = __ballot_sync(full, stopped);
        const int L = hit ? __ffs(hit) - 1 : 31;
        const int stopL = __shfl_sync(full, stop, L);
        const bool edgeL = __shfl_sync(full, edge ? 1 : 0, L) != 0;
        const uint32_t end = min(cnt, (uint32_t)(L * K + stopL));  // terms [pos, end) fit the grid
        if (end > pos) {
            // the grid integer of the partial sum after term end - 1
            const uint32_t last = end - 1, ll = last / K;
            long long val = n0 + before;
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const uint32_t seq = (uint32_t)(lane * K + j);
                if (seq >= pos && seq <= last) val += t[j];
            }
            val = __shfl_sync(full, val, (int)ll);
            s = grid_value(val, ex);
            pos = end;
        }
        if (hit && !edgeL) {
            // term pos does not fit the grid of s (whose binade is unchanged by the run): one
            // ordinary add, which a new step would also take, since its grid is the same
            double v = 0.0;
#pragma unroll
            for (int j = 0; j < K; ++j)
                if ((uint32_t)(lane * K + j) == pos) v = x[j];
            v = __shfl_sync(full, v, (int)(pos / K));
            s = s + v;
            ++pos;
        }
    }
    return s;
}

}  // namespace plan
