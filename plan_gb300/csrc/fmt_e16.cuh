// printf("%24.16e") of a double, exactly as glibc prints it, in plain integer arithmetic that
// runs on the device and on the host alike.
//
// The reference writes member lists with std::scientific, setprecision(16), setw(24)
// (src/tree.hpp:5208-5217), i.e. "%24.16e": 17 significant digits, correctly rounded from the
// double's exact binary value, ties to even. For v = f 2^e (f < 2^53) and the decimal exponent
// k = floor(log10 |v|), the digits are D = round(v / 10^(k-16)), 10^16 <= D < 10^17. Three
// cases cover every finite v:
//   e >= 0, k < 16   v is an integer below 2^53: D = v 10^(16-k) exactly;
//   e >= 0, k >= 16  D = round(f 2^e / 10^(k-16)): divide by 10^(k-17) keeping a sticky bit
//                    for any remainder, then the last digit decides;
//   e < 0            D = round(f 10^(16-k) / 2^-e): a right shift, whose first dropped bit
//                    and the bits below it decide.
// A guessed k that is one off shows as D outside [10^16, 10^17) and is corrected. Big
// integers are little-endian 32-bit limbs (at most 1,200 bits here).
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PLAN_FMT_HD __host__ __device__
#else
#define PLAN_FMT_HD
#endif

namespace plan {

namespace fmt_detail {

constexpr int kLimbs = 44;  // f 10^340 needs 37

struct Big {
    uint32_t w[kLimbs];
    int n;  // limbs in use
};

PLAN_FMT_HD inline void big_set(Big &b, uint64_t v) {
    b.w[0] = (uint32_t)v;
    b.w[1] = (uint32_t)(v >> 32);
    b.n = b.w[1] ? 2 : (b.w[0] ? 1 : 0);
}

PLAN_FMT_HD inline void big_mul_small(Big &b, uint32_t m) {
    uint64_t carry = 0;
    for (int i = 0; i < b.n; ++i) {
        const uint64_t t = (uint64_t)b.w[i] * m + carry;
        b.w[i] = (uint32_t)t;
        carry = t >> 32;
    }
    if (carry) b.w[b.n++] = (uint32_t)carry;
}

// b = b / d, returns the remainder
PLAN_FMT_HD inline uint32_t big_div_small(Big &b, uint32_t d) {
    uint64_t r = 0;
    for (int i = b.n - 1; i >= 0; --i) {
        const uint64_t cur = (r << 32) | b.w[i];
        b.w[i] = (uint32_t)(cur / d);
        r = cur % d;
    }
    while (b.n > 0 && b.w[b.n - 1] == 0) --b.n;
    return (uint32_t)r;
}

PLAN_FMT_HD inline void big_shl(Big &b, int s) {
    const int limbs = s / 32, bits = s % 32;
    if (bits) {
        uint32_t carry = 0;
        for (int i = 0; i < b.n; ++i) {
            const uint32_t v = b.w[i];
            b.w[i] = (v << bits) | carry;
            carry = v >> (32 - bits);
        }
        if (carry) b.w[b.n++] = carry;
    }
    if (limbs && b.n) {
        for (int i = b.n - 1; i >= 0; --i) b.w[i + limbs] = b.w[i];
        for (int i = 0; i < limbs; ++i) b.w[i] = 0;
        b.n += limbs;
    }
}

PLAN_FMT_HD inline void big_mul_pow10(Big &b, int p) {
    while (p >= 9) {
        big_mul_small(b, 1000000000u);
        p -= 9;
    }
    uint32_t m = 1;
    while (p-- > 0) m *= 10;
    if (m > 1) big_mul_small(b, m);
}

// b = b / 10^p; sticky |= any nonzero remainder
PLAN_FMT_HD inline void big_div_pow10(Big &b, int p, bool &sticky) {
    while (p >= 9) {
        sticky |= big_div_small(b, 1000000000u) != 0;
        p -= 9;
    }
    uint32_t d = 1;
    while (p-- > 0) d *= 10;
    if (d > 1) sticky |= big_div_small(b, d) != 0;
}

PLAN_FMT_HD inline uint64_t big_low64(const Big &b) {
    uint64_t v = 0;
    if (b.n > 0) v = b.w[0];
    if (b.n > 1) v |= (uint64_t)b.w[1] << 32;
    return v;
}

PLAN_FMT_HD inline bool big_bit(const Big &b, int i) {
    const int l = i / 32;
    return l < b.n && ((b.w[l] >> (i % 32)) & 1u);
}

PLAN_FMT_HD inline bool big_any_below(const Big &b, int i) {  // any of bits [0, i) set
    for (int l = 0; l < b.n && l * 32 < i; ++l) {
        const int top = i - l * 32;
        const uint32_t mask = top >= 32 ? 0xffffffffu : ((1u << top) - 1u);
        if (b.w[l] & mask) return true;
    }
    return false;
}

// round(v / 10^(k-16)) for v = f 2^e > 0; D may fall outside [10^16, 10^17] when k is off
PLAN_FMT_HD inline uint64_t digits17(uint64_t f, int e, int k) {
    Big b;
    big_set(b, f);
    if (e >= 0) {
        big_shl(b, e);
        if (k < 16) {
            big_mul_pow10(b, 16 - k);
            return big_low64(b);  // exact (callers check the range)
        }
        bool sticky = false;
        if (k >= 17) big_div_pow10(b, k - 17, sticky);  // 18 digits left when k is right
        else big_mul_pow10(b, 17 - k);
        const uint64_t q = big_low64(b);   // b < 10^19 < 2^64 whenever the result is in range
        if (b.n > 2) return ~0ull;          // k too small: out of range
        uint64_t d = q / 10;
        const uint32_t last = (uint32_t)(q % 10);
        if (last > 5 || (last == 5 && (sticky || (d & 1)))) ++d;
        return d;
    }
    const int s = -e;
    if (k > 16) return 0;  // v < 2^53 < 10^16 here: a k this large is a wrong guess (too small a D)
    big_mul_pow10(b, 16 - k);
    // D = round(b / 2^s)
    const bool half = s > 0 && big_bit(b, s - 1);
    const bool below = s > 1 && big_any_below(b, s - 1);
    // shift right by s
    Big q = b;
    {
        const int limbs = s / 32, bits = s % 32;
        if (limbs >= q.n) {
            q.n = 0;
        } else {
            for (int i = 0; i + limbs < q.n; ++i) q.w[i] = q.w[i + limbs];
            q.n -= limbs;
            if (bits) {
                for (int i = 0; i < q.n; ++i) {
                    const uint32_t hi = i + 1 < q.n ? q.w[i + 1] : 0u;
                    q.w[i] = (q.w[i] >> bits) | (hi << (32 - bits));
                }
            }
            while (q.n > 0 && q.w[q.n - 1] == 0) --q.n;
        }
    }
    if (q.n > 2) return ~0ull;
    uint64_t d = big_low64(q);
    if (half && (below || (d & 1))) ++d;
    return d;
}

}  // namespace fmt_detail

// Writes exactly 24 characters (no terminator): v as "%24.16e".
PLAN_FMT_HD inline void fmt_e16_w24(double v, char *out) {
    using namespace fmt_detail;
    char buf[24];
    int len = 0;
    uint64_t bits;
    memcpy(&bits, &v, sizeof bits);
    const bool neg = (bits >> 63) != 0;
    const int bexp = (int)((bits >> 52) & 0x7ff);
    const uint64_t frac = bits & 0xfffffffffffffull;
    if (bexp == 0x7ff) {  // glibc: inf, -inf, nan, -nan
        if (neg) buf[len++] = '-';
        const char *w = frac ? "nan" : "inf";
        for (int i = 0; i < 3; ++i) buf[len++] = w[i];
    } else {
        uint64_t D = 0;
        int k = 0;
        if (bexp != 0 || frac != 0) {
            const uint64_t f = bexp ? (frac | (1ull << 52)) : frac;
            const int e = bexp ? bexp - 1075 : -1074;
            // k from the binary exponent: floor(log10(2) * (position of the top bit)), maybe one low
            int top = 63;
            while (!((f >> top) & 1ull)) --top;
            const int e2 = e + top;  // 2^e2 <= v < 2^(e2+1)
            // floor(e2 log10 2) by a multiply-shift (78913 / 2^18 ~ log10 2; the shift floors
            // negative values too); the true k is this or one more
            k = (int)((e2 * 78913LL) >> 18);
            for (int tries = 0; tries < 4; ++tries) {
                D = digits17(f, e, k);
                if (D < 10000000000000000ull) {
                    --k;
                } else if (D > 100000000000000000ull || D == ~0ull) {
                    ++k;
                } else {
                    break;
                }
            }
            if (D == 100000000000000000ull) {  // rounded up to the next power of ten
                D = 10000000000000000ull;
                ++k;
            }
        }
        if (neg) buf[len++] = '-';
        char dig[17];
        for (int i = 16; i >= 0; --i) {
            dig[i] = (char)('0' + (int)(D % 10));
            D /= 10;
        }
        buf[len++] = dig[0];
        buf[len++] = '.';
        for (int i = 1; i < 17; ++i) buf[len++] = dig[i];
        buf[len++] = 'e';
        buf[len++] = k < 0 ? '-' : '+';
        int ak = k < 0 ? -k : k;
        if (ak >= 100) {
            buf[len++] = (char)('0' + ak / 100);
            ak %= 100;
            buf[len++] = (char)('0' + ak / 10);
            buf[len++] = (char)('0' + ak % 10);
        } else {
            buf[len++] = (char)('0' + ak / 10);
            buf[len++] = (char)('0' + ak % 10);
        }
    }
    const int pad = 24 - len;  // len <= 24 for every double
    for (int i = 0; i < pad; ++i) out[i] = ' ';
    for (int i = 0; i < len; ++i) out[pad + i] = buf[i];
}

// Writes exactly 16 characters: an unsigned 32-bit integer right-aligned ("%16u").
PLAN_FMT_HD inline void fmt_u32_w16(uint32_t v, char *out) {
    char d[10];
    int n = 0;
    do {
        d[n++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    for (int i = 0; i < 16 - n; ++i) out[i] = ' ';
    for (int i = 0; i < n; ++i) out[16 - 1 - i] = d[i];
}

}  // namespace plan
