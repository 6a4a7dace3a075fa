"""The exact division of the speculative acceptance chain, on the CPU (no GPU).

With y the correctly rounded reciprocal of M, q0 = RN(num * y), r = num - q0 M (exact with
one FMA) and q = RN(q0 + r y) (one more FMA), q is the correctly rounded quotient num / M
(Markstein's correction). The speculative acceptance windows of k_rebind_round compute the
reciprocals of a window's masses in parallel and take this two-FMA step in the dependent
chain instead of a division. IEEE arithmetic gives the same bits on the CPU and the GPU, so
the identity is checked here against the CPU's division: random operands over sixty binades,
divisors with all-ones and nearly-empty significands, and the update's own operand ranges.
"""
from __future__ import annotations

import shutil
import subprocess

import pytest

HARNESS = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static uint64_t s = 88172645463325252ull;
static uint64_t xr(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static long n = 0, bad = 0;
static void t(double a, double b) {
    double y = 1.0 / b, q0 = a * y;
    double q = a == 0.0 ? a : fma(fma(-q0, b, a), y, q0);
    ++n;
    if (memcmp(&q, &(double){a / b}, 8) != 0) ++bad;
}
static double rnd(int emin, int span) {
    uint64_t b = (xr() & 0x000fffffffffffffull) | ((uint64_t)(1023 + emin + (int)(xr() % span)) << 52);
    double x;
    memcpy(&x, &b, 8);
    return x;
}
int main(void) {
    for (long i = 0; i < 6000000L; ++i) {
        double a = rnd(-30, 60), b = rnd(-30, 60);
        if (i % 3 == 0) { uint64_t bb; memcpy(&bb, &b, 8); bb |= 0x000ffffffffff000ull; memcpy(&b, &bb, 8); }
        t((xr() & 1) ? -a : a, b);
    }
    for (int e = -40; e <= 10; ++e)
        for (long i = 0; i < 40000; ++i) {
            double a = rnd(e - 10, 20);
            t(a, ldexp(2.0 - ldexp(1.0, -52), e));
            t(a, ldexp(1.0 + ldexp(1.0, -52), e));
            t(-a, ldexp(1.0 + (double)(xr() % 64) * ldexp(1.0, -52), e));
        }
    for (long i = 0; i < 4000000L; ++i) {
        double M = ldexp(1.0 + (double)(xr() >> 12) * ldexp(1.0, -52), -30 + (int)(xr() % 24));
        double m = ldexp(1.0 + (double)(xr() >> 12) * ldexp(1.0, -52), -30 + (int)(xr() % 10));
        double c = ((double)(int64_t)(xr() >> 11) * ldexp(1.0, -53)) * 0.2;
        double q = ((double)(int64_t)(xr() >> 11) * ldexp(1.0, -53)) * 0.2;
        double Mn = M + m;
        t(c * Mn + m * q, Mn);
    }
    t(0.0, 3.0); t(-0.0, 3.0);
    printf("%ld %ld\n", bad, n);
    return 0;
}
"""


def test_reciprocal_correction_is_the_division(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    (tmp_path / "h.c").write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run([cc, "-O2", "-std=c11", "-ffp-contract=off", str(tmp_path / "h.c"), "-o", str(exe), "-lm"], check=True)
    bad, n = map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split())
    assert n > 10_000_000
    assert bad == 0
