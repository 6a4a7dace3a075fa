"""The device's "%24.16e" conversion, on the CPU (no GPU).

plan_gb300/csrc/fmt_e16.cuh formats doubles for the member lists the device writes (the
reference's setw(24) scientific precision-16 output) with integer arithmetic only. Built here
with g++, it must print every double exactly as glibc's printf does: random bit patterns over
all exponents, float-derived values like the snapshot's, values at powers of ten, zeros,
subnormals, infinities and NaNs.
"""
from __future__ import annotations

import shutil
import subprocess

import pytest

from conftest import ROOT

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include "fmt_e16.cuh"

static long bad = 0, n = 0;
static void check(double v) {
    char ref[64], got[25];
    std::snprintf(ref, sizeof ref, "%24.16e", v);
    plan::fmt_e16_w24(v, got);
    got[24] = 0;
    ++n;
    if (std::strcmp(ref, got) != 0) {
        if (bad < 5) std::fprintf(stderr, "%a: [%s] [%s]\n", v, ref, got);
        ++bad;
    }
}

int main(int argc, char **argv) {
    const long N = std::atol(argv[1]);
    std::mt19937_64 rng(11);
    for (long i = 0; i < N; ++i) {
        const uint64_t b = rng();
        double v;
        std::memcpy(&v, &b, 8);
        check(v);
    }
    for (long i = 0; i < N / 4; ++i) {
        const float a = std::ldexp((float)(rng() % 16777216), -(int)(rng() % 40)) * ((rng() & 1) ? -1.f : 1.f);
        const double v = (double)a;
        check(v);
        check(v * 4.0106053636305e-08);
        check(v / 3.0);
    }
    for (int e = -330; e <= 310; ++e) {
        const double p = std::pow(10.0, e);
        check(p);
        check(std::nextafter(p, 0.0));
        check(std::nextafter(p, 1e308));
        check(9.9999999999999999e-1 * p);
    }
    const double sp[] = {0.0, -0.0, 1.0, -1.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, INFINITY, -INFINITY,
                         NAN, -NAN, 9007199254740992.0, 9007199254740993.0, 1e16, 1e17, 99999999999999999.0, 0.1, 0.2, 0.3};
    for (double v : sp) check(v);
    char u[17];
    for (uint32_t v : {0u, 1u, 9u, 10u, 4294967295u, 123456789u}) {
        plan::fmt_u32_w16(v, u);
        u[16] = 0;
        char ref[32];
        std::snprintf(ref, sizeof ref, "%16u", v);
        ++n;
        if (std::strcmp(ref, u) != 0) ++bad;
    }
    std::printf("%ld %ld\n", bad, n);
    return 0;
}
"""


def test_fmt_e16_matches_printf(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    (tmp_path / "h.cpp").write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "plan_gb300" / "csrc"), str(tmp_path / "h.cpp"), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), "2000000"], capture_output=True, text=True, check=True)
    bad, n = map(int, r.stdout.split())
    assert n > 3_000_000
    assert bad == 0, r.stderr
