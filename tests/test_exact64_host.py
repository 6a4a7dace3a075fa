"""The integer forms of two FP64 steps of the clump stage, on the CPU (no GPU).

exact64.cuh replaces FP64 instructions, which are slow on this GPU, by integer arithmetic:
  * split_hilo_bits(x): the float pair (RN32(x), RN32(x - RN32(x))) that the FP32 filters
    of the rebinding loop use, formed from the bits of x;
  * grid_term(x, es): x on the grid of a running sum of biased exponent es, rounded to the
    nearest integer, with ties and oversized terms refused, as the ordered member sums use
    it; grid_value builds the double of a partial sum from its grid integer.
Each is compared here with the FP64 expression it replaces, over random arguments across
all the exponent ranges they accept, rounding ties of both parities, carries into the next
binade, zeros of both signs, subnormal terms and shifts beyond 64 bits.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parent.parent / "plan_gb300" / "csrc"

HARNESS = r"""
#define __host__
#define __device__
#include <cmath>
#include <cstdio>
#include <cstring>
#include "exact64.cuh"
using namespace plan;

static uint64_t st = 0x9e3779b97f4a7c15ull;
static uint64_t xr() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; }
static long n_split = 0, bad_split = 0, refused_split = 0, n_grid = 0, bad_grid = 0, n_val = 0, bad_val = 0;

static uint32_t fb(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

static void t_split(double x) {
    float h, l;
    const uint64_t b = dbits(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    const bool in_range = ((b << 1) == 0) || (ex >= 949 && ex <= 1148);
    const bool ok = split_hilo_bits(x, h, l);
    ++n_split;
    if (ok != in_range) { ++bad_split; return; }
    if (!ok) { ++refused_split; return; }
    const float hr = (float)x;
    const float lr = (float)(x - (double)hr);
    if (fb(h) != fb(hr) || fb(l) != fb(lr)) ++bad_split;
}

static void t_grid(double x, uint32_t es) {
    const double inv_u = dfrom((uint64_t)(2098 - es) << 52);
    const double y = x * inv_u;
    bool ok_ref = false;
    long long n_ref = 0;
    if (std::fabs(y) < 9007199254740992.0) {
        const double fl = std::floor(y);
        if (y - fl != 0.5) { ok_ref = true; n_ref = (long long)std::rint(y); }
    }
    long long n = 0;
    const bool ok = grid_term(x, es, n);
    ++n_grid;
    if (ok != ok_ref || (ok && n != n_ref)) ++bad_grid;
}

static void t_val(long long nn, uint32_t es) {
    const double u = dfrom((uint64_t)(es - 52) << 52);
    const double ref = (double)nn * u;
    ++n_val;
    if (dbits(grid_value(nn, es)) != dbits(ref)) ++bad_val;
}

static double rnd_exp(int ebiased) {
    return dfrom((xr() & 0x800fffffffffffffull) | ((uint64_t)ebiased << 52));
}

int main() {
    // splits: every exponent the function accepts, plus some on either side of the range
    for (int e = 900; e <= 1200; ++e)
        for (int i = 0; i < 20000; ++i) t_split(rnd_exp(e));
    for (int e = 949; e <= 1148; ++e)
        for (int i = 0; i < 200; ++i) {
            uint64_t m = xr() & 0x000fffffe0000000ull;  // low 29 bits cleared
            const uint64_t s = xr() & 0x8000000000000000ull;
            t_split(dfrom(s | ((uint64_t)e << 52) | m | (1ull << 28)));          // tie, either parity
            t_split(dfrom(s | ((uint64_t)e << 52) | m | (1ull << 28) | 1ull));   // just above the tie
            t_split(dfrom(s | ((uint64_t)e << 52) | m | ((1ull << 28) - 1ull))); // just below
            t_split(dfrom(s | ((uint64_t)e << 52) | 0x000fffffffffffffull));     // carry into the next binade
            t_split(dfrom(s | ((uint64_t)e << 52)));                              // a power of two
        }
    t_split(0.0); t_split(-0.0);
    // grid terms: running sums of every exponent class the sums use, terms around them
    for (uint32_t es = 61; es < 2000; es += 7)
        for (int i = 0; i < 2000; ++i) {
            const int off = (int)(xr() % 140) - 100;
            int e = (int)es + off;
            if (e < 0) e = 0;
            if (e > 2046) e = 2046;
            t_grid(rnd_exp(e), es);
        }
    for (uint32_t es = 61; es < 2000; es += 3)
        for (int d = 1; d < 60; ++d) {
            if ((int)es - d < 1) break;
            const uint64_t e = es - (uint32_t)d;
            const uint64_t m = xr() & 0x000fffffffffffffull;
            const uint64_t tie = (m >> d << d) | (1ull << (d - 1));  // exactly half a grid step
            t_grid(dfrom((e << 52) | (tie & 0x000fffffffffffffull)), es);
            t_grid(dfrom((1ull << 63) | (e << 52) | (tie & 0x000fffffffffffffull)), es);
            t_grid(dfrom((e << 52) | m), es);
        }
    for (int i = 0; i < 200000; ++i) t_grid(dfrom(xr() & 0x800fffffffffffffull), 61 + (uint32_t)(xr() % 1900));  // subnormal terms
    t_grid(0.0, 1000); t_grid(-0.0, 1000); t_grid(INFINITY, 1000); t_grid(-NAN, 1000);
    // grid values inside a binade and on its upper edge
    for (uint32_t es = 61; es < 2000; es += 5)
        for (int i = 0; i < 400; ++i) {
            long long a = (long long)((1ull << 52) + 1 + (xr() % ((1ull << 52) - 1)));
            if (i == 0) a = 1ll << 53;
            t_val((xr() & 1) ? -a : a, es);
        }
    printf("%ld %ld %ld %ld %ld %ld %ld\n", n_split, bad_split, refused_split, n_grid, bad_grid, n_val, bad_val);
    return 0;
}
"""


def test_integer_splits_and_grid_terms_match_fp64(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    (tmp_path / "h.cpp").write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(CSRC), str(tmp_path / "h.cpp"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    n_split, bad_split, refused, n_grid, bad_grid, n_val, bad_val = map(int, out)
    assert n_split > 6_000_000 and n_grid > 800_000 and n_val > 100_000
    assert refused < n_split // 2
    assert bad_split == 0
    assert bad_grid == 0
    assert bad_val == 0
