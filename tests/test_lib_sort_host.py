"""The device's replay of std::sort for tied member distances, on the CPU (no GPU).

plan_gb300/csrc/lib_sort.cuh restates GCC's std::sort (introsort with median-of-three
pivots, a heap-sort fallback and a final insertion sort) for (distance, member) pairs compared
by distance alone; the device runs it for clumps whose member sort meets a tie. Built here with
g++, it must leave every sequence in exactly the order std::sort leaves it, ties included,
including the inputs that drive the library into its heap-sort fallback.
"""
from __future__ import annotations

import shutil
import subprocess

import pytest

from conftest import ROOT

HARNESS = r"""
#include <algorithm>
#include <cstdio>
#include <random>
#include <utility>
#include <vector>
#include "lib_sort.cuh"

int main() {
    std::mt19937_64 rng(7);
    long bad = 0, tests = 0;
    for (int t = 0; t < 20000; ++t) {
        const int n = (int)(rng() % (t < 19000 ? 300 : 20000));
        const int nk = 1 + (int)(rng() % 40);  // few distinct keys: many ties
        const int mode = (int)(rng() % 4);
        std::vector<std::pair<uint32_t, double>> v(n);
        for (int i = 0; i < n; ++i) {
            double k;
            if (mode == 0) k = (double)(rng() % nk);
            else if (mode == 1) k = (double)(i % nk);
            else if (mode == 2) k = (double)((n - i) / (1 + nk));
            else k = (double)(rng() % (n + 1));
            if (t % 7 == 0) {  // a median-of-three adversary: reaches the depth limit
                const int half = n / 2;
                if (i < half) k = (i % 2 == 0) ? i + 1 : half + i + (half % 2 == 0 ? 0 : 1);
                else k = (i - half + 1) * 2;
            }
            v[i] = {(uint32_t)i, k};
        }
        std::vector<double> key(n);
        std::vector<uint32_t> val(n);
        for (int i = 0; i < n; ++i) { key[i] = v[i].second; val[i] = v[i].first; }
        std::sort(v.begin(), v.end(), [](const std::pair<uint32_t, double> &a, const std::pair<uint32_t, double> &b) {
            return a.second < b.second;
        });
        plan::lib_sort(key.data(), val.data(), n);
        ++tests;
        for (int i = 0; i < n; ++i)
            if (val[i] != v[i].first || key[i] != v[i].second) { ++bad; break; }
    }
    std::printf("%ld %ld\n", bad, tests);
    return 0;
}
"""


def test_lib_sort_replays_std_sort(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    (tmp_path / "h.cpp").write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "plan_gb300" / "csrc"), str(tmp_path / "h.cpp"), "-o", str(exe)],
                   check=True)
    bad, tests = map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split())
    assert tests == 20000
    assert bad == 0
