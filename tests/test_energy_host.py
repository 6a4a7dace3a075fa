"""The batched boundness arithmetic on the CPU (no GPU).

plan_gb300/csrc/energy.cuh holds what the GPU runs per pair tile: the decoding of a queue
item into its tile of the upper triangle and the FP32 row sums with compensated addition.
Compiled here with g++, the whole tiled pass (tiles, 128-thread rows, the block's FP64 tree
reduction) is replayed over groups of the workload's kind and compared with an FP64 direct
sum: the potential energy must agree to 1e-6 relative (the stated tolerance), the kinetic
energy to FP64 rounding.
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SHIM = r"""
#include <cstdint>
#include <vector>
#include "energy.cuh"

using namespace plan;

extern "C" int pair_items_host(const uint64_t *offsets, uint32_t ngroups, uint64_t *out) {
    std::vector<uint64_t> v;
    const int rc = pair_items(offsets, ngroups, v);
    for (size_t i = 0; i < v.size(); ++i) out[i] = v[i];
    return rc;
}

extern "C" int tiles_cover(uint64_t T) {
    std::vector<uint8_t> seen(T * T, 0);
    const uint64_t n = T * (T + 1) / 2;
    for (uint64_t l = 0; l < n; ++l) {
        uint64_t ti, tj;
        tile_of(l, T, ti, tj);
        if (ti >= T || tj >= T || tj < ti || seen[ti * T + tj]) return 0;
        seen[ti * T + tj] = 1;
    }
    return 1;
}

// the GPU's pass over one group, replayed: every w x w tile, w row threads, FP64 tree
// reduction per tile into its own slot, then the slots added in tile order
extern "C" double pair_sum_host_w(const float *pos3, const float *mass, uint64_t n, int w, uint64_t *zeros_out) {
    const uint64_t T = (n + w - 1) / w;
    double total = 0.0;
    uint64_t zeros = 0;
    std::vector<PairParticle> col(w);
    std::vector<double> red(w);
    for (uint64_t l = 0; l < T * (T + 1) / 2; ++l) {
        uint64_t ti, tj;
        tile_of(l, T, ti, tj);
        const uint64_t c0 = tj * w;
        for (int t = 0; t < w; ++t)
            if (c0 + t < n) col[t] = PairParticle{pos3[3 * (c0 + t)], pos3[3 * (c0 + t) + 1], pos3[3 * (c0 + t) + 2], mass[c0 + t]};
        for (int t = 0; t < w; ++t) {
            const uint64_t r = ti * w + t;
            float s = 0.f, c = 0.f;
            uint32_t z = 0;
            double mrow = 0;
            if (r < n) {
                const uint32_t cn = (uint32_t)(n - c0 < (uint64_t)w ? n - c0 : (uint64_t)w);
                pair_row_sum(PairParticle{pos3[3 * r], pos3[3 * r + 1], pos3[3 * r + 2], mass[r]}, col.data(), cn, ti == tj ? t : -1, s, c, z);
                mrow = mass[r];
            }
            red[t] = mrow * ((double)s + (double)c);
            zeros += z;
        }
        for (int h = w / 2; h > 0; h >>= 1)
            for (int t = 0; t < h; ++t) red[t] += red[t + h];
        total += red[0];
    }
    *zeros_out = zeros;
    return total;
}

extern "C" double pair_sum_host(const float *pos3, const float *mass, uint64_t n, uint64_t *zeros_out) {
    return pair_sum_host_w(pos3, mass, n, kPairTile, zeros_out);
}

extern "C" int energy_class_host(uint64_t n) { return energy_class(n); }

extern "C" int energy_table_ok() {
    for (int k = 0; k < kEnergyClasses; ++k)
        if (!energy_tile_ok(kEnergyTile[k])) return 0;
    for (int k = 0; k + 1 < kEnergyClasses - 1; ++k)
        if (kEnergyClassBound[k] >= kEnergyClassBound[k + 1]) return 0;
    return 1;
}

extern "C" int pair_items_tile_host(const uint64_t *offsets, uint32_t ngroups, uint32_t tile, uint64_t *out) {
    std::vector<uint64_t> v;
    const int rc = pair_items(offsets, ngroups, v, tile);
    for (size_t i = 0; i < v.size(); ++i) out[i] = v[i];
    return rc;
}
"""


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("energy_shim")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "libshim.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I", str(ROOT / "plan_gb300" / "csrc"),
                    str(d / "shim.cpp"), "-o", str(so)], check=True)
    L = C.CDLL(str(so))
    L.tiles_cover.restype = C.c_int
    L.tiles_cover.argtypes = [C.c_uint64]
    L.pair_sum_host.restype = C.c_double
    L.pair_sum_host.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
    L.pair_sum_host_w.restype = C.c_double
    L.pair_sum_host_w.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.POINTER(C.c_uint64)]
    L.energy_class_host.restype = C.c_int
    L.energy_class_host.argtypes = [C.c_uint64]
    L.pair_items_tile_host.restype = C.c_int
    L.pair_items_tile_host.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
    return L


def plummer_group(n: int, seed: int):
    """n equal-mass particles of a Plummer sphere (scale 1e-3) in float32, as the workload's clumps."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(1e-6, 0.99, n)
    r = 1e-3 / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    pos = (np.array([0.031, -0.047, 0.002]) + r[:, None] * v).astype(np.float32)
    vel = rng.normal(scale=1e-3, size=(n, 3)).astype(np.float32)
    mass = np.full(n, 4.0106053e-08, dtype=np.float32)
    return pos, vel, mass


def fp64_potential_sum(pos, mass) -> float:
    p = pos.astype(np.float64)
    m = mass.astype(np.float64)
    tot = 0.0
    for i in range(len(p) - 1):
        d = np.sqrt(((p[i + 1:] - p[i]) ** 2).sum(axis=1))
        tot += float((m[i] * m[i + 1:] / d).sum())
    return tot


def test_tiles_cover_the_upper_triangle(shim):
    for T in list(range(1, 200)) + [511, 1024, 4097]:
        assert shim.tiles_cover(T) == 1, T


@pytest.mark.parametrize("n", [2, 31, 128, 129, 500, 1000, 3000])
def test_tiled_fp32_pass_within_tolerance(n, shim):
    pos, vel, mass = plummer_group(n, n)
    z = C.c_uint64()
    got = shim.pair_sum_host(pos.ctypes.data, mass.ctypes.data, n, C.byref(z))
    want = fp64_potential_sum(pos, mass)
    assert z.value == 0
    assert abs(got - want) <= 1e-6 * abs(want), (got, want)


def test_coincident_pairs_left_out(shim):
    pos, vel, mass = plummer_group(300, 9)
    pos[7] = pos[3]
    pos[200] = pos[3]
    z = C.c_uint64()
    got = shim.pair_sum_host(pos.ctypes.data, mass.ctypes.data, 300, C.byref(z))
    assert z.value == 3  # the three pairs among particles 3, 7 and 200
    keep = np.ones(300, bool)
    p, m = pos.astype(np.float64), mass.astype(np.float64)
    tot = 0.0
    for i in range(299):
        d = np.sqrt(((p[i + 1:] - p[i]) ** 2).sum(axis=1))
        ok = d > 0
        tot += float((m[i] * m[i + 1:][ok] / d[ok]).sum())
    assert abs(got - tot) <= 1e-6 * tot and keep.all()


def test_pair_items_over_groups(shim):
    """The tile queue over all groups: each group's T (T + 1) / 2 upper-triangle tiles of 128,
    empty groups none, and decreasing offsets refused."""
    shim.pair_items_host.restype = C.c_int
    shim.pair_items_host.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
    off = np.array([0, 0, 1, 129, 300, 300 + 128 * 5], dtype=np.uint64)
    out = np.zeros(len(off), dtype=np.uint64)
    assert shim.pair_items_host(off.ctypes.data, len(off) - 1, out.ctypes.data) == 0
    assert out.tolist() == [0, 0, 1, 2, 5, 20]  # n = 0, 1, 128, 171, 640: T = 0, 1, 1, 2, 5
    bad = np.array([0, 10, 5], dtype=np.uint64)
    assert shim.pair_items_host(bad.ctypes.data, 2, out.ctypes.data) == -1


@pytest.mark.parametrize("w", [32, 64, 128, 256])
@pytest.mark.parametrize("n", [2, 33, 300, 1000])
def test_tiled_pass_every_tile_width(w, n, shim):
    """Every width the pass is built for (one per size class) covers each pair once and stays
    within the stated 1e-6 of the FP64 direct sum."""
    pos, vel, mass = plummer_group(n, 7 * n + w)
    z = C.c_uint64()
    got = shim.pair_sum_host_w(pos.ctypes.data, mass.ctypes.data, n, w, C.byref(z))
    want = fp64_potential_sum(pos, mass)
    assert z.value == 0
    assert abs(got - want) <= 1e-6 * abs(want), (w, n, got, want)


def test_size_classes_and_their_queues(shim):
    """Groups of n < 64, < 512, < 8192 and larger particles are classes 0-3; the measured
    table holds widths the pass is built for; each class's queue counts its groups' tiles at
    its own width."""
    assert shim.energy_table_ok() == 1
    got = [shim.energy_class_host(n) for n in (0, 1, 63, 64, 511, 512, 8191, 8192, 10 ** 7)]
    assert got == [0, 0, 0, 1, 1, 2, 2, 3, 3]
    off = np.array([0, 31, 64, 97, 97 + 256], dtype=np.uint64)  # n = 31, 33, 33, 256
    out = np.zeros(len(off), dtype=np.uint64)
    assert shim.pair_items_tile_host(off.ctypes.data, len(off) - 1, 32, out.ctypes.data) == 0
    assert out.tolist() == [0, 1, 4, 7, 43]  # T = 1, 2, 2, 8 tiles per side at width 32
