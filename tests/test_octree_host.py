"""The device's octree rules on the CPU, against the oracle's tree (no GPU).

plan_gb300/csrc/octree_rules.cuh holds the per-point rules the GPU builds the octree with
(shared prefix with the previous key, the (leaf size + 1)-key windows, the leaf level, where
a node starts). Compiled here with g++ and applied to the oracle's sorted keys, they must
give exactly the oracle's nodes (level and first point of every node), which equal the
reference's: with 8-point leaves on the golden snapshots and with the 64-point leaves of
--Density_Vs_Scale runs.
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess

import numpy as np
import pytest

import cases
from conftest import ROOT

SHIM = r"""
#include <cmath>
#include <cstdint>
#include <vector>
#include "octree_rules.cuh"

template <uint32_t LEAF>
static uint64_t nodes(const uint32_t *k, uint32_t n, uint32_t *out, uint64_t cap) {
    std::vector<uint32_t> k0(n), k1(n), k2(n);
    for (uint32_t i = 0; i < n; ++i) { k0[i] = k[3 * i]; k1[i] = k[3 * i + 1]; k2[i] = k[3 * i + 2]; }
    std::vector<uint8_t> a(n), win(n), leaf(n);
    for (uint32_t i = 0; i < n; ++i) {
        a[i] = plan::octree_prev_lcp(k0.data(), k1.data(), k2.data(), i);
        win[i] = plan::octree_window_lcp<LEAF>(k0.data(), k1.data(), k2.data(), n, i);
    }
    for (uint32_t i = 0; i < n; ++i) leaf[i] = plan::octree_leaf_level<LEAF>(win.data(), i);
    uint64_t m = 0;
    if (m < cap) { out[2 * m] = 1; out[2 * m + 1] = 0; }  // the root
    ++m;
    for (uint32_t i = 0; i < n; ++i)
        for (int L = 1; L < 32; ++L)
            if (plan::starts_level(L, a[i], leaf[i])) {
                if (m < cap) { out[2 * m] = (uint32_t)(L + 1); out[2 * m + 1] = i; }
                ++m;
            }
    return m;
}

extern "C" uint64_t octree_nodes(const uint32_t *keys3, uint32_t n, int leaf, uint32_t *out, uint64_t cap) {
    return leaf == 64 ? nodes<64>(keys3, n, out, cap) : nodes<8>(keys3, n, out, cap);
}
"""


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from plan_gb300 import build as b

    d = tmp_path_factory.mktemp("octree_shim")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "libshim.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(ROOT / "plan_gb300" / "csrc"), "-I",
                    str(b._cuda_home() / "include"), str(d / "shim.cpp"), "-o", str(so)], check=True)
    L = C.CDLL(str(so))
    L.octree_nodes.restype = C.c_uint64
    L.octree_nodes.argtypes = [C.c_void_p, C.c_uint32, C.c_int, C.c_void_p, C.c_uint64]
    return L


@pytest.fixture(scope="module")
def oracle_mod(built):
    from plan_gb300 import build as b

    b.build_oracle()
    import oracle

    return oracle


# snapshots of 1 to 14 particles (with their ghosts): trees whose root is a leaf or has only
# a few leaves, as the clump trees of the merge sweeps often are
TINY = [cases.Case(f"tiny_{nb}_{nc}", 1, 20000, 5, 32, edit=f"small:{nb}:{nc}") for nb, nc in ((1, 0), (5, 0), (0, 8), (3, 6), (0, 14))]


def _by_case(name):
    for c in cases.CASES + cases.SPLINE + cases.SMALL + TINY:
        if c.name == name:
            return c, False
    for v in cases.DVS:
        if v[0] == name:
            return v[1], True
    raise KeyError(name)


@pytest.mark.parametrize("name", [c.name for c in cases.CASES + cases.SPLINE + cases.SMALL + TINY] + [v[0] for v in cases.DVS[::2]])
def test_octree_rules_give_the_oracle_nodes(name, shim, oracle_mod, tmp_path):
    case, dvs = _by_case(name)
    m = cases.materialise(case, tmp_path / "in")
    o = oracle_mod.Oracle(m["lis"], m["param"], threads=1, density_vs_scale=dvs)
    keys = np.ascontiguousarray(o.keys(), dtype=np.uint32)
    f4, u7 = o.nodes()
    want = sorted(zip(u7[:, 6].tolist(), u7[:, 0].tolist()))
    out = np.zeros(2 * (len(want) + 16), dtype=np.uint32)
    got_n = shim.octree_nodes(keys.ctypes.data, len(keys), 64 if dvs else 8, out.ctypes.data, len(want) + 16)
    assert got_n == len(want)
    got = sorted(zip(out[0:2 * got_n:2].tolist(), out[1:2 * got_n:2].tolist()))
    assert got == want
