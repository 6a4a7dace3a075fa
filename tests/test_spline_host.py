"""The device's spline-density formula, compiled for the CPU, against the oracle (CPU only).

plan_gb300/csrc/spline.cuh holds the arithmetic of the GPU's spline kernel as host+device
functions. Built here with g++ (no contraction) and fed the oracle's own KNN lists, it must
give every tree point's density bit for bit as the oracle does, on both spline snapshots.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import cases
from conftest import ROOT, golden

SHIM = r"""
#include <cstdint>
#include "spline.cuh"
struct P4 { double x, y, z, w; };
extern "C" void spline_density_host(const double *pos4, const uint32_t *idx, int k, int nq, const double *cl3, double vol,
                                    double *out) {
    const plan::SplineCells c = plan::spline_cells(cl3, vol);
    const P4 *p = reinterpret_cast<const P4 *>(pos4);
    for (int i = 0; i < nq; ++i) {
        const uint32_t *row = idx + (size_t)i * k;
        out[i] = plan::spline_density(p, [&](int j) { return row[j]; }, k, p[i].x, p[i].y, p[i].z, c);
    }
}
"""


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("spline_shim")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "libshim.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I", str(ROOT / "plan_gb300" / "csrc"),
                    str(d / "shim.cpp"), "-o", str(so)], check=True)
    L = C.CDLL(str(so))
    L.spline_density_host.restype = None
    L.spline_density_host.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_void_p]
    return L


@pytest.fixture(scope="module")
def oracle_mod(built):
    from plan_gb300 import build as b

    b.build_oracle()
    import oracle

    return oracle


@pytest.mark.parametrize("name", [c.name for c in cases.SPLINE])
def test_spline_formula_matches_oracle(name, shim, oracle_mod, case_dir, built):
    m = case_dir(name)
    p = built.params(m["param"])
    # the box comes from the snapshot header's float limits (src/tree.hpp:1565-1569), then the
    # derived cell constants follow from it
    lim = np.fromfile(m["lis"][0], dtype="<f4", count=12).astype(np.float64)
    for d in range(3):
        p.box_length[d] = lim[7 + 2 * d] - lim[6 + 2 * d]
    built.lib().plan_params_derive(C.byref(p))
    o = oracle_mod.Oracle(m["lis"], m["param"], threads=os.cpu_count() or 1, pow_mode=1)
    o.find()
    f = o.points()[0]
    assert len(f) == golden(name)["n_tree"]
    # the spline kernel runs only below four particles per horizontal cell
    assert c_n(name) < 4 * p.box_resolution[0] * p.box_resolution[1]
    k = int(p.knn)
    idx, _ = o.knn(np.ascontiguousarray(f[:, :3]), k)
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    pos4 = np.ascontiguousarray(np.stack([f[:, 0], f[:, 1], f[:, 2], f[:, 6]], axis=1))
    cl = np.array([p.cell_length[0], p.cell_length[1], p.cell_length[2]], dtype=np.float64)
    out = np.zeros(len(f))
    shim.spline_density_host(pos4.ctypes.data, idx.ctypes.data, k, len(f), cl.ctypes.data, p.cell_volume, out.ctypes.data)
    np.testing.assert_array_equal(out, f[:, 8])
    assert cases.digest_density(out) == golden(name)["density"]


def c_n(name: str) -> int:
    return cases.BY_NAME[name].n
