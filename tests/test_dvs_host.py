"""The device's --Density_Vs_Scale arithmetic on the CPU, on the oracle's tree (no GPU).

plan_gb300/csrc/dvs.cuh holds what the GPU runs for BasicAnalysesWithTree: the grid set-up,
the decoding of a query thread into its centre and radius, the sheared tree walk and the
density of the largest count. Compiled here with g++ and run over every query on the
oracle's tree (built as that analysis builds it: 64-point leaves, no ghosts), it must give
the oracle's radii and densities bit for bit, and those are the reference's (the RMPL line).
"""
from __future__ import annotations

import ctypes as C
import json
import shutil
import subprocess

import numpy as np
import pytest

import cases
from conftest import GOLDEN, ROOT

SHIM = r"""
#include <cstdint>
#include <vector>
#include "dvs.cuh"

struct HostTree {
    const double *f4;
    const uint32_t *u7;
    const double *p3;
    void node(uint32_t n, double &x, double &y, double &z, double &hw) const { x = f4[4 * n]; y = f4[4 * n + 1]; z = f4[4 * n + 2]; hw = f4[4 * n + 3]; }
    uint32_t begin(uint32_t n) const { return u7[7 * n]; }
    uint32_t end(uint32_t n) const { return u7[7 * n + 1]; }
    uint32_t first(uint32_t n) const { return u7[7 * n + 3]; }
    uint32_t daughters(uint32_t n) const { return u7[7 * n + 5]; }
    void point(uint32_t q, double &x, double &y, double &z) const { x = p3[3 * q]; y = p3[3 * q + 1]; z = p3[3 * q + 2]; }
};

extern "C" int dvs_setup_status(const double *q19, double time, double zlo, double zhi) {
    plan::DvsParams p;
    for (int d = 0; d < 3; ++d) {
        p.box_length[d] = q19[d]; p.box_min[d] = q19[3 + d]; p.box_max[d] = q19[6 + d]; p.box_center[d] = q19[9 + d];
        p.cell_length[d] = q19[14 + d];
    }
    p.box_half_width0 = q19[12]; p.max_half_width = q19[13]; p.shear_speed = q19[17]; p.mass_per_particle0 = q19[18];
    plan::DvsGeom g;
    std::vector<double> xs, ys, zs;
    return plan::dvs_setup(p, time, zlo, zhi, g, xs, ys, zs);
}

extern "C" int dvs_host(const double *f4, const uint32_t *u7, const double *p3, uint32_t np, const double *q19, double time, double *radii,
                        double *rho, int cap) {
    plan::DvsParams p;
    for (int d = 0; d < 3; ++d) {
        p.box_length[d] = q19[d]; p.box_min[d] = q19[3 + d]; p.box_max[d] = q19[6 + d]; p.box_center[d] = q19[9 + d];
        p.cell_length[d] = q19[14 + d];
    }
    p.box_half_width0 = q19[12]; p.max_half_width = q19[13]; p.shear_speed = q19[17]; p.mass_per_particle0 = q19[18];
    double zlo = p3[2], zhi = p3[2];
    for (uint32_t q = 0; q < np; ++q) { if (p3[3 * q + 2] < zlo) zlo = p3[3 * q + 2]; if (p3[3 * q + 2] > zhi) zhi = p3[3 * q + 2]; }
    plan::DvsGeom g;
    std::vector<double> xs, ys, zs;
    if (plan::dvs_setup(p, time, zlo, zhi, g, xs, ys, zs)) return -1;
    std::vector<uint32_t> maxc(g.nlev, 0);
    HostTree t{f4, u7, p3};
    const uint64_t n = (uint64_t)g.nx * g.ny * g.nz * g.nvar;
    for (uint64_t tid = 0; tid < n; ++tid) {
        double x, y, z;
        int lev;
        plan::dvs_query(g, xs.data(), ys.data(), zs.data(), tid, x, y, z, lev);
        bool over = false;
        uint32_t c = plan::dvs_count(t, x, y, z, g.radius[lev], g.maxd[lev], g, &over);
        if (over) return -2;
        if (c > maxc[lev]) maxc[lev] = c;
    }
    for (int i = 0; i < g.nlev && i < cap; ++i) { radii[i] = g.radius[i]; rho[i] = plan::dvs_density(maxc[i], g.radius[i], p.mass_per_particle0); }
    return g.nlev;
}
"""


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("dvs_shim")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "libshim.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I", str(ROOT / "plan_gb300" / "csrc"),
                    str(d / "shim.cpp"), "-o", str(so)], check=True)
    L = C.CDLL(str(so))
    L.dvs_host.restype = C.c_int
    L.dvs_host.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int]
    return L


@pytest.fixture(scope="module")
def oracle_mod(built):
    from plan_gb300 import build as b

    b.build_oracle()
    import oracle

    return oracle


@pytest.mark.parametrize("name", ["w1_20k_dvs16", "w1_20k_dvs32_sheared"])
def test_device_dvs_arithmetic_matches_oracle(name, shim, oracle_mod, tmp_path):
    _, case, _ = next(v for v in cases.DVS if v[0] == name)
    m = cases.materialise(case, tmp_path / "in")
    o = oracle_mod.Oracle(m["lis"], m["param"], threads=1, pow_mode=0, density_vs_scale=True)
    r_o, v_o = o.density_vs_scale()
    f = o.points()[0]
    p3 = np.ascontiguousarray(f[:, :3])
    f4, u7 = o.nodes()
    f4 = np.ascontiguousarray(f4, dtype=np.float64)
    u7 = np.ascontiguousarray(u7, dtype=np.uint32)
    q19 = o.density_vs_scale_params()
    time = float(np.float32(case.time))
    r_h, v_h = np.zeros(32), np.zeros(32)
    n = shim.dvs_host(f4.ctypes.data, u7.ctypes.data, p3.ctypes.data, len(p3), q19.ctypes.data, time, r_h.ctypes.data, v_h.ctypes.data,
                      32)
    assert n == len(r_o) > 0
    np.testing.assert_array_equal(r_h[:n], r_o)
    np.testing.assert_array_equal(v_h[:n], v_o)
    # and they are the reference's RMPL line
    meta = json.loads((GOLDEN / name / "meta.json").read_text())
    rmpl = (GOLDEN / name / "res_RMPL.txt").read_text().splitlines()
    assert rmpl[1] == "%15.6e" % time + "".join("%15.6e" % x for x in v_h[:n])
    assert meta["files"]


def test_dvs_setup_refuses_grids_it_cannot_launch(shim, oracle_mod, tmp_path):
    """The grid set-up's limits, on a golden's parameters with ever finer cells: the golden's
    own grid is accepted; 2^21 centres per axis give more queries than one launch takes (-3);
    more than 2^24 centres along an axis are refused before they are made (-2)."""
    import ctypes as C

    shim.dvs_setup_status.restype = C.c_int
    shim.dvs_setup_status.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
    _, case, _ = cases.DVS[0]
    m = cases.materialise(case, tmp_path / "in")
    o = oracle_mod.Oracle(m["lis"], m["param"], threads=1, pow_mode=0, density_vs_scale=True)
    q19 = np.ascontiguousarray(o.density_vs_scale_params(), dtype=np.float64)
    zlo, zhi = -0.01, 0.01
    assert shim.dvs_setup_status(q19.ctypes.data, 0.0, zlo, zhi) == 0
    fine = q19.copy()
    fine[14:17] = q19[0:3] / 2.0**21
    assert shim.dvs_setup_status(fine.ctypes.data, 0.0, zlo, zhi) == -3
    finer = q19.copy()
    finer[14:17] = q19[0:3] / 2.0**25
    assert shim.dvs_setup_status(finer.ctypes.data, 0.0, zlo, zhi) == -2
