"""Host side of the drop-in boundary, without a GPU: the C-ABI library loads and exports
every declared entry point, parameter files and .lis snapshots are read with the
reference's rules and errors, and the command line keeps the reference's argument handling.
"""
from __future__ import annotations

import ctypes as C
import math
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import cases
from conftest import ROOT

HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions() -> list[str]:
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*\b(plan_[A-Za-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_headers_declare_the_boundary():
    names = declared_functions()
    for must in ("plan_ctx_create", "plan_find_clumps", "plan_build_tree", "plan_find_planetesimals", "plan_params_read",
                 "plan_lis_read", "plan_catalogue_write_peaks", "plan_catalogue_basic_results", "plan_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(str(ROOT / "plan_gb300" / "lib" / "libplan_gpu.so"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(built.EXPORTED) <= set(declared_functions())


def test_nm_shows_only_c_symbols(built):
    """The boundary is extern "C": no mangled plan_ names are exported."""
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--defined-only", str(ROOT / "plan_gb300" / "lib" / "libplan_gpu.so")], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(declared_functions()) <= exported
    assert not [s for s in exported if s.startswith("_Z") and "plan_" in s and "plan_" == s[:5]]


def test_struct_layouts_match_the_header(built, tmp_path):
    """The ctypes mirrors of the ABI structs have the C sizes and field offsets."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    fields = {"plan_params": (built.Params, [f[0] for f in built.Params._fields_]),
              "plan_lis_view": (built.LisView, [f[0] for f in built.LisView._fields_]),
              "plan_clump_info": (built.ClumpInfo, [f[0] for f in built.ClumpInfo._fields_])}
    src = ["#include <cstddef>", "#include <cstdio>", '#include "plan_gpu.h"', "int main() {"]
    for st, (_, names) in fields.items():
        src.append(f'    std::printf("{st} %zu\\n", sizeof({st}));')
        for n in names:
            src.append(f'    std::printf("{st}.{n} %zu\\n", offsetof({st}, {n}));')
    src.append("}")
    (tmp_path / "l.cpp").write_text("\n".join(src) + "\n")
    subprocess.run(["g++", "-I", str(ROOT / "include"), str(tmp_path / "l.cpp"), "-o", str(tmp_path / "l")], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(tmp_path / "l")], capture_output=True, text=True, check=True).stdout.splitlines())
    for st, (cls, names) in fields.items():
        assert int(got[st]) == C.sizeof(cls), st
        for n in names:
            assert int(got[f"{st}.{n}"]) == getattr(cls, n).offset, (st, n)


def test_headers_are_plain_c(built, tmp_path):
    """The boundary is usable from C: both headers compile as C99 with every warning, and a C
    program links against the library and calls it (parameter defaults, no device needed)."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    (tmp_path / "c.c").write_text(
        '#include "plan_gpu.h"\n#include "plan_synth.h"\n#include <stdio.h>\n'
        "int main(void) { plan_params p; plan_params_init(&p); printf(\"%u %u %d\\n\", p.knn, p.hop, (int)p.user_box); return 0; }\n")
    lib = ROOT / "plan_gb300" / "lib"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", str(ROOT / "include"), str(tmp_path / "c.c"),
                    f"-L{lib}", "-lplan_gpu", f"-Wl,-rpath,{lib}", "-o", str(tmp_path / "c")], check=True)
    out = subprocess.run([str(tmp_path / "c")], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["64", "32", "0"]


# ---------------------------------------------------------------- parameters
def test_params_defaults(built):
    p = built.params()
    assert p.knn == 64 and p.hop == 32 and p.fixed_hop == 0
    assert p.solid_to_gas_ratio == 0.02 and list(p.box_resolution) == [128, 128, 128]
    assert p.q == 1.5 and p.Omega == 1.0 and p.four_pi_G == 0.05
    assert p.clump_diffuse_threshold < 0 and p.Hill_fraction_for_merge < 0


def test_params_file_rules(built, tmp_path):
    """src/global.cpp:51-225: comments, a/b fractions, aliases, first occurrence wins."""
    f = tmp_path / "p.txt"
    f.write_text("# comment\n<section>\nNx1 = 64   # trailing comment\nNx2=32\nNx3 = 16\nZ = 1/50\nfour_pi_G_par = 0.5\n"
                 "num_knn = 40\nknn = 48\nhop = 12\nnum_peaks = 5\nNx1 = 999\n")
    p = built.params(str(f))
    assert list(p.box_resolution) == [64, 32, 16]
    assert p.solid_to_gas_ratio == 1 / 50
    assert p.four_pi_G == 0.5
    assert p.knn == 48  # the last alias checked wins, as in the reference
    assert p.hop == 12 and p.fixed_hop == 1
    assert p.num_peaks == 5
    # derived values (CalculateNewParameters, src/global.cpp:28-47)
    assert p.cell_length[0] == 0.2 / 64 and p.cell_length[2] == 0.2 / 16
    assert p.mass_total_code_units == math.sqrt(2 * math.pi) * 0.2 * 0.2 * (1 / 50)
    assert p.grav_constant == 0.5 / (4 * math.pi)
    assert p.shear_speed == 1.5 * 1.0 * 0.2


def test_params_errors(built, tmp_path):
    with pytest.raises(built.PlanError) as e:
        built.params(str(tmp_path / "missing.txt"))
    assert e.value.status == 3
    f = tmp_path / "bad.txt"
    f.write_text("Z = abc\n")
    with pytest.raises(built.PlanError) as e:
        built.params(str(f))
    assert e.value.status == 4
    f.write_text("clump_diffuse_threshold = -1\n")
    with pytest.raises(built.PlanError) as e:
        built.params(str(f))
    assert e.value.status == 4


# ---------------------------------------------------------------- .lis input
def test_lis_read_combined(built, case_dir):
    m = case_dir("w1_20k_sheared")
    s = built.Snapshot(m["lis"])
    assert s.n == 20000
    assert abs(s.time - 0.37) < 1e-6 and s.time == float(np.float32(0.37))
    v = s.view
    assert [v.coor_lim[i] for i in range(6)] == [float(np.float32(x)) for x in (-0.1, 0.1, -0.1, 0.1, -0.1, 0.1)]
    assert v.ntypes == 1 and v.nblocks == 1
    s.close()


def test_lis_read_multiple_files(built, case_dir):
    m = case_dir("w1_24k_split2")
    s = built.Snapshot(m["lis"])
    assert s.n == 24000 and s.view.nblocks == 2
    s.close()


def test_lis_truncated_and_missing(built, case_dir, tmp_path):
    m = case_dir("w1_20k")
    blob = Path(m["lis"][0]).read_bytes()
    t = tmp_path / "cut.lis"
    t.write_bytes(blob[: len(blob) - 44 * 10 - 7])
    with pytest.raises(built.PlanError) as e:
        built.Snapshot(str(t))
    assert e.value.status == 3
    with pytest.raises(built.PlanError) as e:
        built.Snapshot(str(tmp_path / "nope.lis"))
    assert e.value.status == 3


# ---------------------------------------------------------------- synthetic workloads
def test_generator_workloads(built, tmp_path):
    """The named workloads have the configured mixture and put rho_thr at the mean density."""
    L = built.lib()
    for w, frac_u, frac_s, nc in ((1, 0.8, 0.0, 16), (2, 0.6, 0.25, 200), (5, 0.7, 0.2, 2000)):
        spec = built.SynthSpec()
        assert L.plan_synth_default_spec(w, 0, 1, C.byref(spec)) == 0
        assert abs(spec.frac_uniform - frac_u) < 1e-12 and abs(spec.frac_sheets - frac_s) < 1e-12
        assert spec.n_clumps == nc
    assert L.plan_synth_default_spec(1, 0, 1, C.byref(built.SynthSpec())) == 0
    assert L.plan_synth_default_spec(9, 0, 1, C.byref(built.SynthSpec())) != 0
    rec, _ = cases._records(cases.Case("x", 2, 200000, 4, 64))
    pos = rec["pos"]
    assert pos.min() >= -0.1 and pos.max() < 0.1
    # no two particles share a position in the generated workloads
    assert len(np.unique(pos.view(np.dtype((np.void, 12))))) == len(pos)


# ---------------------------------------------------------------- command line
CLI = ROOT / "plan_gb300" / "lib" / "plan_gpu"


def run_cli(args, **kw):
    return subprocess.run([str(CLI)] + args, capture_output=True, text=True, timeout=60, **kw)


def test_cli_usage(built):
    r = run_cli([])
    assert r.returncode == 0 and "USAGE" in r.stdout + r.stderr
    r = run_cli(["-c", "1", "-i", "d", "-b", "b", "-p", "p", "-f", "0:0", "-o", "o.txt", "-t", "x", "--Help"])
    assert r.returncode == 0 and "USAGE" in r.stdout + r.stderr


def test_cli_rejects_what_is_not_on_this_path(built, tmp_path):
    base = ["-c", "1", "-i", str(tmp_path), "-b", "b", "-p", "p", "-f", "0:0", "-o", str(tmp_path / "o.txt"), "-t", "x"]
    for extra in (["--Basic_Analyses"], ["--Temp_Calculation"]):
        r = run_cli(base + extra)
        assert r.returncode == 2, extra
    r = run_cli(base + ["stray"])
    assert r.returncode == 2
    r = run_cli(base + ["-q"])
    assert r.returncode == 2


def test_cli_parameter_file_errors_before_device(built, tmp_path):
    """A missing parameter file is reported (exit 3) before any device is touched."""
    base = ["-c", "1", "-i", str(tmp_path), "-b", "b", "-p", "p", "-f", "0:0", "-o", str(tmp_path / "o.txt"), "-t",
            str(tmp_path / "missing.txt"), "--Combined"]
    r = run_cli(base)
    assert r.returncode == 3


def test_footprint_grows_with_the_snapshot_and_fits_the_largest_workload(built):
    """The device-memory estimate the serving admission uses: monotone in the particle count,
    no overflow up to the largest count the path takes (2^32 - 16), about 35 GiB for the
    2^24-particle workload (a third of it the clump stage's member pool, capped at 24 GiB) and
    under the GB300's 280 GB for 2^27 particles."""
    L = built.lib()
    sizes = [0, 1, 1 << 16, 1 << 20, 1 << 24, 1 << 27, 0xFFFFFFF0]
    fp = [L.plan_footprint_bytes(n, None) for n in sizes]
    assert all(a < b for a, b in zip(fp, fp[1:]))
    assert 24 << 30 < fp[4] < 48 << 30
    assert fp[5] < 280 * 10**9
    assert fp[-1] < 1 << 50


def test_entry_points_refuse_null_handles(built):
    """Every entry point that takes a context, a server or a catalogue checks it before any
    device work: a null one is an argument error (status 2), as are zero workers."""
    import ctypes as C

    L = built.lib()
    p = built.params()
    v = built.LisView()
    out, n, u64, d = C.c_void_p(), C.c_int32(), C.c_uint64(), C.c_double()
    got = {
        "plan_build_tree": L.plan_build_tree(None, C.byref(v), C.byref(p), 1, None),
        "plan_find_planetesimals": L.plan_find_planetesimals(None, C.byref(p), None, C.byref(out)),
        "plan_find_clumps": L.plan_find_clumps(None, C.byref(v), C.byref(p), 1, None, C.byref(out)),
        "plan_density_vs_scale": L.plan_density_vs_scale(None, C.byref(p), 0.0, None, None, 0, C.byref(n)),
        "plan_group_energies": L.plan_group_energies(None, None, None, None, None, 0, C.byref(p), None, None, None),
        "plan_catalogue_write_parlists": L.plan_catalogue_write_parlists(None, None, 0, 1),
        "plan_ctx_release": L.plan_ctx_release(None),
        "plan_submit": L.plan_submit(None, C.byref(v), C.byref(p), 1, C.byref(u64)),
        "plan_poll": L.plan_poll(None, 1, 0, C.byref(out), C.byref(d)),
        "plan_server_stats": L.plan_server_stats(None, None, None),
        "plan_knn": L.plan_knn(None, None, 0, 32, 0.0, None, None),
        "plan_morton_order": L.plan_morton_order(None, None, 0, None),
        "plan_morton_order_noalloc": L.plan_morton_order_noalloc(None, None, 0, None),
        "plan_stage_times": L.plan_stage_times(None, None, 0),
        "plan_counters": L.plan_counters(None, None, 0),
        "plan_server_create (0 workers)": L.plan_server_create(0, 0, 0, C.byref(out)),
    }
    assert got == {k: 2 for k in got}


def test_no_device_no_fallback(built):
    """Without a CUDA device every device entry point fails with status 5: the context, the
    serving loop, and so every computation behind them. There is no CPU path to fall back on."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(built.PlanError) as e:
        built.Finder(0)
    assert e.value.status == 5
    with pytest.raises(built.PlanError) as e:
        built.Server(0, 2, 0)
    assert e.value.status == 5
