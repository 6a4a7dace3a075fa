"""Command-line and parameter variants through the drop-in binary on the GPU (needs a GB300).

Each variant of tests/cases.py (sub-sampled member lists with -s, the num_peaks cap,
--No_Ghost, the merge parameters, and -x/-y/-z user boxes) runs the plan_gpu binary with the
reference's command line; its summary line, catalogue, basic-results file and every
--Save_Clumps member list must equal the reference's own files. The member lists formatted
on the device (plan_catalogue_write_parlists) must equal the host-formatted ones.
"""
from __future__ import annotations

import json
import os
import subprocess

import pytest

import cases
from conftest import GOLDEN, ROOT, golden, run_isolated

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,case,extra", cases.VARIANTS, ids=[v[0] for v in cases.VARIANTS])
def test_cli_variants(name, case, extra, built, tmp_path):
    g = GOLDEN / name
    meta = json.loads((g / "meta.json").read_text())
    m = cases.materialise(case, tmp_path / "in")
    assert m["sha256"] == meta["lis_sha256"]
    out = tmp_path / "out"
    out.mkdir()
    cli = ROOT / "plan_gb300" / "lib" / "plan_gpu"
    r = subprocess.run([str(cli)] + cases.cli_args(m, str(out / "res.txt")) + extra, cwd=out, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert meta["summary"] in r.stdout
    assert (out / meta["peaks_file"]).read_bytes() == (g / meta["peaks_file"]).read_bytes()
    assert (out / "res_planetesimals.txt").read_bytes() == (g / "planetesimals.txt").read_bytes()
    assert cases.parlist_digests(out) == meta["parlist"]


@pytest.mark.parametrize("name,sampling", [("w1_20k", 1), ("w1_20k_sinks", 1), ("w1_20k", 3)])
def test_device_member_lists(name, sampling, request, built, case_dir, tmp_path, monkeypatch):
    """Member lists formatted on the device equal the host-formatted ones byte for byte (and
    so the reference's): same files, same lines, every sub-sampling."""
    if run_isolated(request):
        return
    m = case_dir(name)
    p = built.params(m["param"])
    snap = built.Snapshot(m["lis"])
    f = built.Finder(0)
    try:
        cat = f.find_clumps(snap, p)
        (tmp_path / "host").mkdir()
        (tmp_path / "dev").mkdir()
        monkeypatch.chdir(tmp_path / "host")
        cat.write_peaks(str(tmp_path / "host" / "res.txt"), save_clumps=True, file_number=0, sampling=sampling)
        monkeypatch.chdir(tmp_path / "dev")
        f.write_parlists(cat, file_number=0, sampling=sampling)
        host = sorted((tmp_path / "host" / "ParList.0000").iterdir())
        dev = sorted((tmp_path / "dev" / "ParList.0000").iterdir())
        assert [h.name for h in host] == [d.name for d in dev] and host
        for h, d in zip(host, dev):
            assert h.read_bytes() == d.read_bytes(), h.name
        if sampling == 1:
            assert cases.parlist_digests(tmp_path / "dev") == golden(name)["parlist"]
        cat.close()
    finally:
        f.close()
        snap.close()


def test_cli_device_member_lists(built, tmp_path):
    """The drop-in binary with PLAN_PARLIST_DEVICE=1 writes the reference's sub-sampled lists."""
    name, case, extra = next(v for v in cases.VARIANTS if v[0] == "w1_20k_parlist_s3")
    meta = json.loads((GOLDEN / name / "meta.json").read_text())
    m = cases.materialise(case, tmp_path / "in")
    out = tmp_path / "out"
    out.mkdir()
    cli = ROOT / "plan_gb300" / "lib" / "plan_gpu"
    env = dict(os.environ, PLAN_PARLIST_DEVICE="1")
    r = subprocess.run([str(cli)] + cases.cli_args(m, str(out / "res.txt")) + extra, cwd=out, capture_output=True, text=True,
                       timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    assert cases.parlist_digests(out) == meta["parlist"]


@pytest.mark.parametrize("name,case,extra", cases.DVS, ids=[v[0] for v in cases.DVS])
def test_cli_density_vs_scale(name, case, extra, built, tmp_path):
    """--Density_Vs_Scale through the drop-in binary: the RMPL file of sheared ball counts,
    the clump finder on that run's tree (64-point leaves, no ghosts) and the reference's
    routing of the basic results, every file byte for byte."""
    g = GOLDEN / name
    meta = json.loads((g / "meta.json").read_text())
    m = cases.materialise(case, tmp_path / "in")
    assert m["sha256"] == meta["lis_sha256"]
    out = tmp_path / "out"
    out.mkdir()
    cli = ROOT / "plan_gb300" / "lib" / "plan_gpu"
    r = subprocess.run([str(cli)] + cases.cli_args(m, str(out / "res.txt")) + extra, cwd=out, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln] == meta["summary"]
    assert sorted(p.name for p in out.iterdir() if p.is_file()) == meta["files"]
    for f in meta["files"]:
        assert (out / f).read_bytes() == (g / f).read_bytes(), f
    assert cases.parlist_digests(out) == meta["parlist"]


def test_density_vs_scale_through_the_binding(request, built, tmp_path):
    """plan_density_vs_scale called directly (Finder.density_vs_scale) on a tree built for it:
    the radii and densities equal the oracle's, which equal the reference's, bit for bit."""
    if run_isolated(request):
        return
    import oracle

    name, case, _ = cases.DVS[2]  # the sheared one, at t = 0.37
    m = cases.materialise(case, tmp_path / "in")
    p = built.params(m["param"])
    p.density_vs_scale = 1
    snap = built.Snapshot(m["lis"])
    f = built.Finder(0)
    try:
        f.build_tree(snap, p)
        radii, rho = f.density_vs_scale(p, snap.view.time)
    finally:
        f.close()
        snap.close()
    o = oracle.Oracle(m["lis"], m["param"], threads=1, density_vs_scale=True)
    r_o, v_o = o.density_vs_scale()
    assert radii.tobytes() == r_o.tobytes()
    assert rho.tobytes() == v_o.tobytes()


def test_cli_two_snapshots_density_vs_scale(built, tmp_path):
    """The drop-in binary over two snapshots with --Density_Vs_Scale alone writes the
    reference's files (one RMPL header, lines and basic results interleaved)."""
    from test_oracle_golden import _multi_inputs, multi_snapshot_args

    g = GOLDEN / "multi_density_vs_scale"
    meta = json.loads((g / "meta.json").read_text())
    d, _ = _multi_inputs(tmp_path)
    out = tmp_path / "out"
    out.mkdir()
    cli = ROOT / "plan_gb300" / "lib" / "plan_gpu"
    r = subprocess.run([str(cli)] + multi_snapshot_args(d, out) + ["--Density_Vs_Scale"], cwd=out, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln] == meta["summary"]
    assert sorted(p.name for p in out.iterdir() if p.is_file()) == meta["files"]
    for f in meta["files"]:
        assert (out / f).read_bytes() == (g / f).read_bytes(), f
