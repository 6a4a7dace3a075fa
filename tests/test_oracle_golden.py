"""The oracle restatement against the reference's own outputs (CPU only).

Golden fixtures come from the unmodified reference run on the same snapshots
(tests/golden/make_golden.py). These tests pin the oracle before it is trusted to check the
GPU: every stage digest and both output files must be identical.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import cases
from conftest import GOLDEN, golden

CPU_CASES = [c.name for c in cases.CASES + cases.SPLINE + cases.SMALL]


@pytest.fixture(scope="module")
def oracle_mod(built):
    from plan_gb300 import build as b

    b.build_oracle()
    import oracle

    return oracle


@pytest.mark.parametrize("name", CPU_CASES)
def test_snapshot_bytes_pinned(name, case_dir):
    """The generator and the case edits reproduce the golden snapshot bytes."""
    m = case_dir(name)
    assert m["sha256"] == golden(name)["lis_sha256"]


@pytest.mark.parametrize("name", CPU_CASES)
def test_oracle_matches_reference(name, case_dir, oracle_mod, tmp_path):
    g = golden(name)
    m = case_dir(name)
    o = oracle_mod.Oracle(m["lis"], m["param"], threads=os.cpu_count() or 1, pow_mode=0)
    o.find()
    f, orig, sink = o.points()
    assert len(f) == g["n_tree"]
    assert cases.digest_keys(o.keys()) == g["keys"]
    assert cases.digest_points(f, orig, sink) == g["points"]
    assert int(sink.sum()) == g["n_sinks"]
    assert cases.digest_nodes(*o.nodes()) == g["nodes"]
    assert cases.digest_density(f[:, 8]) == g["density"]
    assert cases.digest_u32(o.densest()) == g["densest"]
    assert cases.digest_clumps(*o.clumps()) == g["clumps"]
    assert o.summary().strip() == g["summary"]
    # output files, byte for byte
    out = tmp_path / "res.txt"
    o.write_outputs(str(out), first=True)
    assert (tmp_path / g["peaks_file"]).read_bytes() == (GOLDEN / name / g["peaks_file"]).read_bytes()
    assert (tmp_path / "res_planetesimals.txt").read_bytes() == (GOLDEN / name / "planetesimals.txt").read_bytes()


@pytest.mark.parametrize("name", ["w1_20k", "w1_20k_sinks", "config1_262k"])
def test_oracle_knn_matches_reference(name, case_dir, oracle_mod):
    """The approximate KNN (radius doubling, heap order) of every strided query point."""
    g = golden(name)
    m = case_dir(name)
    o = oracle_mod.Oracle(m["lis"], m["param"], threads=1, pow_mode=0)
    f = o.points()[0]
    q = f[:: g["knn_stride"], :3]
    idx, dr2 = o.knn(q, g["knn_k"])
    assert cases.digest_knn(idx, dr2) == g["knn"]


@pytest.mark.parametrize("name", ["w1_20k", "w1_20k_sinks", "config1_262k"])
def test_oracle_correctly_rounded_pow(name, case_dir, oracle_mod):
    """With a correctly rounded pow(x, 1.5) (the GPU's) the densities move by at most a few
    units in the last place and every catalogue digest stays the same."""
    g = golden(name)
    m = case_dir(name)
    o0 = oracle_mod.Oracle(m["lis"], m["param"], pow_mode=0)
    o0.find()
    o1 = oracle_mod.Oracle(m["lis"], m["param"], pow_mode=1)
    o1.find()
    d0, d1 = o0.points()[0][:, 8], o1.points()[0][:, 8]
    assert cases.digest_density(d1) == g["density_cr"]
    rel = np.abs(d1 - d0) / np.abs(d0)
    assert float(rel.max()) <= 1e-15  # far inside the stated density tolerance of 1e-5 relative
    assert int((d0 != d1).sum()) == g["n_density_cr_diff"]
    assert cases.digest_u32(o1.densest()) == g["densest_cr"]
    assert cases.digest_clumps(*o1.clumps()) == g["clumps"]


def test_oracle_morton_order_distinct_keys(oracle_mod):
    """Without repeats the comparator order is the plain lexicographic key order."""
    rng = np.random.default_rng(3)
    k = rng.integers(0, 2**32, size=(5000, 3), dtype=np.uint64).astype(np.uint32)
    k[:, 2] &= 0xF
    order = oracle_mod.morton_order(k)
    np.testing.assert_array_equal(order, np.lexsort((k[:, 0], k[:, 1], k[:, 2])))


def _multi_inputs(tmp_path):
    import shutil

    d = tmp_path / "in"
    d.mkdir()
    shas = []
    for k, c in enumerate(cases.MULTI):
        m = cases.materialise(c, tmp_path / f"c{k}")
        shutil.copy(m["lis"][0], d / f"Snap.{k:04d}.ds.lis")
        shas.append(m["sha256"][0])
        if k == 0:
            shutil.copy(m["param"], d / "para.txt")
    return d, shas


def multi_snapshot_args(d, out):
    return ["-c", "1", "-i", str(d), "-b", "Snap", "-p", "ds", "-f", "0:1", "-o", str(out / "res.txt"), "-t", str(d / "para.txt"),
            "--Combined"]


def test_oracle_cli_two_snapshots(oracle_mod, tmp_path):
    """One run over two snapshots (src/main.cpp:64-83): the second summary line keeps the
    scientific notation of the reference's shared stream; the files equal the reference's."""
    import json
    import subprocess

    g = GOLDEN / "multi_snapshot"
    meta = json.loads((g / "meta.json").read_text())
    d, shas = _multi_inputs(tmp_path)
    assert shas == meta["lis_sha256"]
    out = tmp_path / "out"
    out.mkdir()
    cli = oracle_mod.CLI
    r = subprocess.run([str(cli)] + multi_snapshot_args(d, out), cwd=out, capture_output=True, text=True, check=True)
    assert [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln] == meta["summary"]
    for name in meta["peaks_files"]:
        assert (out / name).read_bytes() == (g / name).read_bytes()
    assert (out / "res_planetesimals.txt").read_bytes() == (g / "planetesimals.txt").read_bytes()


@pytest.mark.parametrize("name", ["w1_20k", "w1_20k_sinks", "w2_250k", "config1_262k"])
def test_speculative_windows_replay_the_sequential_loop(name, case_dir, oracle_mod, tmp_path):
    """The device's speculative acceptance windows (PLAN_ACCEPT_SPECULATE) in the reference's
    own Hill rebinding: every call's candidates replayed in 32-candidate windows decided
    against one state, checked against the exact state before each, and cut at the first
    disagreement, accept exactly what the sequential loop accepts, in fewer steps than the
    default loop's one acceptance per step. The run's files stay the reference's."""
    import re
    import subprocess

    g = golden(name)
    m = case_dir(name)
    out = tmp_path / "out"
    out.mkdir()
    env = dict(os.environ, PLAN_ORACLE_WINDOW_STATS="1")
    r = subprocess.run([str(oracle_mod.CLI)] + cases.cli_args(m, str(out / "res.txt")), cwd=out, env=env, capture_output=True, text=True,
                       check=True)
    assert g["summary"] in r.stdout
    assert (out / "res_planetesimals.txt").read_bytes() == (GOLDEN / name / "planetesimals.txt").read_bytes()
    st = re.search(r"(\d+) calls, (\d+) candidates, (\d+) accepted; (\d+) windows cut short, (\d+) calls disagreeing", r.stderr)
    assert st, r.stderr
    calls, cands, acc, cut, disagree = map(int, st.groups())
    assert calls > 0 and acc > 0
    assert disagree == 0
    steps = {m.group(1).strip(): int(m.group(2)) for m in re.finditer(r"\]   (.+?) steps (\d+),", r.stderr)}
    assert len(steps) == 5, r.stderr
    assert steps["speculative windows"] <= steps["first bound, 32 wide"]
    assert steps["first bound, 1024 wide"] <= steps["first bound, 256 wide"] <= steps["first bound, 32 wide"]


@pytest.mark.parametrize("keep", [(0, 0), (20, 0)], ids=["empty", "20_particles"])
def test_oracle_refuses_what_the_reference_cannot_finish(keep, oracle_mod, tmp_path):
    """An empty snapshot, and one with fewer tree points than the neighbours asked for
    (knn = 32). The reference crashes on the first (a segmentation fault here) and never
    returns from the second: KNN_Search_OpenMP's assert is compiled out and its radius keeps
    doubling (src/tree.hpp:3199-3237). The restatement refuses both with an error and exit
    status 5, as the device path does (status 7 from the C ABI, exit status 5 from its CLI)."""
    import subprocess

    m = cases.materialise(cases.Case("refused", 1, 20000, 5, 32, edit="small:%d:%d" % keep), tmp_path / "in")
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(oracle_mod.CLI)] + cases.cli_args(m, str(out / "res.txt")), cwd=out, capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 5
    assert "Error:" in r.stderr
    if keep == (0, 0):
        with pytest.raises(RuntimeError):
            oracle_mod.Oracle(m["lis"], m["param"], threads=1)
    else:
        o = oracle_mod.Oracle(m["lis"], m["param"], threads=1)
        assert len(o.keys()) < 32
        with pytest.raises(ValueError):
            o.find()


@pytest.mark.parametrize("name,case,extra", cases.VARIANTS, ids=[v[0] for v in cases.VARIANTS])
def test_oracle_cli_variants(name, case, extra, oracle_mod, tmp_path):
    """Sub-sampled member lists (-s), the num_peaks cap, --No_Ghost and the merge parameters
    (src/global.cpp:247-289, src/tree.hpp:4302-4316, 5191-5222): the oracle's files equal
    the reference's."""
    import json
    import subprocess

    g = GOLDEN / name
    meta = json.loads((g / "meta.json").read_text())
    m = cases.materialise(case, tmp_path / "in")
    assert m["sha256"] == meta["lis_sha256"]
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(oracle_mod.CLI)] + cases.cli_args(m, str(out / "res.txt")) + extra, cwd=out, capture_output=True, text=True,
                       check=True)
    assert meta["summary"] in r.stdout
    assert (out / meta["peaks_file"]).read_bytes() == (g / meta["peaks_file"]).read_bytes()
    assert (out / "res_planetesimals.txt").read_bytes() == (g / "planetesimals.txt").read_bytes()
    assert cases.parlist_digests(out) == meta["parlist"]


@pytest.mark.parametrize("name,case,extra", cases.DVS, ids=[v[0] for v in cases.DVS])
def test_oracle_cli_density_vs_scale(name, case, extra, oracle_mod, tmp_path):
    """--Density_Vs_Scale (src/analyses.hpp:196-333, src/main.cpp:71-79): the RMPL file of
    sheared ball counts, then the clump finder on that run's tree (64-point leaves, no
    ghosts, doubled root box), with the basic results in the RMPL file when the flag is
    alone. Every file the reference wrote must come out byte for byte."""
    import json
    import subprocess

    g = GOLDEN / name
    meta = json.loads((g / "meta.json").read_text())
    m = cases.materialise(case, tmp_path / "in")
    assert m["sha256"] == meta["lis_sha256"]
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(oracle_mod.CLI)] + cases.cli_args(m, str(out / "res.txt")) + extra, cwd=out, capture_output=True, text=True,
                       check=True)
    assert [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln] == meta["summary"]
    assert sorted(p.name for p in out.iterdir() if p.is_file()) == meta["files"]
    for f in meta["files"]:
        assert (out / f).read_bytes() == (g / f).read_bytes(), f
    assert cases.parlist_digests(out) == meta["parlist"]


def test_oracle_cli_two_snapshots_density_vs_scale(oracle_mod, tmp_path):
    """Two snapshots with --Density_Vs_Scale alone: one RMPL header, then per snapshot its
    line followed by the basic results, and scientific summary lines throughout."""
    import json
    import subprocess

    g = GOLDEN / "multi_density_vs_scale"
    meta = json.loads((g / "meta.json").read_text())
    d, _ = _multi_inputs(tmp_path)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(oracle_mod.CLI)] + multi_snapshot_args(d, out) + ["--Density_Vs_Scale"], cwd=out, capture_output=True,
                       text=True, check=True)
    assert [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln] == meta["summary"]
    assert sorted(p.name for p in out.iterdir() if p.is_file()) == meta["files"]
    for f in meta["files"]:
        assert (out / f).read_bytes() == (g / f).read_bytes(), f
