"""Command-line and parameter variants through the drop-in binary on the GPU (needs a GB300).

Each variant of tests/cases.py (sub-sampled member lists with -s, the num_peaks cap,
--No_Ghost, the merge parameters, and -x/-y/-z user boxes) runs the plan_gpu binary with the
reference's command line; its summary line, catalogue, basic-results file and every
--Save_Clumps member list must equal the reference's own files.
"""
from __future__ import annotations

import json
import subprocess

import pytest

import cases
from conftest import GOLDEN, ROOT

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
