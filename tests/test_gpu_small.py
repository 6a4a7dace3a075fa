"""Small and degenerate snapshots through the GPU path (needs a GB300).

Each case runs the plan_gpu binary with the reference's command line in a child process:
- a few hundred to a thousand particles (spline and median kernels, one to four clumps): the
  reference's files, byte for byte;
- an empty snapshot, and one with fewer tree points than the neighbours asked for: refused
  with exit status 5 and an error message. The reference crashes on the first and never
  returns from the second (its KNN radius keeps doubling, src/tree.hpp:3199-3237).
"""
from __future__ import annotations

import subprocess

import pytest

import cases
from conftest import ROOT
from test_gpu_parity import check_cli_drop_in

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", [c.name for c in cases.SMALL])
def test_small_snapshot_cli_drop_in(name, built, case_dir, tmp_path):
    check_cli_drop_in(name, built, case_dir, tmp_path)


@pytest.mark.parametrize("keep,message", [((0, 0), "no particles"), ((20, 0), "knn and hop")], ids=["empty", "20_particles"])
def test_snapshot_the_reference_cannot_finish_is_refused(keep, message, built, tmp_path):
    m = cases.materialise(cases.Case("refused", 1, 20000, 5, 32, edit="small:%d:%d" % keep), tmp_path / "in")
    out = tmp_path / "out"
    out.mkdir()
    cli = ROOT / "plan_gb300" / "lib" / "plan_gpu"
    r = subprocess.run([str(cli)] + cases.cli_args(m, str(out / "res.txt")), cwd=out, capture_output=True, text=True, timeout=300)
    assert r.returncode == 5
    assert message in r.stderr
