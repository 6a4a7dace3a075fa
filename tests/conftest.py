"""Shared fixtures: the built library, the oracle, and materialised snapshot cases."""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "tests", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built():
    """Build the library (and the oracle restatement) once per session."""
    from plan_gb300 import build as b

    b.build(verbose=False)
    b.build_oracle()
    import plan_gb300

    plan_gb300.lib()
    return plan_gb300


@pytest.fixture(scope="session")
def case_dir(tmp_path_factory, built):
    """Materialise a case once per session: case_dir(name) -> dict from cases.materialise."""
    import cases

    made = {}

    def get(name: str) -> dict:
        if name not in made:
            made[name] = cases.materialise(cases.BY_NAME[name], tmp_path_factory.mktemp(name))
        return made[name]

    return get


def golden(name: str) -> dict:
    return json.loads((GOLDEN / name / "meta.json").read_text())


def run_isolated(request) -> bool:
    """Run the calling test again in a child pytest process, so that a device fault in it
    ends only that process and not the tests collected after it. Returns True in the parent,
    after asserting that the child passed (the child runs with --runxfail, so an expected
    failure fails it); returns False in the child, which then runs the test body."""
    if os.environ.get("PLAN_TEST_CHILD") == "1":
        return False
    path = getattr(request.node, "path", None) or request.node.fspath  # absolute, whatever the parent's rootdir
    node = f"{path}::{request.node.name}"
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "--runxfail", "-p", "no:cacheprovider", node],
                       cwd=ROOT, env=dict(os.environ, PLAN_TEST_CHILD="1"), capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, (r.stdout[-4000:] + r.stderr[-2000:])
    return True
