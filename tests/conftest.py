"""Shared fixtures: the built library, the oracle, and materialised snapshot cases."""
from __future__ import annotations

import json
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
