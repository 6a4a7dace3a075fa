"""The spline-density path on the GPU (needs a GB300).

Snapshots with fewer than four particles per horizontal grid cell take the reference's
QseudoQuadraticSplinesKernel instead of the median-sphere density, and drop small or
low-peak groups right after HOP (src/tree.hpp:3583-3610, 3834-3836). Every stage and both
output files must equal the reference's golden outputs, as for the median-kernel cases.
"""
from __future__ import annotations

import pytest

import cases
from conftest import run_isolated
from test_gpu_parity import check_cli_drop_in, check_stages_and_catalogue

pytestmark = pytest.mark.gpu

SPLINE = [c.name for c in cases.SPLINE]


@pytest.mark.parametrize("name", SPLINE)
def test_spline_stages_and_catalogue(name, request, built, case_dir, tmp_path):
    if run_isolated(request):
        return
    f = built.Finder(0)
    try:
        check_stages_and_catalogue(name, built, f, case_dir, tmp_path)
    finally:
        f.close()


@pytest.mark.parametrize("name", SPLINE[:1])
def test_spline_cli_drop_in(name, built, case_dir, tmp_path):
    check_cli_drop_in(name, built, case_dir, tmp_path)
