"""Workloads beyond one snapshot at a time, on the GPU (needs a GB300).

The serving loop (plan_submit / plan_poll): snapshots of different sizes are submitted
together from several threads and run concurrently on a pool of contexts; each catalogue
must equal the reference's golden output for that snapshot, i.e. be the same in the mix as
alone. A tight budget forces requests to wait for memory and idle workers to give their
buffers back; the results do not change.

Batched boundness (plan_group_energies): kinetic and pairwise potential energies of groups
from two to several thousand particles in one pass, against an FP64 direct sum (potential to
1e-6 relative, the stated tolerance).
"""
from __future__ import annotations

import threading
import time

import pytest

from conftest import GOLDEN, golden, run_isolated

pytestmark = pytest.mark.gpu

MIX = ["w1_20k", "w1_20k_sinks", "w1_20k_border", "w1_24k_split2", "w2_250k", "w1_20k_spline80"]


def _check(pg, name, cat, tmp_path):
    g = golden(name)
    assert cat.summary().strip() == g["summary"], name
    d = tmp_path / name
    d.mkdir(parents=True)
    cat.write_peaks(str(d / "res.txt"))
    assert (d / g["peaks_file"]).read_bytes() == (GOLDEN / name / g["peaks_file"]).read_bytes(), name


def _poll_until(srv, rid, seconds):
    """Poll without blocking inside the library, so a request that never finishes fails the
    test instead of holding it."""
    end = time.monotonic() + seconds
    while time.monotonic() < end:
        got = srv.poll(rid)
        if got is not None:
            return got
        time.sleep(0.01)
    return None


@pytest.mark.parametrize("workers,budget_of_largest", [(3, 0.0), (2, 1.2)])
def test_mixed_requests_match_alone(workers, budget_of_largest, request, built, case_dir, tmp_path):
    if run_isolated(request):
        return
    pg = built
    cases_m = {n: case_dir(n) for n in MIX}
    snaps = {n: pg.Snapshot(m["lis"]) for n, m in cases_m.items()}
    params = {n: pg.params(m["param"]) for n, m in cases_m.items()}
    budget = 0
    if budget_of_largest:
        largest = max(pg.lib().plan_footprint_bytes(s.n, None) for s in snaps.values())
        budget = int(largest * budget_of_largest)
    srv = pg.Server(0, workers, budget)
    try:
        ids = {}
        lock = threading.Lock()

        def submit(names):
            for n in names:
                rid = srv.submit(snaps[n], params[n])
                with lock:
                    ids[n] = rid

        ts = [threading.Thread(target=submit, args=(MIX[k::2],)) for k in range(2)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        assert len(ids) == len(MIX)
        for n in MIX:
            got = _poll_until(srv, ids[n], 600.0)
            assert got is not None, f"request {n} not done after 600 s"
            cat, lat = got
            assert lat > 0
            _check(pg, n, cat, tmp_path / f"w{workers}")
            cat.close()
        st = srv.stats()
        if budget:
            assert st["peak_held_bytes"] <= budget
    finally:
        srv.close()
        for s in snaps.values():
            s.close()


def test_oversized_request_is_refused(request, built, case_dir):
    if run_isolated(request):
        return
    pg = built
    m = case_dir("w1_20k")
    snap = pg.Snapshot(m["lis"])
    srv = pg.Server(0, 1, 1 << 20)  # 1 MiB: nothing fits
    try:
        with pytest.raises(pg.PlanError) as e:
            srv.submit(snap, pg.params(m["param"]))
        assert e.value.status == 6
    finally:
        srv.close()
        snap.close()


def test_group_energies_against_fp64(request, built):
    if run_isolated(request):
        return
    import numpy as np

    from test_energy_host import fp64_potential_sum, plummer_group

    pg = built
    sizes = [2, 31, 128, 129, 500, 2000, 3000, 64]
    parts = [plummer_group(n, 100 + n) for n in sizes]
    pos = np.concatenate([q[0] for q in parts])
    vel = np.concatenate([q[1] for q in parts])
    mass = np.concatenate([q[2] for q in parts])
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    # an empty group after the first one: no energy, and the others unchanged
    off_e = np.concatenate([off[:2], off[1:2], off[2:]]).astype(np.uint64)
    p = pg.params()
    pg.lib().plan_params_derive(__import__("ctypes").byref(p))
    f = pg.Finder(0)
    try:
        ek, ep, zeros = f.group_energies(pos, vel, mass, off, p)
        ek_e, ep_e, zeros_e = f.group_energies(pos, vel, mass, off_e, p)
    finally:
        f.close()
    assert zeros == 0 and zeros_e == 0
    assert ek_e[1] == 0.0 and ep_e[1] == 0.0
    assert np.allclose(np.delete(ek_e, 1), ek, rtol=1e-12, atol=0) and np.allclose(np.delete(ep_e, 1), ep, rtol=1e-9, atol=0)
    G, s = p.grav_constant, p.q * p.Omega
    for g, (gp, gv, gm) in enumerate(parts):
        want_p = -G * fp64_potential_sum(gp, gm)
        assert abs(ep[g] - want_p) <= 1e-6 * abs(want_p), g
        x, v, m = gp.astype(np.float64), gv.astype(np.float64), gm.astype(np.float64)
        M = m.sum()
        xc, vc = (m[:, None] * x).sum(0) / M, (m[:, None] * v).sum(0) / M
        dv = vc[None, :] - v
        dv[:, 1] -= s * (xc[0] - x[:, 0])
        want_k = 0.5 * float((m * (dv ** 2).sum(1)).sum())
        assert abs(ek[g] - want_k) <= 1e-12 * abs(want_k), g
