"""Several GPUs run independent replicas of the path (one snapshot per rank, no data
exchange): the host-side rules of bench.py checked with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = 100.0 + 50.0 * rank  # rank 1 is the slower replica
    slowest = bench.reduce_max(mine, dist)
    out.put((rank, bench.replica_seed(rank), slowest, bench.aggregate(world, 1000, 4, slowest)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    seeds = [g[1] for g in got]
    assert len(set(seeds)) == world  # distinct snapshots per replica
    for _, _, slowest, value in got:
        assert slowest == 150.0  # every rank sees the slowest replica's time
        assert value == pytest.approx(2 * 1000 * 4 / 0.150)


def test_single_process_has_no_collective():
    import bench

    assert bench.reduce_max(7.5, None) == 7.5
    assert bench.aggregate(1, 10, 2, 1000.0) == 20.0


def test_serving_requests_and_latency_stats():
    """The serving leg's request stream: sizes log-uniform in [2^16, 2^k], one seed each,
    the same stream every run; p50/p99 from the latencies."""
    import bench

    a = bench.serve_requests(64, 20, 1)
    assert a == bench.serve_requests(64, 20, 1)
    sizes = [n for n, _ in a]
    assert min(sizes) >= 1 << 16 and max(sizes) <= 1 << 20
    assert len({sd for _, sd in a}) == 64
    st = bench.latency_stats([1.0, 2.0, 3.0, 4.0])
    assert st["p50"] == 2.5 and st["n"] == 4 and 3.9 < st["p99"] <= 4.0


def test_boundness_groups():
    """The boundness leg's groups: sizes log-uniform in range, offsets consistent, float32."""
    import bench

    pos, vel, mass, off = bench.plummer_groups(20, 32, 2000, 1)
    sizes = np.diff(off.astype(np.int64))
    assert len(sizes) == 20 and sizes.min() >= 32 and sizes.max() <= 2000
    assert pos.shape == (int(off[-1]), 3) and vel.shape == pos.shape and mass.shape == (int(off[-1]),)
    assert pos.dtype == np.float32 and mass.dtype == np.float32


def test_cpu_sample_runs_warmups_then_times(built):
    """The CPU legs generate the sample snapshot once, run the warm-up passes untimed and
    return one time per timed pass (read to catalogue through the oracle)."""
    import bench

    r = bench.cpu_sample(20000, 3, 2, reps=2, warmup=1)
    assert r["n"] == 20000 and len(r["seconds"]) == 2 and min(r["seconds"]) > 0
