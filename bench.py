#!/usr/bin/env python3
"""Throughput of the clump-finding path (BuildTree + FindPlanetesimals) on one GB300.

A step is one snapshot through the whole path: ingest of the 44-byte .lis records, ghosts,
Morton keys, radix sort, sinks, octree, KNN densities, densest neighbours, HOP groups and
the clump stage down to the host catalogue. The workload is the 16,777,216-particle
snapshot (60% uniform, 25% in four Gaussian sheets, 15% in 200 Plummer clumps with a
M^-1.6 mass function, 10% of them unbound), generated in memory from a fixed seed.

  value  particles/s with the records already in device memory when the timer starts;
  e2e    particles/s through the same C-ABI call with page-locked HOST records, so the
         host-to-device copy of the records and the read-back of the catalogue are inside
         the timed region.

Several GPUs run independent replicas (one snapshot per rank, no collective on the data
path); value is the particles of all ranks over the slowest rank's time.

`--impl reference` times the CPU restatement of the same path (oracle/, the reference's
algorithm; the reference program itself is not built where this runs) with all host
cores on the same full snapshot, pass after pass until --steps are done or --ref-budget
seconds have run, and prints the same JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = 2
N_FULL = 1 << 24
SEED = 1
NX = 128
KNN, HOP = 32, 16
WORKLOAD_NAME = ("16.7M-particle snapshot (2^24, float32): 60% uniform, 25% in 4 Gaussian sheets (sigma 2e-3), "
                 "15% in 200 Plummer clumps, dN/dM ~ M^-1.6 on [1e-5, 1e-2] M_tot, 10% unbound")
# bytes per tree point the path must move at least once (pos read, keys, sort, tree, KNN +
# density, HOP), per unit for the density kernel: read the query (12 B), write the
# density (8 B), the K_d neighbour list the reference builds (4 * K_d), the radius (4 B)
DENSITY_BYTES_PER_POINT = 12 + 8 + 4 * KNN + 4
# the clump stage's model: 28 bytes per member and pass (the member index, its position and
# mass read once, its distance written); each rebinding pass counts the members of the
# clumps it ran
REBIND_BYTES_PER_MEMBER = 28
# dram bytes read + written per unit, measured with ncu on smaller snapshots of the same
# mixture (the first rebinding launch of a 1M snapshot; the density launch of a 4M one);
# traffic grows with the units processed, so a full-size launch's traffic is taken as units
# times these figures
REBIND_TRAFFIC_PER_MEMBER = (642_154_240 + 417_524_992) / 662_193    # first launch, 1M snapshot: 1,600 B
DENSITY_TRAFFIC_PER_POINT = (928_974_848 + 483_069_184) / 6_736_104  # 4M snapshot: 209.6 B
# the catalogue of the benchmarked snapshot as the unmodified reference writes it
# (tests/golden/w2_16m, made by tests/golden/make_golden.py)
GOLDEN_FULL = ROOT / "tests" / "golden" / "w2_16m" / "meta.json"
# the reference's catalogues recorded for other sizes of the same mixture (seed 1)
GOLDEN_BY_N = {N_FULL: GOLDEN_FULL, 1 << 27: ROOT / "tests" / "golden" / "w2_134m" / "meta.json"}


def _peaks() -> tuple[float, str]:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        for k in ("hbm_gbs", "hbm_GBs", "copy_gbs"):
            if k in d:
                return float(d[k]), "measured"
        for v in d.values():
            if isinstance(v, dict) and "hbm_gbs" in v:
                return float(v["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.p = None
        self.out = tempfile.NamedTemporaryFile(prefix="clocks", suffix=".csv", delete=False)

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.out.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in Path(self.out.name).read_text().splitlines():
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.out.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def synth_lib() -> C.CDLL:
    """The snapshot generator alone (plan_gb300/lib/libplan_synth.so, no CUDA), so that the CPU
    arm never loads the GPU library."""
    import plan_gb300 as pg  # structure layouts only; the GPU library is not loaded

    path = ROOT / "plan_gb300" / "lib" / "libplan_synth.so"
    if not path.exists():
        from plan_gb300 import build as b

        b.build()
    L = C.CDLL(str(path))
    L.plan_synth_default_spec.restype = C.c_int32
    L.plan_synth_default_spec.argtypes = [C.c_int32, C.c_uint64, C.c_uint64, C.POINTER(pg.SynthSpec)]
    L.plan_synth_records.restype = C.c_int32
    L.plan_synth_records.argtypes = [C.POINTER(pg.SynthSpec), C.c_void_p, C.POINTER(pg.SynthInfo)]
    L.plan_synth_four_pi_G_for_mean.restype = C.c_double
    L.plan_synth_four_pi_G_for_mean.argtypes = [C.POINTER(pg.SynthSpec), C.c_int32, C.c_int32]
    return L


def make_records(n: int, seed: int, pinned: bool):
    """The workload's .lis records in (page-locked) host memory; returns (tensor, 4piG)."""
    import torch

    import plan_gb300 as pg

    L = synth_lib()
    spec = pg.SynthSpec()
    rc = L.plan_synth_default_spec(WORKLOAD, n, seed, C.byref(spec))
    assert rc == 0
    spec.nx = NX
    fourpig = L.plan_synth_four_pi_G_for_mean(C.byref(spec), NX, NX)
    spec.G = fourpig / (4 * np.pi)
    rec = torch.empty(n * 44, dtype=torch.uint8, pin_memory=pinned)
    info = pg.SynthInfo()
    rc = L.plan_synth_records(C.byref(spec), C.c_void_p(rec.data_ptr()), C.byref(info))
    assert rc == 0
    return rec, fourpig


def lis_view(pg, ptr: int, n: int):
    v = pg.LisView()
    lim = [-0.1, 0.1] * 6
    for i, x in enumerate(lim):
        v.coor_lim[i] = float(np.float32(x))
    v.ntypes = 1
    v.type_info[0] = 1.0
    v.time = 0.0
    v.dt = 0.0
    v.nblocks = 1
    arr = (C.c_void_p * 1)(ptr)
    cnt = (C.c_uint64 * 1)(n)
    v.records = C.cast(arr, C.POINTER(C.c_void_p))
    v.counts = C.cast(cnt, C.POINTER(C.c_uint64))
    v._keep = (arr, cnt)
    return v


def write_params(path: Path, fourpig: float, threads: int) -> None:
    path.write_text(f"Nx1 = {NX}\nNx2 = {NX}\nNx3 = {NX}\nZ = 0.02\nfour_pi_G_par = {fourpig!r}\nknn = {KNN}\nhop = {HOP}\n"
                    f"num_threads = {threads}\n")


def write_lis(path: Path, rec: np.ndarray, n: int) -> None:
    import struct

    hdr = struct.pack("<12fi1fffq", *([-0.1, 0.1] * 6), 1, 1.0, 0.0, 0.0, n)
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(memoryview(rec))


# ---------------------------------------------------------------- CPU legs
def cpu_sample(n: int, seed: int, threads: int, reps: int = 1, warmup: int = 0) -> dict:
    """The oracle restatement on a sample snapshot of the same workload, generated once:
    `warmup` untimed passes, then the seconds of `reps` timed ones (read to catalogue)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        rec, fourpig = make_records(n, seed, pinned=False)
        write_lis(d / "Snap.0000.ds.lis", rec.numpy(), n)
        write_params(d / "para.txt", fourpig, threads)
        times = []
        for k in range(warmup + reps):
            t0 = time.perf_counter()
            o = oracle.Oracle(str(d / "Snap.0000.ds.lis"), str(d / "para.txt"), threads=threads, pow_mode=0)
            o.find()
            if k >= warmup:
                times.append(time.perf_counter() - t0)
            o.close()
    return {"n": n, "seconds": times}


def run_reference(args) -> None:
    """The reference arm: the CPU implementation of the path on the host cores, on the GPU arm's
    own snapshot (same size, seed and parameters). The snapshot is generated and written once,
    untimed; every timed pass reads it and runs the whole path to the catalogue. The CPU code
    keeps no state between passes, so no warm-up pass is run; passes continue until `steps` are
    done or `--ref-budget` seconds have been spent (at least one pass), and the line reports
    how many ran."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from plan_gb300 import build as b

    b.build_oracle()
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    threads = os.cpu_count() or 1
    n = args.n
    times = []
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        rec, fourpig = make_records(n, SEED, pinned=False)
        write_lis(d / "Snap.0000.ds.lis", rec.numpy(), n)
        write_params(d / "para.txt", fourpig, threads)
        del rec
        while len(times) < args.steps and (not times or sum(times) + times[-1] <= args.ref_budget):
            t0 = time.perf_counter()
            o = oracle.Oracle(str(d / "Snap.0000.ds.lis"), str(d / "para.txt"), threads=threads, pow_mode=0)
            o.find()
            times.append(time.perf_counter() - t0)
            o.close()
            print(f"bench --impl reference: pass {len(times)} {times[-1]:.1f} s", file=sys.stderr, flush=True)
    value = n * len(times) / sum(times)
    sample = (f"the full {n}-particle snapshot of the GPU arm (seed {SEED}), read and processed to the catalogue in each of "
              f"{len(times)} passes ({args.steps} requested; passes stop after {args.ref_budget:.0f} s)")
    line = {"impl": "reference", "metric": "particles/s", "value": value, "unit": "particles/s", "n_gpus": args.gpus,
            "steps": len(times), "requested_steps": args.steps, "warmup": 0, "requested_warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD_NAME, "n_particles": n, "seed": SEED, "knn": KNN, "hop": HOP, "nx": NX},
            "cpu_baseline": {"value": value, "unit": "particles/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "per_step_s": times}
    print(json.dumps(line), flush=True)


def check_parity(cat, n: int, seed: int):
    """The catalogue against the reference's for the benchmarked snapshot (and the 2^27 one):
    the summary line and the SHA-256 of peaks_at_*.txt must be equal. None for snapshots
    without a recorded one."""
    import hashlib

    gf = GOLDEN_BY_N.get(n)
    if seed != SEED or gf is None or not gf.exists():
        return None
    g = json.loads(gf.read_text())
    with tempfile.TemporaryDirectory() as d:
        cat.write_peaks(str(Path(d) / "res.txt"))
        got = hashlib.sha256((Path(d) / g["peaks_file"]).read_bytes()).hexdigest()
    return {"identical": got == g["peaks_sha256"] and cat.summary().strip() == g["summary"], "peaks_sha256": got,
            "against": "catalogue of the unmodified reference on the same snapshot"}


# ---------------------------------------------------------------- replicas
def reduce_max(x: float, dist, device: str = "cpu") -> float:
    """The slowest replica's time (max over ranks); x unchanged without a process group."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank: int) -> int:
    """Each rank finds clumps in its own snapshot (replicas; nothing is exchanged)."""
    return SEED + rank


def aggregate(world: int, n: int, steps: int, total_ms: float) -> float:
    """Whole-job particles/s: every rank's particles over the slowest rank's time."""
    return world * n * steps / (total_ms / 1e3)


# ---------------------------------------------------------------- GPU arm
def run_gpu(args) -> None:
    import torch

    import plan_gb300 as pg

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (this path has no CPU fallback)")
    torch.cuda.set_device(local)
    n = args.n
    rec_h, fourpig = make_records(n, replica_seed(rank), pinned=True)
    rec_d = rec_h.to(f"cuda:{local}")
    with tempfile.TemporaryDirectory() as d:
        par = Path(d) / "para.txt"
        write_params(par, fourpig, os.cpu_count() or 1)
        p = pg.params(str(par))
    f = pg.Finder(local)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    v_dev = lis_view(pg, rec_d.data_ptr(), n)
    v_host = lis_view(pg, rec_h.data_ptr(), n)
    L = pg.lib()

    last = {}

    def step(view):
        h = C.c_void_p()
        rc = L.plan_find_clumps(f._h, C.byref(view), C.byref(p), 1, C.c_void_p(sp), C.byref(h))
        if rc:
            raise pg.PlanError(rc, f.error())
        cat = pg.Catalogue(h)
        nc = len(cat)
        if "cat" in last:
            last["cat"].close()
        last["cat"] = cat  # the last catalogue is checked after the timed region
        return nc

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def timed(view, steps):
        barrier()
        l0 = f.kernel_launches()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        per, dens_ms, densest_ms = [], [], []
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            for i in range(steps):
                step(view)
                ev[i + 1].record(stream)
                st = f.stage_times()
                dens_ms.append(st[20])
                densest_ms.append(st[21])
        barrier()
        per = [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]
        total = reduce_max(ev[0].elapsed_time(ev[steps]), dist, f"cuda:{local}")
        return total, per, f.kernel_launches() - l0, dens_ms, densest_ms

    for w in range(args.warmup):
        t0 = time.perf_counter()
        step(v_dev)
        print(f"bench: warm-up step {w + 1}/{args.warmup} {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
    clocks = ClockSampler(local)
    clocks.start()
    total, per, launches, dens_ms, densest_ms = timed(v_dev, args.steps)
    clk = clocks.stop()
    stage = f.stage_times()
    cnt = f.counters()
    nclumps = int(cnt[7])
    tree_points = int(cnt[2])
    rb_ms, rb_members = stage[19], int(cnt[24])  # the rebinding launches of the last timed step
    parity = check_parity(last["cat"], n, replica_seed(rank))
    # end to end through the same call with host records (buffers and arenas are already sized
    # by the warm-up, so no separate warm-up of this leg)
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    total_e2e, per_e2e, _, _, _ = timed(v_host, e2e_steps)
    last["cat"].close()
    h2d = int(f.counters()[20])
    d2h = int(f.counters()[21])
    value = aggregate(world, n, args.steps, total)
    e2e_value = aggregate(world, n, e2e_steps, total_e2e)
    peak, peak_kind = _peaks()
    # the dominant kernel: the rebinding loop (one launch per pass; its time summed over the
    # launches of a snapshot, CUDA events on the stream it runs on)
    rb_bytes = REBIND_BYTES_PER_MEMBER * rb_members
    rb_achieved = rb_bytes / (rb_ms / 1e3) / 1e9 if rb_ms > 0 else None
    roof = {"kernel": "k_rebind_loop (Hill-sphere rebinding, every clump's calls on the device; all launches of one snapshot)",
            "bound": "hbm", "achieved": rb_achieved, "peak": peak, "unit": "GB/s", "frac": rb_achieved / peak if rb_achieved else None,
            "peak_kind": f"{peak_kind} HBM copy bandwidth", "traffic": REBIND_TRAFFIC_PER_MEMBER * rb_members,
            "traffic_note": "dram bytes read+written per member from one ncu capture (first launch, 1M snapshot), times the members of the step's passes",
            "bytes_per_unit": REBIND_BYTES_PER_MEMBER, "units": rb_members, "kernel_ms": rb_ms,
            "limited_by": "dependent FP64 update chains and exact ordered member sums, not bandwidth"}
    dens_avg = float(np.mean(dens_ms))
    achieved = DENSITY_BYTES_PER_POINT * tree_points / (dens_avg / 1e3) / 1e9 if dens_avg > 0 else None
    roof_dens = {"kernel": "k_density_f (KNN + median density, FP32-filtered exact traversal)", "bound": "hbm", "achieved": achieved,
                 "peak": peak, "unit": "GB/s", "frac": achieved / peak if achieved else None, "peak_kind": f"{peak_kind} HBM copy bandwidth",
                 "traffic": DENSITY_TRAFFIC_PER_POINT * tree_points, "bytes_per_unit": DENSITY_BYTES_PER_POINT,
                 "units_per_launch": tree_points, "launch_ms": dens_avg}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        r = cpu_sample(args.sample_n, SEED, threads)
        cv = args.sample_n / r["seconds"][0]
        cpu = {"value": cv, "unit": "particles/s", "cores": threads, "kind": "port",
               "sample": f"one {args.sample_n}-particle snapshot of the same workload (clump count scaled) through the oracle"}
    if rank == 0:
        line = {"metric": "particles/s", "value": value, "unit": "particles/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD_NAME, "n_particles": n, "seed": SEED, "knn": KNN, "hop": HOP, "nx": NX,
                           "tree_points": tree_points, "clumps_found": nclumps, "parallelism": f"replicas{world}",
                           "l2": "inputs larger than L2 (records 738 MB, tree arrays several GB), no flush"},
                "e2e": {"value": e2e_value, "unit": "particles/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "ms_per_step": total_e2e / e2e_steps, "steps": e2e_steps},
                "parity": parity,
                "roofline": roof, "roofline_density": roof_dens, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
                "snapshots_per_s": world * args.steps / (total / 1e3),
                "latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99))},
                "stage_ms": {"ingest_ghosts_keys": stage[0], "sort": stage[1], "sinks_tree": stage[2], "tree_tail": stage[3],
                             "density": stage[4], "densest": stage[5], "hop": stage[6], "clump_stage": stage[7],
                             "catalogue": stage[8], "density_kernel": stage[20], "densest_kernel": stage[21],
                             "rebinding": stage[12], "rebinding_kernel": stage[19]},
                "rebinding": {"passes": int(cnt[12]), "launches": int(stage[14]), "reruns": int(cnt[14])}}
        print(json.dumps(line), flush=True)
    f.close()
    if dist is not None:
        dist.destroy_process_group()


# ---------------------------------------------------------------- serving (opt-in: --serve K)
def serve_requests(k: int, max_log2: int, seed: int):
    """K snapshots of the workload's mixture, sizes log-uniform in [2^16, 2^max_log2], clump
    count proportional to N (the generator scales it), each with its own seed."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(2.0 ** 16), np.log(2.0 ** max_log2), k)).astype(np.int64)
    return [(int(n), 1000 + i) for i, n in enumerate(sizes)]


def latency_stats(lat_ms) -> dict:
    return {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)), "n": len(lat_ms)}


class _ViewOnly:
    """A snapshot given by its .lis view alone (records owned by the caller)."""

    def __init__(self, view):
        self.view = view


def run_serve(args) -> None:
    """Poisson arrivals of mixed-size snapshots through the serving loop (plan_submit /
    plan_poll), and the same requests one by one through the plain path on one context.
    Every served catalogue must equal the plain one; prints one JSON line."""
    import torch

    import plan_gb300 as pg

    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (this path has no CPU fallback)")
    reqs = []
    with tempfile.TemporaryDirectory() as d:
        for n, sd in serve_requests(args.serve, args.serve_max_log2, SEED):
            rec, fourpig = make_records(n, sd, pinned=True)
            par = Path(d) / f"para{sd}.txt"
            write_params(par, fourpig, os.cpu_count() or 1)
            reqs.append({"n": n, "rec": rec, "view": lis_view(pg, rec.data_ptr(), n), "param": pg.params(str(par))})
    rng = np.random.default_rng(SEED + 7)
    gaps = rng.exponential(1.0 / args.serve_rate, len(reqs))
    # the plain path, one snapshot after another on one context (also the warm-up)
    f = pg.Finder(0)
    plain_lat, plain_sum = [], []
    t0 = time.perf_counter()
    for r in reqs:
        t = time.perf_counter()
        p = pg.Params.from_buffer_copy(r["param"])
        cat = f.find_clumps(_ViewOnly(r["view"]), p)
        plain_lat.append(1e3 * (time.perf_counter() - t))
        plain_sum.append(cat.summary())
        cat.close()
    plain_s = time.perf_counter() - t0
    f.close()
    # served: arrivals on their Poisson schedule from a submitting thread
    srv = pg.Server(0, args.serve_workers, 0)
    ids = [None] * len(reqs)

    def submitter():
        for i, r in enumerate(reqs):
            time.sleep(gaps[i])
            ids[i] = srv.submit(_ViewOnly(r["view"]), pg.Params.from_buffer_copy(r["param"]))

    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    served_lat, same = [], True
    deadline = time.monotonic() + 300.0 + 20.0 * plain_s  # a request that never finishes ends the run
    for i in range(len(reqs)):
        got = srv.poll(ids[i])
        while got is None and time.monotonic() < deadline:
            time.sleep(0.005)
            got = srv.poll(ids[i])
        if got is None:
            raise SystemExit(f"bench.py --serve: request {i} not done by the deadline")
        cat, lat = got
        served_lat.append(lat)
        same = same and cat.summary() == plain_sum[i]
        cat.close()
    served_s = time.perf_counter() - t0
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    n_tot = sum(r["n"] for r in reqs)
    line = {"metric": "snapshots/s served", "value": len(reqs) / served_s, "unit": "snapshots/s", "n_gpus": 1,
            "higher_is_better": True, "data": "synthetic", "dtype": "f64",
            "config": {"workload": f"{len(reqs)} requests of the workload's mixture, N log-uniform in [2^16, 2^{args.serve_max_log2}], "
                                   f"Poisson arrivals at {args.serve_rate}/s", "workers": args.serve_workers, "particles": n_tot},
            "served": {"snapshots_per_s": len(reqs) / served_s, "particles_per_s": n_tot / served_s,
                       "latency_ms": latency_stats(served_lat), "peak_held_bytes": st["peak_held_bytes"], "releases": st["releases"],
                       "busy_ms": st["busy_ms"], "two_or_more_running_ms": st["overlap_ms"]},
            "plain": {"snapshots_per_s": len(reqs) / plain_s, "particles_per_s": n_tot / plain_s, "latency_ms": latency_stats(plain_lat)},
            "identical_catalogues": same, "clocks": clk}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- boundness (opt-in: --boundness K)
def plummer_groups(k: int, n_lo: int, n_hi: int, seed: int):
    """K Plummer groups (scale 1e-3, equal masses, float32), sizes log-uniform in [n_lo, n_hi]."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), k)).astype(np.int64)
    pos, vel = [], []
    for i, n in enumerate(sizes):
        u = rng.uniform(1e-6, 0.99, n)
        r = 1e-3 / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        c = rng.uniform(-0.09, 0.09, 3)
        pos.append((c + r[:, None] * d).astype(np.float32))
        vel.append(rng.normal(scale=1e-3, size=(n, 3)).astype(np.float32))
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    return np.concatenate(pos), np.concatenate(vel), np.full(int(off[-1]), 4.0106053e-08, np.float32), off


def boundness_error(pos, vel, mass, off, ek, ep, p, max_n: int = 3000, max_groups: int = 64) -> dict:
    """The largest relative error of the pass's energies against FP64 direct sums, over up to
    max_groups groups spread over the sizes up to max_n particles: potential -G sum m_i m_j / r
    and kinetic 1/2 sum m |v_c - s (x_c - x) - v|^2, both with all inputs widened to FP64."""
    sizes = np.diff(off.astype(np.int64))
    worst_p = worst_k = 0.0
    checked = largest = 0
    small = np.flatnonzero((sizes >= 2) & (sizes <= max_n))
    small = small[np.argsort(sizes[small])]
    pick = small[np.unique(np.linspace(0, len(small) - 1, min(max_groups, len(small))).astype(np.int64))] if len(small) else small
    for g in pick:  # spread over the sizes up to max_n
        b, e = int(off[g]), int(off[g + 1])
        if e - b < 2:
            continue
        x, v, m = pos[b:e].astype(np.float64), vel[b:e].astype(np.float64), mass[b:e].astype(np.float64)
        d = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
        iu = np.triu_indices(e - b, 1)
        want_p = -p.grav_constant * float((m[:, None] * m[None, :])[iu][d[iu] > 0].dot(1.0 / d[iu][d[iu] > 0]))
        M = m.sum()
        xc, vc = (m[:, None] * x).sum(0) / M, (m[:, None] * v).sum(0) / M
        dv = vc[None, :] - v
        dv[:, 1] -= p.q * p.Omega * (xc[0] - x[:, 0])
        want_k = 0.5 * float((m * (dv ** 2).sum(1)).sum())
        if want_p != 0:
            worst_p = max(worst_p, abs(ep[g] - want_p) / abs(want_p))
        if want_k != 0:
            worst_k = max(worst_k, abs(ek[g] - want_k) / abs(want_k))
        checked += 1
        largest = max(largest, e - b)
    return {"groups_checked": checked, "largest_checked_n": largest,
            "max_rel_potential": worst_p, "max_rel_kinetic": worst_k, "tolerance": 1e-6}


def run_boundness(args) -> None:
    """All groups' energies through plan_group_energies; pair interactions per second."""
    import torch

    import plan_gb300 as pg

    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (this path has no CPU fallback)")
    pos, vel, mass, off = plummer_groups(args.boundness, 32, args.boundness_max, SEED)
    sizes = np.diff(off.astype(np.int64))
    pairs = int((sizes * (sizes - 1) // 2).sum())
    p = pg.params()
    pg.lib().plan_params_derive(C.byref(p))
    f = pg.Finder(0)
    for _ in range(args.warmup):
        f.group_energies(pos, vel, mass, off, p)
    clocks = ClockSampler(0)
    clocks.start()
    t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ek, ep, zeros = f.group_energies(pos, vel, mass, off, p)
        t.append(time.perf_counter() - t0)
    clk = clocks.stop()
    f.close()
    sec = sum(t) / len(t)
    err = boundness_error(pos, vel, mass, off, ek, ep, p)
    line = {"metric": "pair interactions/s (batched boundness)", "value": pairs / sec, "unit": "pairs/s", "n_gpus": 1,
            "higher_is_better": True, "data": "synthetic", "dtype": "f32 pairs, f64 sums", "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sec,
            "config": {"workload": f"{args.boundness} Plummer groups, sizes log-uniform in [32, {args.boundness_max}]",
                       "particles": int(off[-1]), "pairs": pairs, "bound_groups": int((ek + ep < 0).sum()), "coincident_pairs": zeros},
            "e2e": {"value": pairs / sec, "unit": "pairs/s", "h2d_bytes_per_step": int(off[-1]) * 28, "d2h_bytes_per_step": 16 * len(sizes)},
            "value_note": "through plan_group_energies with host arrays: the H2D copy of the particles is inside every step",
            "error_vs_fp64": err, "clocks": clk}
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--n", type=int, default=N_FULL, help="particles per snapshot (default: the full workload)")
    ap.add_argument("--sample-n", type=int, default=1 << 22, help="particles of the CPU sample snapshot (GPU arm's cpu_baseline)")
    ap.add_argument("--ref-budget", type=float, default=480.0, help="reference arm: seconds of timed full-size passes (at least one)")
    ap.add_argument("--e2e-steps", type=int, default=3, help="steps of the end-to-end leg (at most --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve", type=int, default=0, help="instead: K requests through the serving loop (plan_submit/plan_poll)")
    ap.add_argument("--serve-workers", type=int, default=3)
    ap.add_argument("--serve-rate", type=float, default=4.0, help="Poisson arrivals per second")
    ap.add_argument("--serve-max-log2", type=int, default=22, help="largest request 2^k particles")
    ap.add_argument("--boundness", type=int, default=0, help="instead: K groups through plan_group_energies")
    ap.add_argument("--boundness-max", type=int, default=200000, help="largest group")
    args = ap.parse_args()
    if args.boundness and args.impl == "gpu":
        run_boundness(args)
    elif args.serve and args.impl == "gpu":
        run_serve(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
