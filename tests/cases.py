"""Snapshot cases shared by the parity tests and the golden-fixture script.

Every case is generated deterministically: the workload generator of the library
(plan_synth_*) writes the base snapshot and a few integer / float32 edits made here turn it
into the edge cases the clump finder has to handle (sinks from duplicated positions, clumps
straddling the periodic faces, a sheared time, a multi-file snapshot, a clump-free field).
The same bytes come out on x86-64 and aarch64; the golden fixtures pin each case by the
SHA-256 of its .lis files.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import struct
import sys
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

REC = np.dtype([("pos", "<f4", 3), ("vel", "<f4", 3), ("density", "<f4"), ("type", "<i4"), ("id_in_run", "<i8"),
                ("cpu_id", "<i4")])
assert REC.itemsize == 44


@dataclass
class Case:
    name: str
    workload: int
    n: int
    seed: int
    nx: int
    edit: str = ""          # "", "sinks", "border", "split2", "uniform", "small:<nb>:<nc>"
    time: float = 0.0
    knn: int = 32
    hop: int = 16
    extra: dict = field(default_factory=dict)


# small cases: the oracle and the reference finish each in well under a second
CASES = [
    Case("w1_20k", 1, 20000, 5, 32),
    Case("w1_20k_sinks", 1, 20000, 7, 32, edit="sinks"),
    Case("w1_20k_border", 1, 20000, 9, 32, edit="border"),
    Case("w1_20k_sheared", 1, 20000, 11, 32, edit="border", time=0.37),
    Case("w1_24k_split2", 1, 24000, 13, 32, edit="split2"),
    Case("w1_20k_uniform", 1, 20000, 15, 32, edit="uniform"),
    Case("w1_20k_knn48", 1, 20000, 17, 32, knn=48, hop=24),
    Case("w2_250k", 2, 250000, 3, 64),
    Case("config1_262k", 1, 262144, 1, 128),
]
# fewer than four particles per horizontal grid cell (N < 4 Nx Ny): the spline density kernel
# and the small-mass / low-peak pruning right after HOP
SPLINE = [
    Case("w1_50k_spline", 1, 50000, 31, 128),
    Case("w1_20k_spline80", 1, 20000, 35, 80),
]
# small snapshots cut from the 20k one (the first records, from the uniform background, and
# the last ones, from the clumps): a few hundred particles with clumps among them
SMALL = [
    Case("w1_1k_small", 1, 20000, 5, 32, edit="small:100:900"),   # spline kernel, 4 clumps
    Case("w1_1k_small8", 1, 20000, 5, 8, edit="small:600:400"),   # median kernel (N >= 4 Nx Ny)
    Case("w1_200_small", 1, 20000, 5, 8, edit="small:60:140"),    # spline kernel, 1 clump
]
BY_NAME = {c.name: c for c in CASES + SPLINE + SMALL}
# command-line and parameter variants of one snapshot: (name, case, extra arguments)
VARIANTS = [
    ("w1_20k_parlist_s3", Case("w1_20k", 1, 20000, 5, 32), ["--Save_Clumps", "-s", "3"]),
    ("w1_20k_num_peaks5", Case("w1_20k_num_peaks5", 1, 20000, 5, 32, extra={"num_peaks": 5}), ["--Save_Clumps"]),
    ("w1_20k_no_ghost", Case("w1_20k", 1, 20000, 5, 32), ["--No_Ghost", "--Save_Clumps"]),
    ("w1_20k_diffuse_hill", Case("w1_20k_dh", 1, 20000, 5, 32, extra={"clump_diffuse_threshold": 0.45, "Hill_fraction_for_merge": 0.4}),
     ["--Save_Clumps"]),
    # user boxes (-x/-y/-z): only the particles inside take part, with their ids; limits given
    # high before low are swapped; a box holding the whole domain changes nothing
    ("w1_20k_box_x", Case("w1_20k", 1, 20000, 5, 32), ["-x", "-0.06,0.07", "--Save_Clumps"]),
    ("w1_20k_box_yz", Case("w1_20k_border", 1, 20000, 9, 32, edit="border"),
     ["-y", "0.09,-0.06", "-z", "-0.06,0.05", "--No_Ghost", "--Save_Clumps"]),
    ("w1_20k_box_all", Case("w1_20k", 1, 20000, 5, 32), ["-x", "-0.2,0.2"]),
]
# --Density_Vs_Scale runs (src/analyses.hpp:196-333): the sheared ball counts at every cell
# centre, written to <out>_RMPL.txt, and the clump finder on that run's tree (64-point leaves,
# no ghosts, doubled root box); alone, the flag sends the basic results into the RMPL file
DVS = [
    ("w1_20k_dvs16", Case("w1_20k_dvs16", 1, 20000, 41, 16), ["--Density_Vs_Scale", "--Save_Clumps"]),
    ("w1_20k_dvs16_find", Case("w1_20k_dvs16", 1, 20000, 41, 16), ["--Density_Vs_Scale", "--Find_Clumps"]),
    ("w1_20k_dvs32_sheared", Case("w1_20k_dvs32s", 1, 20000, 43, 32, edit="border", time=0.37), ["--Density_Vs_Scale"]),
]
# one run over two snapshot files (-f 0:1): the second is later in time and uses the first's box
MULTI = [Case("multi_0", 1, 20000, 5, 32), Case("multi_1", 1, 20000, 6, 32, time=0.25)]


def _records(c: Case):
    import plan_gb300 as pg

    L = pg.lib()
    spec = pg.SynthSpec()
    rc = L.plan_synth_default_spec(c.workload, c.n, c.seed, C.byref(spec))
    if rc:
        raise RuntimeError(f"unknown workload {c.workload}")
    spec.nx = c.nx
    spec.time = c.time
    fourpig = L.plan_synth_four_pi_G_for_mean(C.byref(spec), spec.nx, spec.nx)
    spec.G = fourpig / (4 * np.pi)
    rec = np.zeros(c.n, dtype=REC)
    info = pg.SynthInfo()
    rc = L.plan_synth_records(C.byref(spec), rec.ctypes.data, C.byref(info))
    if rc:
        raise RuntimeError(f"generator failed ({rc})")
    return rec, fourpig


def _header(n: int, time: float) -> bytes:
    lim = [-0.1, 0.1, -0.1, 0.1, -0.1, 0.1, -0.1, 0.1, -0.1, 0.1, -0.1, 0.1]
    return struct.pack("<12fi1fffq", *lim, 1, 1.0, time, 0.0, n)


def _edit(c: Case, rec: np.ndarray) -> list[np.ndarray]:
    """Apply the case's edit; returns one record array per output file."""
    n = len(rec)
    rng = np.random.default_rng(1000 + c.seed)
    if c.edit == "sinks":
        # exact positional duplicates inside the clumps (sink particles), some with equal
        # velocities, and triples in the background
        cl = np.arange(n - n // 5, n)
        a = rng.choice(cl, 600, replace=False)
        b = rng.choice(cl, 600, replace=False)
        keep = a != b
        a, b = a[keep], b[keep]
        rec["pos"][b] = rec["pos"][a]
        rec["vel"][b[:300]] = rec["vel"][a[:300]]
        t = rng.choice(np.arange(n // 2 - 2), 50, replace=False)
        rec["pos"][t + 1] = rec["pos"][t]
        rec["pos"][t + 2] = rec["pos"][t]
    elif c.edit == "border":
        # shift the box by 0.1 in x and y (float32, wrapped) so clumps straddle the faces
        p = rec["pos"]
        for d in (0, 1):
            x = (p[:, d] + np.float32(0.1)).astype(np.float32)
            x = np.where(x >= np.float32(0.1), (x - np.float32(0.2)).astype(np.float32), x)
            x = np.where(x < np.float32(-0.1), np.float32(-0.1), x)
            p[:, d] = x
    elif c.edit.startswith("small:"):
        # the first nb records and the last nc, renumbered
        nb, nc = (int(v) for v in c.edit.split(":")[1:])
        rec = np.concatenate([rec[:nb], rec[n - nc:]]).copy()
        rec["id_in_run"] = np.arange(len(rec))
    elif c.edit == "uniform":
        # the background only: no clump should survive
        keep = n - n // 5
        rec = rec[:keep].copy()
        rec["id_in_run"] = np.arange(keep)
    if c.edit == "split2":
        # two files of one snapshot (cpu_id 0 and 1), records shuffled inside each file
        half = n // 2
        parts = [rec[:half].copy(), rec[half:].copy()]
        for k, part in enumerate(parts):
            part["cpu_id"] = k
            part["id_in_run"] = np.arange(len(part))
            perm = rng.permutation(len(part))
            parts[k] = part[perm]
        return parts
    return [rec]


def materialise(c: Case, d: str | os.PathLike) -> dict:
    """Write the case under directory d in the reference's input layout.

    Returns {"lis": [paths], "param": path, "four_pi_G": value, "data_dir": d,
    "combined": bool, "sha256": [hex per file]}."""
    d = Path(d)
    d.mkdir(parents=True, exist_ok=True)
    rec, fourpig = _records(c)
    files = _edit(c, rec)
    paths = []
    if len(files) == 1:
        paths.append(d / "Snap.0000.ds.lis")
    else:
        for k in range(len(files)):
            sub = d / f"id{k}"
            sub.mkdir(exist_ok=True)
            paths.append(sub / ("Snap.0000.ds.lis" if k == 0 else f"Snap-id{k}.0000.ds.lis"))
    shas = []
    for path, part in zip(paths, files):
        blob = _header(len(part), c.time) + part.tobytes()
        path.write_bytes(blob)
        shas.append(hashlib.sha256(blob).hexdigest())
    par = d / "para.txt"
    lines = [f"Nx1 = {c.nx}", f"Nx2 = {c.nx}", f"Nx3 = {c.nx}", "Z = 0.02", f"four_pi_G_par = {fourpig!r}", f"knn = {c.knn}",
             f"hop = {c.hop}", f"num_threads = {os.cpu_count() or 1}"]
    for k, v in c.extra.items():
        lines.append(f"{k} = {v}")
    par.write_text("\n".join(lines) + "\n")
    return {"lis": [str(p) for p in paths], "param": str(par), "four_pi_G": fourpig, "data_dir": str(d),
            "combined": len(files) == 1, "sha256": shas}


def cli_args(m: dict, out_stem: str) -> list[str]:
    """The reference's command line for a materialised case (src/global.cpp:247-289)."""
    a = ["-c", str(len(m["lis"])), "-i", m["data_dir"], "-b", "Snap", "-p", "ds", "-f", "0:0", "-o", out_stem, "-t", m["param"]]
    if m["combined"]:
        a.append("--Combined")
    return a


# ---------------------------------------------------------------- canonical digests
# Every stage result is hashed in one canonical layout, whichever side produced it: the
# reference's dump files (golden script), the oracle restatement or the GPU stage arrays.

def _sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def digest_keys(keys3: np.ndarray) -> str:
    return _sha(np.asarray(keys3, dtype="<u4").reshape(-1, 3))


def digest_points(f9: np.ndarray, orig: np.ndarray, sink: np.ndarray) -> str:
    """Tree points in key order: pos, vel, mass, ath_density (f64), original_id, sink flag."""
    return _sha(np.asarray(f9, dtype="<f8")[:, :8], np.asarray(orig, dtype="<u4"), np.asarray(sink, dtype="u1"))


def digest_density(dens: np.ndarray) -> str:
    return _sha(np.asarray(dens, dtype="<f8"))


def digest_nodes(f4: np.ndarray, u7: np.ndarray) -> str:
    return _sha(np.asarray(f4, dtype="<f8").reshape(-1, 4), np.asarray(u7, dtype="<u4").reshape(-1, 7))


def digest_u32(a: np.ndarray) -> str:
    return _sha(np.asarray(a, dtype="<u4"))


def digest_clumps(peak_n: np.ndarray, f11: np.ndarray, members: np.ndarray) -> str:
    """Clumps in ascending peak order: (peak, n), 11 f64 (M, R_H, COM, v_COM, J), members."""
    order = np.argsort(peak_n[:, 0], kind="stable")
    off = np.concatenate([[0], np.cumsum(peak_n[:, 1].astype(np.int64))])
    h = hashlib.sha256()
    for k in order:
        h.update(np.asarray(peak_n[k], dtype="<u4").tobytes())
        h.update(np.asarray(f11[k], dtype="<f8").tobytes())
        h.update(np.asarray(members[off[k]:off[k + 1]], dtype="<u4").tobytes())
    return h.hexdigest()


def digest_knn(idx: np.ndarray, dr2: np.ndarray) -> str:
    return _sha(np.asarray(idx, dtype="<u4"), np.asarray(dr2, dtype="<f8"))


def find_peaks_file(d: str | os.PathLike) -> Path:
    got = sorted(Path(d).glob("peaks_at_*.txt"))
    if len(got) != 1:
        raise FileNotFoundError(f"expected one peaks_at_*.txt in {d}, found {len(got)}")
    return got[0]


def parlist_digests(d: str | os.PathLike) -> dict:
    """SHA-256 of every ParList.*/<peak_id>.txt (written by --Save_Clumps into the working
    directory), keyed by its relative path."""
    d = Path(d)
    return {str(p.relative_to(d)): hashlib.sha256(p.read_bytes()).hexdigest() for p in sorted(d.glob("ParList.*/*.txt"))}
