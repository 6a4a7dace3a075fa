"""Write the golden fixtures of the parity tests from the reference itself.

For every case of tests/cases.py this script builds the snapshot, runs the UNMODIFIED
reference (oracle/_ref/plan_ref, compiled from the reference checkout by `make -C oracle
ref`) with its stage dump switched on, and stores under tests/golden/<case>/:

  meta.json        SHA-256 of the .lis files, the parameters, the reference's summary line,
                   sizes, and canonical digests of its Morton keys, tree points, node table,
                   densities, densest-neighbour pointers, clumps and (strided) KNN lists
  peaks_at_*.txt   the reference's clump catalogue, byte for byte
  planetesimals.txt  the reference's basic-results file
  (the per-clump member lists of --Save_Clumps are pinned by their SHA-256 in meta.json)

Run it in a checkout where the reference is present:  python tests/golden/make_golden.py
(`python tests/golden/make_golden.py full_workload` writes tests/golden/w2_16m, the catalogue
of the benchmarked 16.7M-particle snapshot). It needs the reference binary and the library's
generator; nothing at test time runs it.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT))
import cases  # noqa: E402

REF = ROOT / "oracle" / "_ref" / "plan_ref"


def read_dumps(d: Path, stride: int) -> dict:
    t = np.fromfile(d / "tree.bin", dtype=np.uint8)
    n = int(t[:8].view("<u8")[0])
    rec = np.dtype([("f", "<f8", 9), ("orig", "<u4"), ("sink", "u1")])
    assert rec.itemsize == 77
    tr = t[8:].view(rec)
    assert len(tr) == n
    k = np.fromfile(d / "keys.bin", dtype=np.uint8)
    keys = k[8:].view("<u4").reshape(-1, 3)
    nb = np.fromfile(d / "nodes.bin", dtype=np.uint8)
    nn = int(nb[:8].view("<u8")[0])
    nrec = np.dtype([("f", "<f8", 4), ("u", "<u4", 4), ("orth", "<u2"), ("nd", "u1"), ("lvl", "u1")])
    assert nrec.itemsize == 52
    nd = nb[8:].view(nrec)
    assert len(nd) == nn
    u7 = np.zeros((nn, 7), dtype=np.uint32)
    u7[:, :4] = nd["u"]
    u7[:, 4] = nd["orth"]
    u7[:, 5] = nd["nd"]
    u7[:, 6] = nd["lvl"]
    hop = np.fromfile(d / "hop.bin", dtype=np.uint8)[8:].view("<u4")
    kb = np.fromfile(d / "knn.bin", dtype=np.uint8)
    hdr = kb[:12].view("<u4")
    kd = int(hdr[2])
    assert int(hdr[1]) == stride
    kr = kb[12:].view(np.dtype([("i", "<u4"), ("d", "<f8")])).reshape(-1, kd)
    cb = np.fromfile(d / "clumps.bin", dtype=np.uint8)
    nc = int(cb[:8].view("<u8")[0])
    off = 8
    pn = np.zeros((nc, 2), dtype=np.uint32)
    f11 = np.zeros((nc, 11))
    mem = []
    for c in range(nc):
        pn[c] = cb[off:off + 8].view("<u4")
        off += 8
        f11[c] = cb[off:off + 88].view("<f8")
        off += 88
        m = int(pn[c, 1])
        mem.append(cb[off:off + 4 * m].view("<u4").copy())
        off += 4 * m
    assert off == len(cb)
    members = np.concatenate(mem) if mem else np.zeros(0, dtype=np.uint32)
    return {
        "n_tree": n, "n_nodes": nn, "n_clumps": nc, "knn_stride": stride, "knn_k": kd,
        "keys": cases.digest_keys(keys),
        "points": cases.digest_points(tr["f"], tr["orig"], tr["sink"]),
        "density": cases.digest_density(tr["f"][:, 8]),
        "nodes": cases.digest_nodes(nd["f"], u7),
        "densest": cases.digest_u32(hop),
        "clumps": cases.digest_clumps(pn, f11, members),
        "knn": cases.digest_knn(kr["i"], kr["d"]),
        "n_sinks": int(tr["sink"].sum()),
    }


def oracle_cr(m: dict) -> dict:
    """Digests of the oracle restatement run with a correctly rounded pow(x, 1.5), which is
    what the GPU computes; the reference calls the host libm. The number of densities that
    differ (each by one unit in the last place) is recorded with them."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    o0 = oracle.Oracle(m["lis"], m["param"], pow_mode=0)
    o0.find()
    o1 = oracle.Oracle(m["lis"], m["param"], pow_mode=1)
    o1.find()
    d0 = o0.points()[0][:, 8]
    d1 = o1.points()[0][:, 8]
    diff = d0 != d1
    rel = float(np.max(np.abs(d1[diff] - d0[diff]) / np.abs(d0[diff]))) if diff.any() else 0.0
    return {"density_cr": cases.digest_density(d1), "densest_cr": cases.digest_u32(o1.densest()),
            "clumps_cr": cases.digest_clumps(*o1.clumps()), "n_density_cr_diff": int(diff.sum()),
            "max_rel_density_cr_diff": rel}


def multi_snapshot() -> None:
    """Two snapshots in one run (-f 0:1, the second at t = 0.25): the reference's summary
    stream keeps the scientific notation WriteBasicResults leaves on it, and the second file
    takes the box and masses of the first."""
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        shas = []
        for k, c in enumerate(cases.MULTI):
            m = cases.materialise(c, tmp / f"c{k}")
            dst = tmp / "in" / f"Snap.{k:04d}.ds.lis"
            dst.parent.mkdir(exist_ok=True)
            shutil.copy(m["lis"][0], dst)
            shas.append(m["sha256"][0])
            if k == 0:
                shutil.copy(m["param"], tmp / "in" / "para.txt")
        out = tmp / "ref"
        out.mkdir()
        args = ["-c", "1", "-i", str(tmp / "in"), "-b", "Snap", "-p", "ds", "-f", "0:1", "-o", str(out / "res.txt"), "-t",
                str(tmp / "in" / "para.txt"), "--Combined"]
        r = subprocess.run([str(REF)] + args, cwd=out, capture_output=True, text=True, check=True)
        g = HERE / "multi_snapshot"
        if g.exists():
            shutil.rmtree(g)
        g.mkdir()
        peaks = sorted(out.glob("peaks_at_*.txt"))
        for pk in peaks:
            shutil.copy(pk, g / pk.name)
        shutil.copy(out / "res_planetesimals.txt", g / "planetesimals.txt")
        summary = [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln]
        meta = {"lis_sha256": shas, "summary": summary, "peaks_files": [pk.name for pk in peaks]}
        (g / "meta.json").write_text(json.dumps(meta, indent=1) + "\n")
        print("multi_snapshot:", *summary, sep="\n  ")


def multi_density_vs_scale() -> None:
    """The two-snapshot run with --Density_Vs_Scale alone: one RMPL header, a line per
    snapshot, the basic results in the same file, the summary stream scientific throughout."""
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        d = tmp / "in"
        d.mkdir()
        for k, c in enumerate(cases.MULTI):
            m = cases.materialise(c, tmp / f"c{k}")
            shutil.copy(m["lis"][0], d / f"Snap.{k:04d}.ds.lis")
            if k == 0:
                shutil.copy(m["param"], d / "para.txt")
        out = tmp / "ref"
        out.mkdir()
        args = ["-c", "1", "-i", str(d), "-b", "Snap", "-p", "ds", "-f", "0:1", "-o", str(out / "res.txt"), "-t", str(d / "para.txt"),
                "--Combined", "--Density_Vs_Scale"]
        r = subprocess.run([str(REF)] + args, cwd=out, capture_output=True, text=True, check=True)
        g = HERE / "multi_density_vs_scale"
        if g.exists():
            shutil.rmtree(g)
        g.mkdir()
        files = sorted(p.name for p in out.iterdir() if p.is_file())
        for f in files:
            shutil.copy(out / f, g / f)
        summary = [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln]
        (g / "meta.json").write_text(json.dumps({"summary": summary, "files": files}, indent=1) + "\n")
        print("multi_density_vs_scale:", files, *summary, sep="\n  ")


def variants() -> None:
    """Command-line and parameter variants of one snapshot, run by the reference's CLI."""
    for name, c, extra in cases.VARIANTS:
        with tempfile.TemporaryDirectory() as tmp:
            tmp = Path(tmp)
            m = cases.materialise(c, tmp / "in")
            out = tmp / "ref"
            out.mkdir()
            r = subprocess.run([str(REF)] + cases.cli_args(m, str(out / "res.txt")) + extra, cwd=out, capture_output=True, text=True,
                               check=True)
            g = HERE / name
            if g.exists():
                shutil.rmtree(g)
            g.mkdir()
            pk = cases.find_peaks_file(out)
            shutil.copy(pk, g / pk.name)
            shutil.copy(out / "res_planetesimals.txt", g / "planetesimals.txt")
            summary = [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln]
            meta = {"case": name, "lis_sha256": m["sha256"], "args": extra, "summary": summary[0].strip(), "peaks_file": pk.name,
                    "parlist": cases.parlist_digests(out)}
            (g / "meta.json").write_text(json.dumps(meta, indent=1) + "\n")
            print(f"{name}: {meta['summary']} ({len(meta['parlist'])} member lists)")


def dvs_variants() -> None:
    """--Density_Vs_Scale runs of the reference's CLI: every file it writes, byte for byte."""
    for name, c, extra in cases.DVS:
        with tempfile.TemporaryDirectory() as tmp:
            tmp = Path(tmp)
            m = cases.materialise(c, tmp / "in")
            out = tmp / "ref"
            out.mkdir()
            r = subprocess.run([str(REF)] + cases.cli_args(m, str(out / "res.txt")) + extra, cwd=out, capture_output=True, text=True,
                               check=True)
            g = HERE / name
            if g.exists():
                shutil.rmtree(g)
            g.mkdir()
            files = sorted(p.name for p in out.iterdir() if p.is_file())
            for f in files:
                shutil.copy(out / f, g / f)
            summary = [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln]
            meta = {"case": name, "lis_sha256": m["sha256"], "args": extra, "summary": summary, "files": files,
                    "parlist": cases.parlist_digests(out)}
            (g / "meta.json").write_text(json.dumps(meta, indent=1) + "\n")
            print(f"{name}: {files} {summary}")


def full_workload(n: int = 0, name: str = "w2_16m", keep_peaks: bool = True) -> None:
    """The benchmarked snapshot itself (bench.py's default: 16,777,216 particles of the
    workload-2 mixture, seed 1), run by the reference without stage dumps, which would be
    gigabytes at this size: its catalogue, its basic-results file and the catalogue's SHA-256,
    which bench.py and the full-size GPU test compare with. With n = 2^27 (name w2_134m) the
    same for the largest snapshot; its catalogue (half a megabyte) is kept as a digest only.
    That run takes about 20 minutes and 41 GB on 8 cores."""
    import hashlib

    import bench

    n = n or bench.N_FULL
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        (tmp / "in").mkdir()
        rec, fourpig = bench.make_records(n, bench.SEED, pinned=False)
        lis = tmp / "in" / "Snap.0000.ds.lis"
        bench.write_lis(lis, rec.numpy(), n)
        del rec
        bench.write_params(tmp / "in" / "para.txt", fourpig, os.cpu_count() or 1)
        out = tmp / "ref"
        out.mkdir()
        args = ["-c", "1", "-i", str(tmp / "in"), "-b", "Snap", "-p", "ds", "-f", "0:0", "-o", str(out / "res.txt"), "-t",
                str(tmp / "in" / "para.txt"), "--Combined"]
        r = subprocess.run([str(REF)] + args, cwd=out, capture_output=True, text=True, check=True)
        summary = [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln]
        assert len(summary) == 1, r.stdout
        g = HERE / name
        if g.exists():
            shutil.rmtree(g)
        g.mkdir()
        pk = cases.find_peaks_file(out)
        if keep_peaks:
            shutil.copy(pk, g / pk.name)
        shutil.copy(out / "res_planetesimals.txt", g / "planetesimals.txt")
        h = hashlib.sha256()
        with open(lis, "rb") as fh:
            for blk in iter(lambda: fh.read(1 << 24), b""):
                h.update(blk)
        meta = {"case": name, "n": n, "seed": bench.SEED, "workload": bench.WORKLOAD, "lis_sha256": h.hexdigest(), "four_pi_G": fourpig,
                "summary": summary[0].strip(), "peaks_file": pk.name, "peaks_sha256": hashlib.sha256(pk.read_bytes()).hexdigest()}
        (g / "meta.json").write_text(json.dumps(meta, indent=1) + "\n")
        print(f"{name}:", meta["summary"])


def main() -> None:
    if not REF.exists():
        sys.exit(f"{REF} missing: run `make -C oracle ref` in a checkout with the reference")
    only = set(sys.argv[1:])
    if "full_workload" in only:  # the benchmarked snapshot only on request: minutes of CPU time
        full_workload()
    if "full_workload_2p27" in only:  # 2^27 particles: tens of minutes of CPU time
        full_workload(1 << 27, "w2_134m", keep_peaks=False)
    if not only or "multi_snapshot" in only:
        multi_snapshot()
    if not only or "variants" in only:
        variants()
    if not only or "dvs" in only:
        dvs_variants()
        multi_density_vs_scale()
    for c in cases.CASES + cases.SPLINE + cases.SMALL:
        if only and c.name not in only:
            continue
        with tempfile.TemporaryDirectory() as tmp:
            tmp = Path(tmp)
            m = cases.materialise(c, tmp / "in")
            out = tmp / "ref"
            out.mkdir()
            dump = tmp / "dump"
            dump.mkdir()
            stride = 1 if c.n <= 100000 else 97
            env = dict(os.environ, PLAN_REF_DUMP=str(dump), PLAN_REF_KNN_STRIDE=str(stride))
            r = subprocess.run([str(REF)] + cases.cli_args(m, str(out / "res.txt")) + ["--Save_Clumps"], env=env, cwd=out,
                               capture_output=True, text=True, check=True)
            summary = [ln for ln in r.stdout.splitlines() if "Finish clump finding" in ln]
            assert len(summary) == 1, r.stdout
            g = HERE / c.name
            if g.exists():
                shutil.rmtree(g)
            g.mkdir()
            pk = cases.find_peaks_file(out)
            shutil.copy(pk, g / pk.name)
            shutil.copy(out / "res_planetesimals.txt", g / "planetesimals.txt")
            meta = {"case": c.name, "lis_sha256": m["sha256"], "four_pi_G": m["four_pi_G"], "summary": summary[0].strip(),
                    "peaks_file": pk.name, "parlist": cases.parlist_digests(out)}
            meta.update(read_dumps(dump, stride))
            meta.update(oracle_cr(m))
            (g / "meta.json").write_text(json.dumps(meta, indent=1) + "\n")
            print(f"{c.name}: {meta['n_tree']} points, {meta['n_nodes']} nodes, {meta['n_clumps']} clumps, "
                  f"{meta['n_sinks']} sinks | {meta['summary']}")


if __name__ == "__main__":
    main()
