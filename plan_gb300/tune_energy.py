#!/usr/bin/env python3
"""Choose the tile width of the batched boundness pass per group-size class, on the GPU.

For every size class of plan_group_energies (groups of n < 64, < 512, < 8192 and larger
particles) a batch of Plummer groups of that class is timed with every tile width the pass
is built for (32, 64, 128, 256); the fastest width per class is written to
plan_gb300/csrc/energy_tiles.h (rebuild the library afterwards), and the timings as a
Markdown table to stdout. PLAN_ENERGY_TILES selects the widths for each trial.

    python plan_gb300/tune_energy.py [--write]
"""
from __future__ import annotations

import argparse
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
WIDTHS = (32, 64, 128, 256)
# (lower, upper) group sizes per class and the number of groups timed; the classes'
# bounds are those of energy_tiles.h
CLASSES = [((2, 64), 20000), ((64, 512), 4000), ((512, 8192), 400), ((8192, 131072), 12)]
DEFAULT = (32, 64, 128, 128)


def groups(lo: int, hi: int, k: int, seed: int):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), k)).astype(np.int64)
    sizes = np.clip(sizes, lo, hi - 1)
    n = int(sizes.sum())
    r = 1e-3 * (rng.uniform(0, 1, n) ** (-2 / 3) - 1) ** -0.5  # Plummer radii
    u = rng.normal(size=(n, 3))
    pos = (u / np.linalg.norm(u, axis=1)[:, None] * r[:, None]).astype(np.float32)
    vel = (1e-3 * rng.normal(size=(n, 3))).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    return pos, vel, mass, off


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--write", action="store_true", help="write the chosen widths to energy_tiles.h")
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    sys.path.insert(0, str(HERE.parent))
    import ctypes as C

    import plan_gb300 as pg

    p = pg.params()
    pg.lib().plan_params_derive(C.byref(p))
    f = pg.Finder(0)
    best = list(DEFAULT)
    rows = []
    try:
        for k, ((lo, hi), count) in enumerate(CLASSES):
            pos, vel, mass, off = groups(lo, hi, count, 11 + k)
            sizes = np.diff(off.astype(np.int64))
            pairs = int((sizes * (sizes - 1) // 2).sum())
            times = {}
            for w in WIDTHS:
                tiles = list(DEFAULT)
                tiles[k] = w
                os.environ["PLAN_ENERGY_TILES"] = ",".join(map(str, tiles))
                f.group_energies(pos, vel, mass, off, p)  # warm-up
                t = []
                for _ in range(args.reps):
                    t0 = time.perf_counter()
                    f.group_energies(pos, vel, mass, off, p)
                    t.append(time.perf_counter() - t0)
                times[w] = min(t)
            best[k] = min(times, key=times.get)
            rows.append((k, lo, hi, count, pairs, times, best[k]))
    finally:
        os.environ.pop("PLAN_ENERGY_TILES", None)
        f.close()
    print("| class | group sizes | groups | pairs | " + " | ".join(f"w={w} (ms)" for w in WIDTHS) + " | chosen |")
    print("|---|---|---|---|" + "---|" * len(WIDTHS) + "---|")
    for k, lo, hi, count, pairs, times, b in rows:
        print(f"| {k} | [{lo}, {hi}) | {count} | {pairs:.3e} | " + " | ".join(f"{1e3 * times[w]:.2f}" for w in WIDTHS) + f" | {b} |")
    if args.write:
        h = HERE / "csrc" / "energy_tiles.h"
        s = h.read_text()
        import re

        s = re.sub(r"constexpr int kEnergyTile\[kEnergyClasses\] = \{[^}]*\};",
                   "constexpr int kEnergyTile[kEnergyClasses] = {" + ", ".join(map(str, best)) + "};", s)
        h.write_text(s)
        print(f"\nwrote {h.name}: {best}")


if __name__ == "__main__":
    main()
