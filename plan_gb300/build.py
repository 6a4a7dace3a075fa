"""Build recipe for the in-tree native code.

Compiles the CUDA translation units for sm_103a only and the host C++ with g++, links
``plan_gb300/lib/libplan_gpu.so`` (the C ABI of ``include/plan_gpu.h``), the drop-in
command-line program ``plan_gb300/lib/plan_gpu`` and ``plan_gb300/lib/libplan_synth.so`` (the
snapshot generator of ``include/plan_synth.h`` alone, for callers without a GPU). All floating-point code is built without
contraction (``--fmad=false`` / ``-ffp-contract=off``) so results round exactly like the
reference's x86-64 build on both x86-64 and aarch64 hosts. Objects go to
``plan_gb300/_build/``; nothing is installed outside the tree.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
OBJ = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["radix_sort.cu", "scan.cu", "introsort.cu", "front.cu", "knn.cu", "hop.cu", "clumps.cu", "dvs.cu", "energy.cu", "parlist.cu", "server.cu", "capi.cu"]
HOST_SOURCES = ["host/params.cpp", "host/lis.cpp", "host/catalogue.cpp", "host/synth.cpp"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build plan_gb300")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile everything that is out of date; return the path of libplan_gpu.so."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    OUT.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    headers = (list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((CSRC / "host").glob("*.hpp")) +
               list((ROOT / "include").glob("*.h")))
    inc = ["-I" + str(ROOT / "include"), "-I" + str(CSRC)]
    steps = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = OBJ / (Path(src).stem + ".o")
        objs.append(o)
        if not _newer(o, [s] + headers):
            steps.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "--extended-lambda", "-Xcompiler",
                          "-fPIC,-ffp-contract=off", *inc, "-c", str(s), "-o", str(o)])
    for src in HOST_SOURCES:
        s = CSRC / src
        o = OBJ / (Path(src).stem + ".o")
        objs.append(o)
        if not _newer(o, [s] + headers):
            steps.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", *inc, "-I" + str(cuda / "include"),
                          "-c", str(s), "-o", str(o)])
    jobs = jobs or min(len(steps) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for fut in [ex.submit(_run, c) for c in steps]:
            fut.result()
    lib = OUT / "libplan_gpu.so"
    if not _newer(lib, objs):
        _run(["g++", "-shared", "-o", str(lib), *map(str, objs), "-L" + str(cuda / "lib64"), "-lcudart", "-fopenmp",
              "-Wl,-rpath," + str(cuda / "lib64")])
    # the snapshot generator alone (no CUDA): what the CPU-only benchmark arm loads
    synth = OUT / "libplan_synth.so"
    synth_o = OBJ / "synth.o"
    if not _newer(synth, [synth_o]):
        _run(["g++", "-shared", "-o", str(synth), str(synth_o), "-fopenmp"])
    cli = OUT / "plan_gpu"
    cli_src = CSRC / "host" / "cli.cpp"
    if not _newer(cli, [cli_src, lib] + headers):
        _run(["g++", "-O2", "-std=c++17", *inc, str(cli_src), "-o", str(cli), "-L" + str(OUT), "-lplan_gpu", "-Wl,-rpath,$ORIGIN",
              "-L" + str(cuda / "lib64"), "-lcudart", "-Wl,-rpath," + str(cuda / "lib64")])
    if verbose:
        print(f"built {lib} and {cli} ({len(steps)} units recompiled)")
    return lib


def build_oracle(reference_src: str | None = None) -> None:
    """Build the CPU restatement (always) and the reference oracle when the reference's
    src/ directory is given (argument, else the PLAN_REF_SRC environment variable) and holds
    its sources."""
    _run(["make", "-C", str(ROOT / "oracle"), "port"])
    src = reference_src or os.environ.get("PLAN_REF_SRC")
    if src and (Path(src) / "tree.hpp").exists():
        _run(["make", "-C", str(ROOT / "oracle"), "ref", f"REF_SRC={Path(src).resolve()}"])


if __name__ == "__main__":
    build(verbose=True)
    build_oracle(sys.argv[1] if len(sys.argv) > 1 else None)
    sys.exit(0)
