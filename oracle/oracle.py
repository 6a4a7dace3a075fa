"""ctypes view of the oracle restatement (oracle/port), for tests and the CPU baseline only.

The oracle is test infrastructure: it checks the GPU product and times the CPU baseline;
the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle_port.so"
CLI = HERE / "build" / "oracle_plan"
REF = HERE / "_ref" / "plan_ref"
_lib = None


def build() -> None:
    subprocess.run(["make", "-C", str(HERE), "port"], check=True, capture_output=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
        L.orc_open.restype = vp
        L.orc_open.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int]
        L.orc_close.argtypes = [vp]
        L.orc_load.argtypes = [vp, C.c_char_p]
        L.orc_find.argtypes = [vp]
        L.orc_timings.argtypes = [vp, C.POINTER(C.c_double)]
        L.orc_summary.restype = C.c_char_p
        L.orc_summary.argtypes = [vp]
        for f in ("orc_num_points", "orc_num_nodes", "orc_num_input", "orc_num_clumps"):
            getattr(L, f).restype = u32
            getattr(L, f).argtypes = [vp]
        L.orc_points.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_keys.argtypes = [vp, C.c_void_p]
        L.orc_nodes.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.orc_tree_box.argtypes = [vp, C.c_void_p]
        L.orc_knn.restype = C.c_int
        L.orc_knn.argtypes = [vp, C.c_void_p, C.c_uint, C.c_double, C.c_void_p, C.c_void_p]
        L.orc_densest.argtypes = [vp, C.c_void_p]
        L.orc_peaks.argtypes = [vp, C.c_void_p]
        L.orc_thresholds.argtypes = [vp, C.c_void_p]
        L.orc_stats.argtypes = [vp, C.c_void_p]
        L.orc_clumps.restype = u64
        L.orc_clumps.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_write_outputs.argtypes = [vp, C.c_char_p, C.c_int]
        L.orc_morton_order.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
        L.orc_set_user_box.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.orc_set_density_vs_scale.argtypes = [vp]
        L.orc_density_vs_scale.restype = C.c_int
        L.orc_density_vs_scale.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_density_vs_scale_params.argtypes = [vp, C.c_void_p]
        _lib = L
    return _lib


def morton_order(keys3: np.ndarray) -> np.ndarray:
    """Input indices in the order std::sort with the reference's Morton comparator leaves them."""
    k = np.ascontiguousarray(keys3, dtype=np.uint32).reshape(-1, 3)
    out = np.empty(len(k), dtype=np.uint32)
    lib().orc_morton_order(k.ctypes.data, len(k), out.ctypes.data)
    return out


class Oracle:
    """One snapshot through the CPU restatement: tree, densities, HOP, clumps."""

    def __init__(self, lis, param: str | None, threads: int = 0, pow_mode: int = 0, no_ghost: bool = False, user_box=None,
                 density_vs_scale: bool = False):
        """lis: one path or the list of files of one snapshot (id0 first); user_box: optional
        ((lo_x, lo_y, lo_z), (hi_x, hi_y, hi_z)) as given by -x/-y/-z (0, 0 = unrestricted)."""
        L = lib()
        self._h = L.orc_open((param or "").encode(), int(threads), int(pow_mode), int(no_ghost))
        if not self._h:
            raise RuntimeError(f"oracle: cannot read parameters {param}")
        if user_box is not None:
            lo = np.ascontiguousarray(user_box[0], dtype=np.float64)
            hi = np.ascontiguousarray(user_box[1], dtype=np.float64)
            L.orc_set_user_box(self._h, lo.ctypes.data, hi.ctypes.data)
        if density_vs_scale:
            L.orc_set_density_vs_scale(self._h)
        paths = [lis] if isinstance(lis, (str, bytes)) or not hasattr(lis, "__iter__") else list(lis)
        rc = L.orc_load(self._h, "\n".join(str(p) for p in paths).encode())
        if rc:
            raise RuntimeError(f"oracle: cannot read {lis} (status {rc})")

    def density_vs_scale(self):
        """BasicAnalysesWithTree on the loaded tree: (radii, densities)."""
        r = np.zeros(32)
        v = np.zeros(32)
        n = lib().orc_density_vs_scale(self._h, r.ctypes.data, v.ctypes.data, 32)
        return r[:n], v[:n]

    def density_vs_scale_params(self) -> np.ndarray:
        out = np.zeros(19)
        lib().orc_density_vs_scale_params(self._h, out.ctypes.data)
        return out

    def find(self) -> int:
        n = int(lib().orc_find(self._h))
        if n < 0:
            raise ValueError(f"oracle: {self.summary()}")
        return n

    def timings(self) -> np.ndarray:
        a = np.zeros(3)
        lib().orc_timings(self._h, a.ctypes.data)
        return a

    def summary(self) -> str:
        return lib().orc_summary(self._h).decode()

    def points(self):
        n = lib().orc_num_points(self._h)
        f = np.empty((n, 9))
        orig = np.empty(n, dtype=np.uint32)
        sink = np.empty(n, dtype=np.uint8)
        lib().orc_points(self._h, f.ctypes.data, orig.ctypes.data, sink.ctypes.data)
        return f, orig, sink

    def keys(self) -> np.ndarray:
        n = lib().orc_num_points(self._h)
        k = np.empty((n, 3), dtype=np.uint32)
        lib().orc_keys(self._h, k.ctypes.data)
        return k

    def nodes(self):
        n = lib().orc_num_nodes(self._h)
        f = np.empty((n, 4))
        u = np.empty((n, 7), dtype=np.uint32)
        lib().orc_nodes(self._h, f.ctypes.data, u.ctypes.data)
        return f, u

    def tree_box(self) -> np.ndarray:
        a = np.empty(5)
        lib().orc_tree_box(self._h, a.ctypes.data)
        return a

    def knn(self, pos, k: int, est: float = 0.0):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        idx = np.empty((pos.shape[0], k), dtype=np.uint32)
        dr2 = np.empty((pos.shape[0], k))
        for i in range(pos.shape[0]):
            rc = lib().orc_knn(self._h, pos[i].ctypes.data, k, float(est), idx[i].ctypes.data, dr2[i].ctypes.data)
            if rc:
                raise LookupError(f"oracle: position {pos[i].tolist()} has no leaf in the tree")
        return idx, dr2

    def densest(self) -> np.ndarray:
        a = np.empty(lib().orc_num_points(self._h), dtype=np.uint32)
        lib().orc_densest(self._h, a.ctypes.data)
        return a

    def peaks(self) -> np.ndarray:
        a = np.empty(lib().orc_num_points(self._h), dtype=np.uint32)
        lib().orc_peaks(self._h, a.ctypes.data)
        return a

    def thresholds(self) -> np.ndarray:
        a = np.empty(4)
        lib().orc_thresholds(self._h, a.ctypes.data)
        return a

    def stats(self) -> np.ndarray:
        a = np.empty(8, dtype=np.uint64)
        lib().orc_stats(self._h, a.ctypes.data)
        return a

    def clumps(self):
        nc = lib().orc_num_clumps(self._h)
        pn = np.empty((nc, 2), dtype=np.uint32)
        f = np.empty((nc, 11))
        m = int(lib().orc_clumps(self._h, pn.ctypes.data, f.ctypes.data, None))
        mem = np.empty(m, dtype=np.uint32)
        lib().orc_clumps(self._h, None, None, mem.ctypes.data)
        return pn, f, mem

    def write_outputs(self, out_path: str, first: bool = True) -> None:
        rc = lib().orc_write_outputs(self._h, str(out_path).encode(), int(first))
        if rc:
            raise RuntimeError(f"oracle: cannot write outputs next to {out_path}")

    def close(self):
        if self._h:
            lib().orc_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
