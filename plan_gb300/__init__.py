"""plan_gb300: GB300-native clump finding with PLAN's find-clumps interface.

Python view of the C ABI in ``include/plan_gpu.h``: the parameter file reader, the
``.lis`` reader, the two calls the reference's main program makes per snapshot
(``BHtree::BuildTree`` and ``BHtree::FindPlanetesimals``) and the catalogue writers, plus
inspection of stage arrays. Everything runs in ``lib/libplan_gpu.so``; there is no CPU
implementation behind this module, and importing the bindings fails if the native library
has not been built (``plan_gb300.build.build()``).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "lib" / "libplan_gpu.so"
_lib = None

PLAN_ARR_TREE_POS = 1
PLAN_ARR_TREE_VEL = 2
PLAN_ARR_DENSITY = 3
PLAN_ARR_ORIG_ID = 4
PLAN_ARR_KEYS = 5
PLAN_ARR_NODE_F = 6
PLAN_ARR_NODE_U = 7
PLAN_ARR_DENSEST = 8
PLAN_ARR_PEAK = 9
PLAN_ARR_SINK_COUNT = 10
PLAN_NOALLOC_SORT_MAX = 65536

STATUS = {0: "ok", 2: "argument", 3: "I/O", 4: "parameter", 5: "CUDA", 6: "out of device memory", 7: "unsupported input",
          8: "device loop limit"}


class PlanError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        super().__init__(f"plan_gpu status {status} ({STATUS.get(status, '?')}): {msg}")
        self.status = status


class Params(C.Structure):
    _fields_ = [
        ("solid_to_gas_ratio", C.c_double), ("box_resolution", C.c_uint32 * 3), ("four_pi_G", C.c_double),
        ("num_threads", C.c_uint32), ("num_peaks", C.c_uint32), ("knn", C.c_uint32), ("hop", C.c_uint32),
        ("fixed_hop", C.c_int32), ("clump_diffuse_threshold", C.c_double), ("Hill_fraction_for_merge", C.c_double),
        ("q", C.c_double), ("Omega", C.c_double), ("rho_g0", C.c_double), ("ghost_zone_width", C.c_double * 3),
        ("box_min", C.c_double * 3), ("box_max", C.c_double * 3), ("box_center", C.c_double * 3),
        ("box_length", C.c_double * 3), ("box_half_width", C.c_double * 3), ("max_half_width", C.c_double),
        ("max_ghost_zone_width", C.c_double), ("cell_length", C.c_double * 3), ("cell_volume", C.c_double),
        ("mass_total_code_units", C.c_double), ("G_tilde", C.c_double), ("mass_physical", C.c_double),
        ("grav_constant", C.c_double), ("shear_speed", C.c_double), ("min_trusted_mass", C.c_double),
        ("ntypes", C.c_uint32), ("mass_per_particle", C.c_double * 16), ("mass_fraction_per_species", C.c_double * 16),
        ("box_set", C.c_int32), ("no_ghost", C.c_int32), ("user_box", C.c_int32), ("user_box_min", C.c_double * 3),
        ("user_box_max", C.c_double * 3), ("density_vs_scale", C.c_int32),
    ]


class LisView(C.Structure):
    _fields_ = [("coor_lim", C.c_double * 12), ("ntypes", C.c_uint32), ("type_info", C.c_double * 16), ("time", C.c_double),
                ("dt", C.c_double), ("nblocks", C.c_uint32), ("records", C.POINTER(C.c_void_p)), ("counts", C.POINTER(C.c_uint64))]


class ClumpInfo(C.Structure):
    _fields_ = [("peak_id", C.c_uint32), ("npar", C.c_uint32), ("total_mass", C.c_double), ("hill_radius", C.c_double),
                ("com", C.c_double * 3), ("vel_com", C.c_double * 3), ("J", C.c_double * 3)]


class SynthSpec(C.Structure):
    _fields_ = [("n", C.c_uint64), ("seed", C.c_uint64), ("frac_uniform", C.c_double), ("frac_sheets", C.c_double),
                ("n_sheets", C.c_int32), ("sheet_sigma", C.c_double), ("n_clumps", C.c_int32), ("mass_function", C.c_int32),
                ("mf_slope", C.c_double), ("mf_lo", C.c_double), ("mf_hi", C.c_double), ("a_lo", C.c_double), ("a_hi", C.c_double),
                ("unbound_frac", C.c_double), ("unbound_vscale", C.c_double), ("G", C.c_double), ("half_box", C.c_double),
                ("nx", C.c_int32), ("Z", C.c_double), ("time", C.c_float)]


class SynthInfo(C.Structure):
    _fields_ = [("n_uniform", C.c_uint64), ("n_sheets", C.c_uint64), ("n_clumps", C.c_uint64), ("particle_mass", C.c_double),
                ("mean_density", C.c_double), ("clump_mass_min", C.c_double), ("clump_mass_max", C.c_double)]


def lib() -> C.CDLL:
    """The native library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise ImportError(f"{_LIB_PATH} is missing: run plan_gb300.build.build() (there is no CPU fallback)")
        L = C.CDLL(str(_LIB_PATH))
        vp, i32, u32, u64, dp = C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.POINTER(C.c_double)
        sig = {
            "plan_params_init": (None, [C.POINTER(Params)]),
            "plan_params_read": (i32, [C.c_char_p, C.POINTER(Params)]),
            "plan_params_derive": (None, [C.POINTER(Params)]),
            "plan_lis_read": (i32, [C.POINTER(C.c_char_p), i32, C.POINTER(vp)]),
            "plan_lis_free": (None, [vp]),
            "plan_lis_count": (u64, [vp]),
            "plan_lis_time": (C.c_double, [vp]),
            "plan_lis_get_view": (i32, [vp, C.POINTER(LisView)]),
            "plan_ctx_create": (i32, [i32, C.POINTER(vp)]),
            "plan_ctx_destroy": (None, [vp]),
            "plan_last_error": (C.c_char_p, [vp]),
            "plan_footprint_bytes": (u64, [u64, C.POINTER(Params)]),
            "plan_build_tree": (i32, [vp, C.POINTER(LisView), C.POINTER(Params), i32, vp]),
            "plan_find_planetesimals": (i32, [vp, C.POINTER(Params), vp, C.POINTER(vp)]),
            "plan_find_clumps": (i32, [vp, C.POINTER(LisView), C.POINTER(Params), i32, vp, C.POINTER(vp)]),
            "plan_catalogue_free": (None, [vp]),
            "plan_catalogue_count": (u32, [vp]),
            "plan_catalogue_get": (i32, [vp, u32, C.POINTER(ClumpInfo)]),
            "plan_catalogue_summary": (C.c_char_p, [vp]),
            "plan_catalogue_write_peaks": (i32, [vp, C.c_char_p, i32, i32, u32]),
            "plan_catalogue_write_parlists": (i32, [vp, vp, i32, u32]),
            "plan_ctx_release": (i32, [vp]),
            "plan_group_energies": (i32, [vp, vp, vp, vp, vp, u32, C.POINTER(Params), vp, vp, C.POINTER(C.c_uint64)]),
            "plan_density_vs_scale": (i32, [vp, C.POINTER(Params), C.c_double, dp, dp, i32, C.POINTER(C.c_int32)]),
            "plan_server_create": (i32, [i32, i32, u64, C.POINTER(vp)]),
            "plan_server_destroy": (None, [vp]),
            "plan_submit": (i32, [vp, C.POINTER(LisView), C.POINTER(Params), i32, C.POINTER(C.c_uint64)]),
            "plan_poll": (i32, [vp, u64, i32, C.POINTER(vp), C.POINTER(C.c_double)]),
            "plan_server_error": (C.c_char_p, [vp]),
            "plan_server_stats": (i32, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
            "plan_server_overlap": (i32, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "plan_catalogue_basic_results": (i32, [vp, C.POINTER(Params), i32, C.c_char_p, C.c_size_t]),
            "plan_stage_count": (u64, [vp, i32]),
            "plan_stage_copy": (i32, [vp, i32, vp, C.c_size_t]),
            "plan_knn": (i32, [vp, dp, u32, u32, C.c_double, C.POINTER(C.c_uint32), dp]),
            "plan_morton_order": (i32, [vp, vp, u32, vp]),
            "plan_morton_order_noalloc": (i32, [vp, vp, u32, vp]),
            "plan_stage_times": (i32, [vp, dp, i32]),
            "plan_kernel_launches": (u64, [vp]),
            "plan_counters": (i32, [vp, C.POINTER(C.c_uint64), i32]),
            "plan_synth_default_spec": (i32, [i32, u64, u64, C.POINTER(SynthSpec)]),
            "plan_synth_records": (i32, [C.POINTER(SynthSpec), vp, C.POINTER(SynthInfo)]),
            "plan_synth_write_lis": (i32, [C.c_char_p, C.POINTER(SynthSpec), C.POINTER(SynthInfo)]),
            "plan_synth_four_pi_G_for_mean": (C.c_double, [C.POINTER(SynthSpec), C.c_int32, C.c_int32]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


EXPORTED = [
    "plan_params_init", "plan_params_read", "plan_params_derive", "plan_lis_read", "plan_lis_free", "plan_lis_count",
    "plan_lis_time", "plan_lis_get_view", "plan_ctx_create", "plan_ctx_destroy", "plan_last_error", "plan_footprint_bytes",
    "plan_build_tree", "plan_find_planetesimals", "plan_find_clumps", "plan_catalogue_free", "plan_catalogue_count",
    "plan_catalogue_get", "plan_catalogue_summary", "plan_catalogue_write_peaks", "plan_catalogue_write_parlists",
    "plan_catalogue_basic_results", "plan_ctx_release", "plan_group_energies", "plan_density_vs_scale", "plan_server_create", "plan_server_destroy", "plan_submit", "plan_poll",
    "plan_server_error", "plan_server_stats", "plan_server_overlap",
    "plan_stage_count", "plan_stage_copy", "plan_knn", "plan_morton_order", "plan_morton_order_noalloc", "plan_stage_times", "plan_kernel_launches", "plan_counters",
    "plan_synth_default_spec", "plan_synth_records", "plan_synth_write_lis", "plan_synth_four_pi_G_for_mean",
]


def params(path: str | None = None) -> Params:
    """NumericalParameters: defaults, then the parameter file when given."""
    p = Params()
    lib().plan_params_init(C.byref(p))
    if path:
        rc = lib().plan_params_read(str(path).encode(), C.byref(p))
        if rc:
            raise PlanError(rc, f"reading {path}")
    return p


def synth_lis(path: str, workload: int, n: int = 0, seed: int = 1, nx: int = 128, time: float = 0.0) -> tuple[float, SynthInfo]:
    """Write a synthetic snapshot; returns (four_pi_G_par putting rho_thr at the mean density, info)."""
    L = lib()
    s = SynthSpec()
    rc = L.plan_synth_default_spec(int(workload), int(n), int(seed), C.byref(s))
    if rc:
        raise PlanError(rc, "unknown workload")
    s.nx = int(nx)
    s.time = float(time)
    fourpig = L.plan_synth_four_pi_G_for_mean(C.byref(s), s.nx, s.nx)
    s.G = fourpig / (4 * np.pi)
    info = SynthInfo()
    rc = L.plan_synth_write_lis(str(path).encode(), C.byref(s), C.byref(info))
    if rc:
        raise PlanError(rc, f"writing {path}")
    return fourpig, info


def write_param_file(path: str, nx: int, four_pi_G: float, knn: int = 32, hop: int = 16, threads: int | None = None,
                     extra: dict | None = None) -> None:
    lines = [f"Nx1 = {nx}", f"Nx2 = {nx}", f"Nx3 = {nx}", "Z = 0.02", f"four_pi_G_par = {four_pi_G!r}", f"knn = {knn}",
             f"hop = {hop}", f"num_threads = {threads or os.cpu_count() or 1}"]
    for k, v in (extra or {}).items():
        lines.append(f"{k} = {v}")
    Path(path).write_text("\n".join(lines) + "\n")


class Snapshot:
    """A .lis snapshot read into page-locked host memory (ReadSingleLisFile / ReadMultipleLisFile)."""

    def __init__(self, paths):
        if isinstance(paths, (str, os.PathLike)):
            paths = [paths]
        arr = (C.c_char_p * len(paths))(*[str(p).encode() for p in paths])
        h = C.c_void_p()
        rc = lib().plan_lis_read(arr, len(paths), C.byref(h))
        if rc:
            raise PlanError(rc, f"reading {paths}")
        self._h = h
        self.view = LisView()
        lib().plan_lis_get_view(h, C.byref(self.view))

    @property
    def n(self) -> int:
        return int(lib().plan_lis_count(self._h))

    @property
    def time(self) -> float:
        return float(self.view.time)

    def close(self):
        if self._h:
            lib().plan_lis_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Catalogue:
    def __init__(self, h):
        self._h = h

    def __len__(self):
        return int(lib().plan_catalogue_count(self._h))

    def clumps(self) -> list[dict]:
        out = []
        ci = ClumpInfo()
        for i in range(len(self)):
            lib().plan_catalogue_get(self._h, i, C.byref(ci))
            out.append(dict(peak_id=ci.peak_id, npar=ci.npar, total_mass=ci.total_mass, hill_radius=ci.hill_radius,
                            com=tuple(ci.com), vel_com=tuple(ci.vel_com), J=tuple(ci.J)))
        return out

    def summary(self) -> str:
        return lib().plan_catalogue_summary(self._h).decode()

    def write_peaks(self, out_path: str, save_clumps: bool = False, file_number: int = 0, sampling: int = 1) -> None:
        rc = lib().plan_catalogue_write_peaks(self._h, str(out_path).encode(), int(save_clumps), int(file_number), int(sampling))
        if rc:
            raise PlanError(rc, f"writing peaks next to {out_path}")

    def basic_results(self, p: Params, with_header: bool) -> str:
        buf = C.create_string_buffer(4096)
        n = lib().plan_catalogue_basic_results(self._h, C.byref(p), int(with_header), buf, len(buf))
        if n < 0:
            raise PlanError(2, "basic results line")
        return buf.value.decode()

    def close(self):
        if self._h:
            lib().plan_catalogue_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Finder:
    """One device context (BHtree + PlanetesimalList of the reference, on one GPU)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = lib().plan_ctx_create(int(device), C.byref(h))
        if rc:
            raise PlanError(rc, "no usable CUDA device (there is no CPU path)")
        self._h = h

    def error(self) -> str:
        return lib().plan_last_error(self._h).decode()

    def build_tree(self, snap: Snapshot, p: Params, first_file: bool = True, stream: int | None = None) -> None:
        rc = lib().plan_build_tree(self._h, C.byref(snap.view), C.byref(p), int(first_file), C.c_void_p(stream or 0))
        if rc:
            raise PlanError(rc, self.error())

    def find_planetesimals(self, p: Params, stream: int | None = None) -> Catalogue:
        h = C.c_void_p()
        rc = lib().plan_find_planetesimals(self._h, C.byref(p), C.c_void_p(stream or 0), C.byref(h))
        if rc:
            raise PlanError(rc, self.error())
        return Catalogue(h)

    def find_clumps(self, snap: Snapshot, p: Params, first_file: bool = True, stream: int | None = None) -> Catalogue:
        h = C.c_void_p()
        rc = lib().plan_find_clumps(self._h, C.byref(snap.view), C.byref(p), int(first_file), C.c_void_p(stream or 0), C.byref(h))
        if rc:
            raise PlanError(rc, self.error())
        return Catalogue(h)

    _ELEM = {PLAN_ARR_TREE_POS: (np.float64, 4), PLAN_ARR_TREE_VEL: (np.float64, 4), PLAN_ARR_DENSITY: (np.float64, 1),
             PLAN_ARR_ORIG_ID: (np.uint32, 1), PLAN_ARR_KEYS: (np.uint32, 3), PLAN_ARR_NODE_F: (np.float64, 4),
             PLAN_ARR_NODE_U: (np.uint32, 7), PLAN_ARR_DENSEST: (np.uint32, 1), PLAN_ARR_PEAK: (np.uint32, 1),
             PLAN_ARR_SINK_COUNT: (np.uint32, 1)}

    def stage(self, which: int) -> np.ndarray:
        n = int(lib().plan_stage_count(self._h, which))
        dt, w = self._ELEM[which]
        a = np.empty((n, w) if w > 1 else n, dtype=dt)
        if n:
            rc = lib().plan_stage_copy(self._h, which, a.ctypes.data, a.nbytes)
            if rc:
                raise PlanError(rc, self.error())
        return a

    def knn(self, pos: np.ndarray, k: int, est: float = 0.0) -> tuple[np.ndarray, np.ndarray]:
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        nq = pos.shape[0]
        idx = np.empty((nq, k), dtype=np.uint32)
        dr2 = np.empty((nq, k), dtype=np.float64)
        rc = lib().plan_knn(self._h, pos.ctypes.data_as(C.POINTER(C.c_double)), nq, int(k), float(est),
                            idx.ctypes.data_as(C.POINTER(C.c_uint32)), dr2.ctypes.data_as(C.POINTER(C.c_double)))
        if rc:
            raise PlanError(rc, self.error())
        return idx, dr2

    def morton_order(self, keys3: np.ndarray) -> np.ndarray:
        """Input indices in std::sort order of 96-bit keys (reference comparator)."""
        k = np.ascontiguousarray(keys3, dtype=np.uint32).reshape(-1, 3)
        out = np.empty(len(k), dtype=np.uint32)
        rc = lib().plan_morton_order(self._h, k.ctypes.data, len(k), out.ctypes.data)
        if rc:
            raise PlanError(rc, self.error())
        return out

    def group_energies(self, pos, vel, mass, offsets, p: Params):
        """Kinetic and potential energy of each group [offsets[g], offsets[g+1]) (float32 inputs);
        returns (e_kin, e_pot, coincident pairs left out)."""
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        mass = np.ascontiguousarray(mass, dtype=np.float32)
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        ng = len(off) - 1
        ek, ep = np.zeros(ng), np.zeros(ng)
        z = C.c_uint64()
        rc = lib().plan_group_energies(self._h, pos.ctypes.data, vel.ctypes.data, mass.ctypes.data, off.ctypes.data, ng, C.byref(p),
                                       ek.ctypes.data, ep.ctypes.data, C.byref(z))
        if rc:
            raise PlanError(rc, self.error())
        return ek, ep, int(z.value)

    def density_vs_scale(self, p: Params, time: float):
        """--Density_Vs_Scale on the tree of the last build_tree, which must have run with
        p.density_vs_scale = 1: (radii, densities), one per length scale."""
        radii = np.zeros(32)
        rho = np.zeros(32)
        nlev = C.c_int32()
        rc = lib().plan_density_vs_scale(self._h, C.byref(p), float(time), radii.ctypes.data_as(C.POINTER(C.c_double)),
                                         rho.ctypes.data_as(C.POINTER(C.c_double)), 32, C.byref(nlev))
        if rc:
            raise PlanError(rc, self.error())
        return radii[:nlev.value].copy(), rho[:nlev.value].copy()

    def write_parlists(self, cat: "Catalogue", file_number: int = 0, sampling: int = 1) -> None:
        """The --Save_Clumps member lists of cat (ParList.<NNNN>/ in the working directory),
        formatted on this context's device."""
        rc = lib().plan_catalogue_write_parlists(self._h, cat._h, int(file_number), int(sampling))
        if rc:
            raise PlanError(rc, self.error())

    def morton_order_noalloc(self, keys3: np.ndarray) -> np.ndarray:
        """morton_order without device allocation (at most PLAN_NOALLOC_SORT_MAX keys)."""
        k = np.ascontiguousarray(keys3, dtype=np.uint32).reshape(-1, 3)
        out = np.empty(len(k), dtype=np.uint32)
        rc = lib().plan_morton_order_noalloc(self._h, k.ctypes.data, len(k), out.ctypes.data)
        if rc:
            raise PlanError(rc, self.error())
        return out

    def stage_times(self) -> np.ndarray:
        a = np.zeros(32)
        lib().plan_stage_times(self._h, a.ctypes.data_as(C.POINTER(C.c_double)), 32)
        return a

    def counters(self) -> np.ndarray:
        a = np.zeros(32, dtype=np.uint64)
        lib().plan_counters(self._h, a.ctypes.data_as(C.POINTER(C.c_uint64)), 32)
        return a

    def kernel_launches(self) -> int:
        return int(lib().plan_kernel_launches(self._h))

    def close(self):
        if self._h:
            lib().plan_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


PLAN_PENDING = 9


class Server:
    """The serving loop (plan_server_*): snapshots submitted here run concurrently on one
    device over `workers` contexts, admitted by device footprint against `hbm_budget` bytes
    (0 = 90% of the free memory). Keep each Snapshot alive until its request is polled."""

    def __init__(self, device: int = 0, workers: int = 2, hbm_budget: int = 0):
        h = C.c_void_p()
        rc = lib().plan_server_create(int(device), int(workers), int(hbm_budget), C.byref(h))
        if rc:
            raise PlanError(rc, "creating the serving loop")
        self._h = h
        self._params = {}  # request -> Params copy kept alive with the request

    def submit(self, snap: Snapshot, p: Params, first_file: bool = True) -> int:
        rid = C.c_uint64()
        rc = lib().plan_submit(self._h, C.byref(snap.view), C.byref(p), int(first_file), C.byref(rid))
        if rc:
            raise PlanError(rc, self.error())
        return int(rid.value)

    def poll(self, request: int, wait: bool = False):
        """(Catalogue, latency in ms) when done, None while queued or running."""
        h = C.c_void_p()
        lat = C.c_double()
        rc = lib().plan_poll(self._h, int(request), int(wait), C.byref(h), C.byref(lat))
        if rc == PLAN_PENDING:
            return None
        if rc:
            raise PlanError(rc, self.error())
        return Catalogue(h), float(lat.value)

    def error(self) -> str:
        return lib().plan_server_error(self._h).decode()

    def stats(self) -> dict:
        peak, rel = C.c_uint64(), C.c_uint64()
        lib().plan_server_stats(self._h, C.byref(peak), C.byref(rel))
        busy, both = C.c_double(), C.c_double()
        lib().plan_server_overlap(self._h, C.byref(busy), C.byref(both))
        return {"peak_held_bytes": int(peak.value), "releases": int(rel.value), "busy_ms": float(busy.value),
                "overlap_ms": float(both.value)}

    def close(self):
        if self._h:
            lib().plan_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
