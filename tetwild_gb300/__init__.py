"""tetwild_gb300 -- GB300 (sm_103a) kernels for TetWild's mesh-optimisation
query path, behind a C-ABI (include/tw_gb300.h).

``Context`` is a thin ctypes binding of that ABI (numpy in, numpy out);
``LocalOperations`` and ``VertexSmoother`` mirror the reference classes'
method names (LocalOperations.h:69-111, VertexSmoother.h:28-30) over it.

There is no CPU fallback: if libtw_gb300.so is missing or no GPU is present,
every call raises.
"""
from __future__ import annotations

import ctypes
import struct
from pathlib import Path

import numpy as np

__all__ = [
    "Context", "LocalOperations", "VertexSmoother", "TetWildGpuError", "load_library",
    "library_path", "TW_OK", "TW_NEEDS_EXACT_HOST", "TW_ENERGY_RAW", "TW_ENERGY_QUALITY",
    "TW_SURFACE_INPUT", "TW_SURFACE_BOUNDARY", "MAX_ENERGY", "EXPORTED_SYMBOLS",
]

TW_OK = 0
TW_NEEDS_EXACT_HOST = 1
TW_ERR_ARG = -1
TW_ERR_CUDA = -2
TW_ERR_OOM = -3
TW_ERR_NO_SURFACE = -4
TW_ERR_NO_MESH = -5
TW_ERR_TIMEOUT = -6
TW_ERR_TOO_LARGE = -7
TW_ERR_CANCELLED = -8
TW_OP_SPLIT = 0
TW_OP_COLLAPSE = 1
TW_ENERGY_RAW = 0
TW_ENERGY_QUALITY = 1
TW_SURFACE_INPUT = 0
TW_SURFACE_BOUNDARY = 1
TW_BUSY = 2
TW_REQ_POINTS = 0
TW_REQ_FACES = 1
TW_REQ_AMIPS = 2
TW_REQ_SMOOTH = 3
TW_REQ_RAW = 1
TW_REQ_APPLY = 2
TW_CV_V1_SURFACE = 1
TW_CV_V1_BOUNDARY = 2
TW_CV_V2_SURFACE = 4
TW_CV_V2_BOUNDARY = 8
TW_CV_V1_UNROUNDED = 16
TW_STAR_INTERIOR = 0
TW_STAR_SURFACE = 1
TW_STAR_BOUNDARY = 2
TW_SMOOTH_INVALID = 0
TW_SMOOTH_NOT_MOVED = 1
TW_SMOOTH_MOVED = 2
TW_SMOOTH_REJECT_FLIP = 3
TW_SMOOTH_REJECT_QUALITY = 4
TW_SMOOTH_REJECT_ENVELOPE = 5
MAX_ENERGY = 1e50  # State.h:29

_PKG = Path(__file__).resolve().parent


def library_path() -> Path:
    return _PKG / "libtw_gb300.so"


class TetWildGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tw error {code}: {msg}")
        self.code = code


_P = ctypes.c_void_p
_I = ctypes.c_int
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double
_SZ = ctypes.c_size_t

TW_PRECISION_FP64 = 0
TW_PRECISION_FP32_CERTIFIED = 1
TW_ENERGY_FORM_REFERENCE = 0
TW_ENERGY_FORM_CLOSED = 1
TW_COLLAPSE_SUCCESS = 0
TW_COLLAPSE_FLIP = 1
TW_COLLAPSE_QUALITY = 2
TW_COLLAPSE_ENVELOP = 3
TW_SWAP_SUCCESS = 0
TW_SWAP_FLIP = 1
TW_SWAP_QUALITY = 2
TW_SWAP_SIZE = 3
TW_SWAP_NEEDS_HOST = 4
TW_NEWTON_SHAPES = 10
TW_NOALLOC_MAX_TETS = 65536

_STAT_FIELDS = ("exact_orientations", "env_queries", "env_facet_tests", "env_facet_fp64",
                "amips_tets", "amips_fp64", "env_warp_fallbacks")


class TwStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in _STAT_FIELDS]


# name -> argtypes (restype int unless noted)
class TwRequest(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("flags", ctypes.c_int32), ("n", ctypes.c_int64),
                ("in0", ctypes.c_void_p), ("in1", ctypes.c_void_p), ("in2", ctypes.c_void_p),
                ("in3", ctypes.c_void_p), ("in4", ctypes.c_void_p), ("out0", ctypes.c_void_p),
                ("out1", ctypes.c_void_p), ("out2", ctypes.c_void_p), ("out3", ctypes.c_void_p)]


class TwServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("jobs_open", "bytes_used", "budget", "requests_done",
                                               "batches", "queries_done",
                                               "max_requests_per_batch")]


_SIGS = {
    "tw_set_precision": [_P, _I],
    "tw_set_energy_form": [_P, _I],
    "tw_get_stats": [_P, ctypes.POINTER(TwStats)],
    "tw_reset_stats": [_P],
    "tw_ctx_create": [_I, _SZ, ctypes.POINTER(_P)],
    "tw_ctx_destroy": [_P],
    "tw_last_error": [_P],
    "tw_set_params": [_P, _D, _D, _I, _I],
    "tw_stream": [_P, ctypes.POINTER(_P)],
    "tw_synchronize": [_P],
    "tw_memory_used": [_P, ctypes.POINTER(_SZ)],
    "tw_amips_soa": [_P, _P, _I64, _I, _P, _P, _P, _P],
    "tw_amips_soa_device": [_P, _P, _I64, _I, _P, _P, _P, _P],
    "tw_amips_soa_noalloc": [_P, _I64, _I, _P, _P, _P, _P, _P],
    "tw_mesh_upload": [_P, _P, _I32, _P],
    "tw_mesh_update_vertices": [_P, _P, _P, _P, _I32],
    "tw_tet_quality": [_P, _P, _I64, _P, _P, _P],
    "tw_tet_quality_device": [_P, _P, _I64, _P, _P, _P],
    "tw_surface_upload": [_P, _P, _I32, _P, _I32, _I],
    "tw_envelope_points": [_P, _P, _I64, _I, _P],
    "tw_envelope_points_device": [_P, _P, _I64, _I, _P],
    "tw_envelope_faces": [_P, _P, _I64, _P],
    "tw_envelope_faces_device": [_P, _P, _I64, _P],
    "tw_sample_triangle": [_P, _P, _D, _P, _I64, ctypes.POINTER(_I64)],
    "tw_newton_stars": [_P, _P, _P, _P, _I32, _P, _P],
    "tw_newton_stars_device": [_P, _P, _P, _P, _I32, _P, _P],
    "tw_set_newton_shape": [_P, _I],
    "tw_set_tuning": [_P, _I, _D],
    "tw_kernel_times": [_P, _P, _I, ctypes.POINTER(_I)],
    "tw_nearest_points": [_P, _P, _I64, _I, _P, _P, _P],
    "tw_nearest_points_device": [_P, _P, _I64, _I, _P, _P, _P],
    "tw_smooth_stars": [_P, _P, _P, _P, _P, _P, _I32, _P, _P],
    "tw_collapse_check": [_P, _P, _P, _P, _P, _P, _I32, _I, _D, _P],
    "tw_energy_stats": [_P, _P, _I64, _P, _D, _P, _P, _P, _P],
    "tw_dihedral_stats": [_P, _P, _I64, _P, _P, _P, _P, _P],
    "tw_filter_energy": [_P, _D, _P],
    "tw_smooth_stars_device": [_P, _P, _P, _P, _P, _P, _I32, _I64, _P, _P],
    "tw_smooth_autotune_device": [_P, _P, _P, _P, _P, _P, _I32, _I64, _P, _P, ctypes.POINTER(_I),
                                  ctypes.POINTER(ctypes.c_float)],
    "tw_newton_autotune_device": [_P, _P, _P, _P, _I32, _P, _P, ctypes.POINTER(_I),
                                  ctypes.POINTER(ctypes.c_float)],
    "tw_capture_begin": [_P],
    "tw_capture_end": [_P, ctypes.POINTER(_P)],
    "tw_graph_launch": [_P, _P],
    "tw_graph_destroy": [_P],
    "tw_host_alloc": [_SZ, ctypes.POINTER(_P)],
    "tw_host_free": [_P],
    "tw_probe_peaks": [_P, ctypes.POINTER(_D), ctypes.POINTER(_D)],
    "tw_self_test": [_P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)],
    "tw_self_test_wait": [_P, _I32, ctypes.POINTER(ctypes.c_uint64)],
    "tw_server_create": [_I, _SZ, _I, ctypes.POINTER(_P)],
    "tw_server_destroy": [_P],
    "tw_server_last_error": [_P],
    "tw_server_set_params": [_P, _I, _I, _I, _I],
    "tw_server_job_open": [_P, _P, _I32, _P, _I32, _D, _D, ctypes.POINTER(_I32)],
    "tw_server_job_boundary": [_P, _I32, _P, _I32, _P, _I32],
    "tw_server_job_mesh": [_P, _I32, _P, _I32, _D],
    "tw_server_job_read_mesh": [_P, _I32, _P, _D],
    "tw_server_job_close": [_P, _I32, _D],
    "tw_server_job_cancel": [_P, _I32, _D],
    "tw_swap_check": [_P, _P, _P, _P, _P, _I32, _P, _P, _P],
    "tw_schedule_edges": [_P, _P, _I32, _P, _D, _I, _P, _I32, _P, _P],
    "tw_server_submit": [_P, _I32, ctypes.POINTER(TwRequest), ctypes.POINTER(ctypes.c_uint64)],
    "tw_server_wait": [_P, ctypes.c_uint64, _D, ctypes.POINTER(_D)],
    "tw_server_get_stats": [_P, ctypes.POINTER(TwServerStats)],
}
EXPORTED_SYMBOLS = tuple(_SIGS)

_LIB = None


def load_library() -> ctypes.CDLL:
    """Load libtw_gb300.so (built in-tree by tetwild_gb300/build.py)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        raise TetWildGpuError(TW_ERR_CUDA, f"{path} is not built; run __graft_entry__.build()")
    lib = ctypes.CDLL(str(path))
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = (ctypes.c_char_p if name.endswith("last_error")
                      else _D if name == "tw_filter_energy" else _I)
    _LIB = lib
    return lib


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    return a.ctypes.data


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class Context:
    """One device context: surfaces, resident mesh, scratch and streams."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = load_library()
        h = _P()
        st = self.lib.tw_ctx_create(device, hbm_budget_bytes, ctypes.byref(h))
        if st != TW_OK:
            raise TetWildGpuError(st, "tw_ctx_create failed (no usable CUDA device?)")
        self.h = h
        self.device = device
        self.eps_2 = 0.0
        self.sampling_dist = 0.0

    def close(self):
        if getattr(self, "h", None):
            self.lib.tw_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, allow=(TW_OK,)):
        if st not in allow:
            msg = self.lib.tw_last_error(self.h)
            raise TetWildGpuError(st, msg.decode() if msg else "")
        return st

    # -- params / streams -------------------------------------------------------
    def set_params(self, eps_2: float, sampling_dist: float, newton_max_step: int = 15,
                   newton_max_it: int = 20):
        self._check(self.lib.tw_set_params(self.h, eps_2, sampling_dist, newton_max_step,
                                           newton_max_it))
        self.eps_2 = eps_2
        self.sampling_dist = sampling_dist

    def stream(self) -> int:
        s = _P()
        self._check(self.lib.tw_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def synchronize(self):
        self._check(self.lib.tw_synchronize(self.h))

    def memory_used(self) -> int:
        b = _SZ()
        self._check(self.lib.tw_memory_used(self.h, ctypes.byref(b)))
        return b.value

    def set_precision(self, mode: int):
        """TW_PRECISION_FP64 or TW_PRECISION_FP32_CERTIFIED (same decisions)."""
        self._check(self.lib.tw_set_precision(self.h, mode))

    def set_energy_form(self, form: int):
        """TW_ENERGY_FORM_REFERENCE (default: the reference's own operations, in
        its order) or TW_ENERGY_FORM_CLOSED (the accurate closed form)."""
        self._check(self.lib.tw_set_energy_form(self.h, form))

    def stats(self) -> dict:
        s = TwStats()
        self._check(self.lib.tw_get_stats(self.h, ctypes.byref(s)))
        return {f: int(getattr(s, f)) for f in _STAT_FIELDS}

    def reset_stats(self):
        self._check(self.lib.tw_reset_stats(self.h))

    # -- AMIPS --------------------------------------------------------------------
    def amips(self, T_soa, mode=TW_ENERGY_QUALITY, energy=True, jacobian=True, hessian=True,
              flip=True):
        """T_soa: [12, n] float64.  Returns dict of E [n], J [3,n], H [9,n], flip [n]."""
        T = _c(T_soa, np.float64)
        if T.ndim != 2 or T.shape[0] != 12:
            raise ValueError("T_soa must have shape [12, n]")
        n = T.shape[1]
        out = {}
        E = np.empty(n) if energy else None
        J = np.empty((3, n)) if jacobian else None
        H = np.empty((9, n)) if hessian else None
        F = np.empty(n, np.uint8) if flip else None
        self._check(self.lib.tw_amips_soa(self.h, _ptr(T), n, mode, _ptr(E), _ptr(J), _ptr(H),
                                          _ptr(F)))
        if energy:
            out["E"] = E
        if jacobian:
            out["J"] = J
        if hessian:
            out["H"] = H
        if flip:
            out["flip"] = F
        return out

    def amips_device(self, T_ptr: int, n: int, mode: int, E_ptr, J_ptr, H_ptr, flip_ptr):
        """Device-pointer variant; asynchronous on the context stream."""
        self._check(self.lib.tw_amips_soa_device(self.h, T_ptr, n, mode, E_ptr, J_ptr, H_ptr,
                                                 flip_ptr))

    # -- resident mesh -------------------------------------------------------------
    def mesh_upload(self, xyz, rounded=None):
        X = _c(xyz, np.float64).reshape(-1, 3)
        R = None if rounded is None else _c(rounded, np.uint8)
        self._check(self.lib.tw_mesh_upload(self.h, _ptr(X), X.shape[0], _ptr(R)))

    def mesh_update_vertices(self, ids, xyz, rounded=None):
        I = _c(ids, np.int32)
        X = _c(xyz, np.float64).reshape(-1, 3)
        R = None if rounded is None else _c(rounded, np.uint8)
        self._check(self.lib.tw_mesh_update_vertices(self.h, _ptr(I), _ptr(X), _ptr(R), I.size))

    def tet_quality(self, tets):
        """Returns (energy [n], flip [n], needs_host [n], status)."""
        T = _c(tets, np.int32).reshape(-1, 4)
        n = T.shape[0]
        E = np.empty(n)
        F = np.empty(n, np.uint8)
        N = np.empty(n, np.uint8)
        st = self._check(self.lib.tw_tet_quality(self.h, _ptr(T), n, _ptr(E), _ptr(F), _ptr(N)),
                         allow=(TW_OK, TW_NEEDS_EXACT_HOST))
        return E, F, N, st

    # -- envelope --------------------------------------------------------------------
    def surface_upload(self, V, F, which=TW_SURFACE_INPUT):
        Vv = _c(V, np.float64).reshape(-1, 3)
        Ff = _c(F, np.int32).reshape(-1, 3)
        self._check(self.lib.tw_surface_upload(self.h, _ptr(Vv), Vv.shape[0], _ptr(Ff),
                                               Ff.shape[0], which))

    def envelope_points(self, P, which=TW_SURFACE_INPUT):
        X = _c(P, np.float64).reshape(-1, 3)
        out = np.empty(X.shape[0], np.uint8)
        self._check(self.lib.tw_envelope_points(self.h, _ptr(X), X.shape[0], which, _ptr(out)))
        return out

    def envelope_points_device(self, P_ptr: int, n: int, out_ptr: int, which=TW_SURFACE_INPUT):
        self._check(self.lib.tw_envelope_points_device(self.h, P_ptr, n, which, out_ptr))

    def envelope_faces(self, tris):
        X = _c(tris, np.float64).reshape(-1, 9)
        out = np.empty(X.shape[0], np.uint8)
        self._check(self.lib.tw_envelope_faces(self.h, _ptr(X), X.shape[0], _ptr(out)))
        return out

    def envelope_faces_device(self, tris_ptr: int, n: int, out_ptr: int):
        self._check(self.lib.tw_envelope_faces_device(self.h, tris_ptr, n, out_ptr))

    def sample_triangle(self, tri9, sampling_dist, cap=1 << 20):
        t = _c(tri9, np.float64).reshape(9)
        out = np.empty((cap, 3))
        cnt = _I64()
        self._check(self.lib.tw_sample_triangle(self.h, _ptr(t), sampling_dist, _ptr(out), cap,
                                                ctypes.byref(cnt)))
        return out[: min(cnt.value, cap)].copy(), cnt.value

    # -- Newton -----------------------------------------------------------------------
    def newton_stars(self, star_off, tets, centers):
        O = _c(star_off, np.int32)
        T = _c(tets, np.int32).reshape(-1, 4)
        C = _c(centers, np.int32)
        ns = C.size
        out = np.empty((ns, 3))
        moved = np.empty(ns, np.uint8)
        self._check(self.lib.tw_newton_stars(self.h, _ptr(O), _ptr(T), _ptr(C), ns, _ptr(out),
                                             _ptr(moved)))
        return out, moved

    def newton_stars_device(self, off_ptr: int, tets_ptr: int, centers_ptr: int, nstars: int,
                            out_ptr: int, moved_ptr: int):
        """Device-pointer variant; asynchronous on the context stream."""
        self._check(self.lib.tw_newton_stars_device(self.h, off_ptr, tets_ptr, centers_ptr, nstars,
                                                    out_ptr, moved_ptr))

    NEWTON_SHAPES = 10
    TUNE_GRID_CELL = 0
    TUNE_SORT_POINTS = 1
    TUNE_TIME_KERNELS = 2
    TUNE_POINT_BLOCK = 3
    TUNE_BIN_CELL = 4

    def set_tuning(self, knob: int, value: float):
        """Work-only knobs (TW_TUNE_*): results are the same for every value."""
        self._check(self.lib.tw_set_tuning(self.h, knob, value))

    def kernel_times(self, max_n: int = 64):
        """Durations (ms) of the point-envelope kernel launches recorded since the last call."""
        ms = np.zeros(max_n, np.float32)
        cnt = _I()
        self._check(self.lib.tw_kernel_times(self.h, _ptr(ms), max_n, ctypes.byref(cnt)))
        return ms[:cnt.value].astype(float).tolist()

    # -- smoothing pass ------------------------------------------------------------------
    def smooth_stars(self, star_off, tets, centers, face_flags=None, kinds=None):
        """One smoothing pass (smoothSingle / smoothSurface bodies) over independent stars.
        Returns (positions [ns,3], status [ns] TW_SMOOTH_*)."""
        O = _c(star_off, np.int32)
        T = _c(tets, np.int32).reshape(-1, 4)
        C = _c(centers, np.int32)
        FF = None if face_flags is None else _c(face_flags, np.uint8)
        K = None if kinds is None else _c(kinds, np.uint8)
        ns = C.size
        out = np.empty((ns, 3))
        st = np.empty(ns, np.uint8)
        self._check(self.lib.tw_smooth_stars(self.h, _ptr(O), _ptr(T), _ptr(FF), _ptr(C), _ptr(K),
                                             ns, _ptr(out), _ptr(st)))
        return out, st

    def smooth_stars_device(self, off_ptr: int, tets_ptr: int, ff_ptr, centers_ptr: int, kinds_ptr,
                            nstars: int, ntets: int, out_ptr: int, status_ptr: int):
        """Device-pointer variant; asynchronous on the context stream."""
        self._check(self.lib.tw_smooth_stars_device(self.h, off_ptr, tets_ptr, ff_ptr, centers_ptr,
                                                    kinds_ptr, nstars, ntets, out_ptr, status_ptr))

    def smooth_autotune_device(self, off_ptr: int, tets_ptr: int, ff_ptr, centers_ptr: int,
                               kinds_ptr, nstars: int, ntets: int, out_ptr: int, status_ptr: int):
        """Times the pass for every launch shape on this batch; returns (best, ms per shape)."""
        best = _I()
        ms = (ctypes.c_float * self.NEWTON_SHAPES)()
        self._check(self.lib.tw_smooth_autotune_device(self.h, off_ptr, tets_ptr, ff_ptr,
                                                       centers_ptr, kinds_ptr, nstars, ntets,
                                                       out_ptr, status_ptr, ctypes.byref(best), ms))
        return int(best.value), [float(x) for x in ms]

    # -- energy sweeps -------------------------------------------------------------------
    def energy_stats(self, tets, locked=None, filter_energy_thres=10.0):
        """(avg, max, second max, buckets[11]) over tets of the resident mesh."""
        T = _c(tets, np.int32).reshape(-1, 4)
        L = None if locked is None else _c(locked, np.uint8)
        a, m, m2 = _D(), _D(), _D()
        b = np.zeros(11, np.int64)
        self._check(self.lib.tw_energy_stats(self.h, _ptr(T), T.shape[0], _ptr(L),
                                             filter_energy_thres, ctypes.byref(a), ctypes.byref(m),
                                             ctypes.byref(m2), _ptr(b)))
        return a.value, m.value, m2.value, b

    def dihedral_stats(self, tets, locked=None, per_tet=False):
        """calTetQuality_AD over tets of the resident mesh and outputInfo's statistics:
        (out[4] = min, mean min, max, mean max; counts[7]; per-tet mins, maxs or None)."""
        T = _c(tets, np.int32).reshape(-1, 4)
        L = None if locked is None else _c(locked, np.uint8)
        n = T.shape[0]
        out = np.zeros(4)
        cnt = np.zeros(7, np.int64)
        mins = np.empty(n) if per_tet else None
        maxs = np.empty(n) if per_tet else None
        self._check(self.lib.tw_dihedral_stats(self.h, _ptr(T), n, _ptr(L), _ptr(out), _ptr(cnt),
                                               _ptr(mins), _ptr(maxs)))
        return out, cnt, mins, maxs

    def filter_energy(self, buckets, filter_energy_thres=10.0):
        b = _c(buckets, np.int64)
        c = _I()
        e = self.lib.tw_filter_energy(_ptr(b), filter_energy_thres, ctypes.byref(c))
        return e, bool(c.value)

    # -- edge-collapse checks -----------------------------------------------------------
    def collapse_check(self, v12, flags, star_off, tets, face_flags, check_quality=True,
                       soft_energy=-1.0):
        """Checks of candidate collapses (EdgeCollapser::collapseAnEdge): codes [n]."""
        V = _c(v12, np.int32).reshape(-1, 2)
        FL = _c(flags, np.uint8)
        O = _c(star_off, np.int32)
        T = _c(tets, np.int32).reshape(-1, 4)
        FF = _c(face_flags, np.uint8)
        n = V.shape[0]
        out = np.empty(n, np.uint8)
        self._check(self.lib.tw_collapse_check(self.h, _ptr(V), _ptr(FL), _ptr(O), _ptr(T),
                                               _ptr(FF), n, 1 if check_quality else 0,
                                               soft_energy, _ptr(out)))
        return out

    def swap_check(self, v12, shell_off, tets, budget=None):
        """Checks of candidate edge removals (EdgeRemover::removeAnEdge_32 / _44 / _56):
        (result, config, spent) [n]; TW_NEEDS_EXACT_HOST is allowed (result 4 marks them)."""
        V = _c(v12, np.int32).reshape(-1, 2)
        O = _c(shell_off, np.int32)
        T = _c(tets, np.int32).reshape(-1, 4)
        B = None if budget is None else _c(budget, np.int32)
        n = V.shape[0]
        res = np.empty(n, np.uint8)
        cfg = np.empty(n, np.int8)
        sp = np.empty(n, np.uint8)
        self._check(self.lib.tw_swap_check(self.h, _ptr(V), _ptr(O), _ptr(T), _ptr(B), n,
                                           _ptr(res), _ptr(cfg), _ptr(sp)),
                    allow=(TW_OK, TW_NEEDS_EXACT_HOST))
        return res, cfg, sp

    def schedule_edges(self, tets, op, ideal_weight, scale=None):
        """Operator candidates of the tet list and their conflict-free batch, on the device
        (tw_schedule_edges): ((v1, v2) chosen [m, 2] in priority order, number of
        candidates)."""
        T = _c(tets, np.int32).reshape(-1, 4)
        S = None if scale is None else _c(scale, np.float64)
        cap = max(1, T.shape[0])
        out = np.empty((cap, 2), np.int32)
        ns, nc = _I32(), _I32()
        self._check(self.lib.tw_schedule_edges(self.h, _ptr(T), T.shape[0], _ptr(S), ideal_weight,
                                               op, _ptr(out), cap, ctypes.byref(ns),
                                               ctypes.byref(nc)))
        return out[:min(ns.value, cap)].copy(), nc.value

    # -- nearest facet -----------------------------------------------------------------
    def nearest_points(self, P, which=TW_SURFACE_INPUT):
        """(closest points [n,3], squared distances [n], input facet ids [n])."""
        X = _c(P, np.float64).reshape(-1, 3)
        n = X.shape[0]
        Q = np.empty((n, 3))
        D = np.empty(n)
        F = np.empty(n, np.int32)
        self._check(self.lib.tw_nearest_points(self.h, _ptr(X), n, which, _ptr(Q), _ptr(D),
                                               _ptr(F)))
        return Q, D, F

    def nearest_points_device(self, P_ptr: int, n: int, Q_ptr, D_ptr, F_ptr,
                              which=TW_SURFACE_INPUT):
        self._check(self.lib.tw_nearest_points_device(self.h, P_ptr, n, which, Q_ptr, D_ptr,
                                                      F_ptr))

    def set_newton_shape(self, shape: int):
        self._check(self.lib.tw_set_newton_shape(self.h, shape))

    def newton_autotune_device(self, off_ptr: int, tets_ptr: int, centers_ptr: int, nstars: int,
                               out_ptr: int, moved_ptr: int):
        """Times every launch shape on this batch; returns (best shape, ms per shape)."""
        best = _I()
        ms = (ctypes.c_float * self.NEWTON_SHAPES)()
        self._check(self.lib.tw_newton_autotune_device(self.h, off_ptr, tets_ptr, centers_ptr,
                                                       nstars, out_ptr, moved_ptr,
                                                       ctypes.byref(best), ms))
        return int(best.value), [float(x) for x in ms]

    # -- CUDA graphs of the context stream ---------------------------------------------
    def capture_begin(self):
        self._check(self.lib.tw_capture_begin(self.h))

    def capture_end(self) -> "Graph":
        g = _P()
        self._check(self.lib.tw_capture_end(self.h, ctypes.byref(g)))
        return Graph(self, g.value)

    # -- misc ---------------------------------------------------------------------------
    def self_test(self, samples: int = 1 << 26):
        """(d2f_rn mismatches, f2d_exact mismatches) against the hardware conversions."""
        f = (ctypes.c_uint64 * 2)()
        self._check(self.lib.tw_self_test(self.h, samples, f))
        return int(f[0]), int(f[1])

    def self_test_wait(self, limit: int = 1 << 14):
        """The bulk kernel's bounded wait: {'timed_out', 'completed', 'cycles', 'copied'}."""
        r = (ctypes.c_uint64 * 4)()
        self._check(self.lib.tw_self_test_wait(self.h, limit, r))
        return {"timed_out": bool(r[0]), "completed": bool(r[1]), "cycles": int(r[2]),
                "copied": struct.unpack("<d", struct.pack("<Q", r[3]))[0]}

    def probe_peaks(self):
        a, b = _D(), _D()
        self._check(self.lib.tw_probe_peaks(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value


class PinnedArray:
    """numpy view of page-locked host memory (tw_host_alloc) for fast copies."""

    def __init__(self, shape, dtype):
        self.lib = load_library()
        dt = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dt.itemsize
        p = _P()
        st = self.lib.tw_host_alloc(max(nbytes, 16), ctypes.byref(p))
        if st != TW_OK:
            raise TetWildGpuError(st, "tw_host_alloc failed")
        self.p = p
        buf = (ctypes.c_char * max(nbytes, 16)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if getattr(self, "p", None):
            self.array = None
            self.lib.tw_host_free(self.p)
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class LocalOperations:
    """Mirror of the reference's LocalOperations query methods (LocalOperations.h:69-111)
    over a resident mesh and surface trees, batched.

    tet_vertices: [nv, 3] float64 (TetVertex::posf), rounded: [nv] (is_rounded).
    """

    def __init__(self, ctx: Context, tet_vertices, rounded=None):
        self.ctx = ctx
        self.ctx.mesh_upload(tet_vertices, rounded)

    # static AMIPS routines, batched over [n,12] tets (LocalOperations.h:109-111)
    def comformalAMIPSEnergy_new(self, T):
        T = np.atleast_2d(np.asarray(T, np.float64))
        return self.ctx.amips(T.T, TW_ENERGY_RAW, True, False, False, False)["E"]

    def comformalAMIPSJacobian_new(self, T):
        T = np.atleast_2d(np.asarray(T, np.float64))
        return self.ctx.amips(T.T, TW_ENERGY_RAW, False, True, False, False)["J"].T.copy()

    def comformalAMIPSHessian_new(self, T):
        T = np.atleast_2d(np.asarray(T, np.float64))
        return self.ctx.amips(T.T, TW_ENERGY_RAW, False, False, True, False)["H"].T.copy()

    def calTetQualities(self, new_tets):
        """slim_energy of each tet (LocalOperations.cpp:695-773)."""
        E, _, needs, st = self.ctx.tet_quality(new_tets)
        if st == TW_NEEDS_EXACT_HOST:
            raise TetWildGpuError(st, "tets with unrounded vertices need the host's exact path")
        return E

    def isFlip(self, new_tets) -> bool:
        """LocalOperations.cpp:559-573."""
        _, F, needs, st = self.ctx.tet_quality(new_tets)
        if st == TW_NEEDS_EXACT_HOST:
            raise TetWildGpuError(st, "tets with unrounded vertices need the host's exact path")
        return bool(F.any())

    def isTetFlip(self, t) -> bool:
        return self.isFlip([t])

    def isPointOutEnvelop(self, p) -> bool:
        return bool(self.ctx.envelope_points(np.asarray(p).reshape(1, 3), TW_SURFACE_INPUT)[0])

    def isPointOutBoundaryEnvelop(self, p) -> bool:
        return bool(self.ctx.envelope_points(np.asarray(p).reshape(1, 3), TW_SURFACE_BOUNDARY)[0])

    def isFaceOutEnvelop(self, tri) -> bool:
        return bool(self.ctx.envelope_faces(np.asarray(tri).reshape(1, 9))[0])

    # full-mesh sweeps over the live tets (LocalOperations.cpp:605-693, :783-860);
    # locked: isTetLocked_ui per tet
    def getAvgMaxEnergy(self, tets, locked=None):
        a, m, _, _ = self.ctx.energy_stats(tets, locked)
        return a, m

    def getMaxEnergy(self, tets, locked=None) -> float:
        return self.ctx.energy_stats(tets, locked)[1]

    def getSecondMaxEnergy(self, tets, locked=None) -> float:
        return self.ctx.energy_stats(tets, locked)[2]

    def getFilterEnergy(self, tets, filter_energy_thres=10.0):
        """(filter energy, is_clean_up); is_clean_up is set only by the first branch, as in
        the reference (False otherwise)."""
        b = self.ctx.energy_stats(tets, None, filter_energy_thres)[3]
        return self.ctx.filter_energy(b, filter_energy_thres)

    def calTetQuality_AD(self, tets):
        """(min_d_angle [n], max_d_angle [n]) of each tet, radians."""
        _, _, mins, maxs = self.ctx.dihedral_stats(tets, None, per_tet=True)
        return mins, maxs


class Server:
    """The serving loop (tw_server_*): many jobs resident in HBM, their query batches joined
    across jobs as they arrive and run on ``lanes`` CUDA streams."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, lanes: int = 4):
        self.lib = load_library()
        h = _P()
        st = self.lib.tw_server_create(device, hbm_budget_bytes, lanes, ctypes.byref(h))
        if st != TW_OK:
            raise TetWildGpuError(st, "tw_server_create failed")
        self.h = h
        self._keep = {}

    def _check(self, st, allow=(TW_OK,)):
        if st not in allow:
            msg = self.lib.tw_server_last_error(self.h)
            raise TetWildGpuError(st, msg.decode() if msg else "")
        return st

    def close(self):
        if getattr(self, "h", None):
            self.lib.tw_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_params(self, precision=TW_PRECISION_FP32_CERTIFIED, newton_max_step=15,
                   newton_max_it=20, newton_shape=5):
        self._check(self.lib.tw_server_set_params(self.h, precision, newton_max_step,
                                                  newton_max_it, newton_shape))

    def job_open(self, V, F, eps_2, sampling_dist):
        """Returns the job id, or None when the job does not fit in the budget now (TW_BUSY)."""
        Vv = _c(V, np.float64).reshape(-1, 3)
        Ff = _c(F, np.int32).reshape(-1, 3)
        j = _I32()
        st = self._check(self.lib.tw_server_job_open(self.h, _ptr(Vv), Vv.shape[0], _ptr(Ff),
                                                     Ff.shape[0], eps_2, sampling_dist,
                                                     ctypes.byref(j)), allow=(TW_OK, TW_BUSY))
        return None if st == TW_BUSY else int(j.value)

    def job_boundary(self, job, V, F):
        Vv = _c(V, np.float64).reshape(-1, 3)
        Ff = _c(F, np.int32).reshape(-1, 3)
        self._check(self.lib.tw_server_job_boundary(self.h, job, _ptr(Vv), Vv.shape[0], _ptr(Ff),
                                                    Ff.shape[0]))

    def job_mesh(self, job, xyz, timeout_s=60.0):
        X = _c(xyz, np.float64).reshape(-1, 3)
        self._check(self.lib.tw_server_job_mesh(self.h, job, _ptr(X), X.shape[0], timeout_s))

    def job_read_mesh(self, job, nv, timeout_s=60.0):
        out = np.empty((nv, 3))
        self._check(self.lib.tw_server_job_read_mesh(self.h, job, _ptr(out), timeout_s))
        return out

    def job_close(self, job, timeout_s=60.0):
        self._check(self.lib.tw_server_job_close(self.h, job, timeout_s))

    def job_cancel(self, job, timeout_s=60.0):
        """Cancels the job: queued requests end with TW_ERR_CANCELLED, batches on a lane
        finish, then its memory is freed."""
        self._check(self.lib.tw_server_job_cancel(self.h, job, timeout_s))

    def wait_status(self, ticket, timeout_s=60.0):
        """(status, latency ms) of a request without raising on its status."""
        lat = _D()
        st = self.lib.tw_server_wait(self.h, ticket, timeout_s, ctypes.byref(lat))
        if st != TW_ERR_TIMEOUT:
            self._keep.pop(ticket, None)
        return st, lat.value

    def _submit(self, job, req, keep):
        t = ctypes.c_uint64()
        self._check(self.lib.tw_server_submit(self.h, job, ctypes.byref(req), ctypes.byref(t)))
        self._keep[t.value] = keep
        return t.value

    def submit_points(self, job, P, out=None):
        X = _c(P, np.float64).reshape(-1, 3)
        out = np.empty(X.shape[0], np.uint8) if out is None else out
        r = TwRequest(TW_REQ_POINTS, 0, X.shape[0], _ptr(X), None, None, None, None, _ptr(out))
        return self._submit(job, r, (X, out)), out

    def submit_faces(self, job, tris, out=None):
        X = _c(tris, np.float64).reshape(-1, 9)
        out = np.empty(X.shape[0], np.uint8) if out is None else out
        r = TwRequest(TW_REQ_FACES, 0, X.shape[0], _ptr(X), None, None, None, None, _ptr(out))
        return self._submit(job, r, (X, out)), out

    def submit_amips(self, job, T_soa, raw=False, out=None, jacobian=True, hessian=True):
        """out: optional (E, J, H, flip) arrays; J / H may be None (not computed)."""
        T = _c(T_soa, np.float64)
        n = T.shape[1]
        if out is None:
            out = (np.empty(n), np.empty((3, n)) if jacobian else None,
                   np.empty((9, n)) if hessian else None, np.empty(n, np.uint8))
        E, J, H, Fl = out
        r = TwRequest(TW_REQ_AMIPS, TW_REQ_RAW if raw else 0, n, _ptr(T), None, None, None, None,
                      _ptr(E), _ptr(J), _ptr(H), _ptr(Fl))
        return self._submit(job, r, (T, E, J, H, Fl)), (E, J, H, Fl)

    def submit_smooth(self, job, star_off, tets, centers, face_flags=None, kinds=None,
                      apply=False, out=None):
        O = _c(star_off, np.int32)
        T = _c(tets, np.int32).reshape(-1, 4)
        C = _c(centers, np.int32)
        FF = None if face_flags is None else _c(face_flags, np.uint8)
        K = None if kinds is None else _c(kinds, np.uint8)
        ns = C.size
        out, st = (np.empty((ns, 3)), np.empty(ns, np.uint8)) if out is None else out
        r = TwRequest(TW_REQ_SMOOTH, TW_REQ_APPLY if apply else 0, ns, _ptr(O), _ptr(T), _ptr(FF),
                      _ptr(C), _ptr(K), _ptr(out), _ptr(st))
        return self._submit(job, r, (O, T, FF, C, K, out, st)), (out, st)

    def wait(self, ticket, timeout_s=60.0):
        """Returns the latency in ms (submit to completion); raises on a failed request."""
        lat = _D()
        st = self.lib.tw_server_wait(self.h, ticket, timeout_s, ctypes.byref(lat))
        if st == TW_ERR_TIMEOUT:
            raise TimeoutError(f"request {ticket} not done after {timeout_s} s")
        self._keep.pop(ticket, None)
        self._check(st)
        return lat.value

    def stats(self):
        s = TwServerStats()
        self._check(self.lib.tw_server_get_stats(self.h, ctypes.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in TwServerStats._fields_}


class Graph:
    """An executable CUDA graph captured from the context stream."""

    def __init__(self, ctx: Context, handle: int):
        self.ctx = ctx
        self.handle = handle

    def launch(self):
        self.ctx._check(self.ctx.lib.tw_graph_launch(self.ctx.h, self.handle))

    def close(self):
        if self.handle:
            self.ctx.lib.tw_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class VertexSmoother(LocalOperations):
    """Mirror of VertexSmoother::NewtonsMethod (VertexSmoother.cpp:465-542), batched over
    independent stars: star i is centre ``centers[i]`` with tets
    ``tets[star_off[i]:star_off[i+1]]`` in the caller's order."""

    def NewtonsMethod(self, star_off, tets, centers):
        return self.ctx.newton_stars(star_off, tets, centers)
