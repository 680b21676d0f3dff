"""ctypes wrappers for the CPU oracle (libtw_oracle.so) and for the
reference's own code compiled into oracle/_ref/libtwref.so.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference legs of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "libtw_oracle.so"
# the same source built with TW_RF_LIBM: the reference-form AMIPS routines take
# libm's pow as the reference does (the bit-for-bit pin against oracle/_ref)
ORACLE_LIBM_SO = HERE / "libtw_oracle_libm.so"
REF_SO = HERE / "_ref" / "libtwref.so"

_P = ctypes.c_void_p
_I = ctypes.c_int
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return ORACLE_SO


def _recipe():
    """oracle/ref/build_ref.py, the recipe that slices and compiles the reference."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("tw_build_ref", HERE / "ref" / "build_ref.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def build_ref() -> Path | None:
    """Slice (when the reference checkout is present) and compile oracle/_ref."""
    mod = _recipe()
    mod.do_slice()
    return mod.do_compile()


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)


class Oracle:
    """The CPU restatement (oracle/tw_oracle.c); libm=True loads its libm-pow
    build (libtw_oracle_libm.so)."""

    def __init__(self, libm: bool = False):
        so = ORACLE_LIBM_SO if libm else ORACLE_SO
        if not so.exists():
            build_oracle()
        L = ctypes.CDLL(str(so))
        sig = {
            "two_icbrt": ([_D], _D),
            "two_set_energy_form": ([_I], None),
            "two_get_energy_form": ([], _I),
            "two_rf_pow_m13": ([_D], _D),
            "two_amips_energy_rf": ([_P], _D),
            "two_amips_jacobian_rf": ([_P, _P], None),
            "two_amips_hessian_rf": ([_P, _P], None),
            "two_amips_energy": ([_P], _D),
            "two_amips_jacobian": ([_P, _P], None),
            "two_amips_hessian": ([_P, _P], None),
            "two_orient3d": ([_P, _P, _P, _P], _I),
            "two_orient3d_exact": ([_P, _P, _P, _P], _I),
            "two_collinear": ([_P, _P, _P], _I),
            "two_tet_quality": ([_P], _D),
            "two_tet_flip": ([_P], _I),
            "two_point_triangle_sqdist": ([_P, _P, _P, _P, _P], _D),
            "two_sample_triangle": ([_P, _D, _P, _I64], _I64),
            "two_sample_count": ([_P, _D], _I64),
            "two_surface_build": ([_P, _I32, _P, _I32], _P),
            "two_surface_free": ([_P], None),
            "two_point_out": ([_P, _P, _D], _I),
            "two_point_out_brute": ([_P, _P, _D], _I),
            "two_face_out": ([_P, _P, _D, _D], _I),
            "two_qr_solve3": ([_P, _P, _P], _I),
            "two_newton_star": ([_P, _P, _I32, _I32, _I, _I, _P], _I),
            "two_amips_batch_soa": ([_P, _I64, _I, _P, _P, _P, _P, _I], None),
            "two_points_out_batch": ([_P, _P, _I64, _D, _P, _I], None),
            "two_faces_out_batch": ([_P, _P, _I64, _D, _D, _P, _I], None),
            "two_newton_stars_batch": ([_P, _P, _P, _P, _I64, _I, _I, _P, _P, _I], None),
            "two_nearest_facet": ([_P, _P, _P, _P], _I32),
            "two_nearest_facet_brute": ([_P, _P, _P, _P], _I32),
            "two_nearest_batch": ([_P, _P, _I64, _P, _P, _P, _I], None),
            "two_smooth_star": ([_P, _P, _P, _I32, _I32, _I, _P, _P, _D, _D, _I, _I, _P], _I),
            "two_smooth_stars_batch": ([_P, _P, _P, _P, _P, _P, _I64, _P, _P, _D, _D, _I, _I, _P,
                                        _P, _I], None),
            "two_collapse_check_batch": ([_P, _P, _P, _P, _P, _P, _I64, _P, _P, _D, _D, _I, _D,
                                          _P, _I], None),
            "two_swap_check_batch": ([_P, _P, _P, _P, _P, _I64, _P, _P, _P], None),
            "two_energy_stats": ([_P, _P, _I64, _P, _D, _P, _P, _P, _P], None),
            "two_dihedral_minmax": ([_P, _P, _P], None),
            "two_dihedral_stats": ([_P, _P, _I64, _P, _P, _P, _P, _P], None),
            "two_filter_energy": ([_P, _D, _P], _D),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        self.L = L

    # scalar helpers
    def icbrt(self, x: float) -> float:
        return self.L.two_icbrt(x)

    def set_energy_form(self, form: int):
        """0: reference form (default), 1: closed form; process-wide."""
        self.L.two_set_energy_form(form)

    def energy_form(self) -> int:
        return self.L.two_get_energy_form()

    def orient3d(self, p, q, r, s) -> int:
        a = [_c(v, np.float64) for v in (p, q, r, s)]
        return self.L.two_orient3d(*[_p(v) for v in a])

    def orient3d_exact(self, p, q, r, s) -> int:
        a = [_c(v, np.float64) for v in (p, q, r, s)]
        return self.L.two_orient3d_exact(*[_p(v) for v in a])

    def collinear(self, a, b, c) -> int:
        v = [_c(x, np.float64) for x in (a, b, c)]
        return self.L.two_collinear(*[_p(x) for x in v])

    def point_triangle_sqdist(self, p, a, b, c) -> float:
        v = [_c(x, np.float64) for x in (p, a, b, c)]
        return self.L.two_point_triangle_sqdist(*[_p(x) for x in v], None)

    def qr_solve3(self, H, b):
        Hm = _c(H, np.float64).reshape(9)
        bb = _c(b, np.float64)
        x = np.empty(3)
        self.L.two_qr_solve3(_p(Hm), _p(bb), _p(x))
        return x

    def sample_triangle(self, tri9, sd):
        t = _c(tri9, np.float64).reshape(9)
        n = self.L.two_sample_count(_p(t), sd)
        out = np.empty((max(n, 1), 3))
        self.L.two_sample_triangle(_p(t), sd, _p(out), n)
        return out[:n]

    # batches
    def amips_batch_soa(self, T, quality=True, nthreads=1, energy=True, jacobian=True,
                        hessian=True, flip=True):
        T = _c(T, np.float64)
        n = T.shape[1]
        E = np.empty(n) if energy else None
        J = np.empty((3, n)) if jacobian else None
        H = np.empty((9, n)) if hessian else None
        F = np.empty(n, np.uint8) if flip else None
        self.L.two_amips_batch_soa(_p(T), n, 1 if quality else 0, _p(E), _p(J), _p(H), _p(F),
                                   nthreads)
        return E, J, H, F

    def surface(self, V, F):
        return OracleSurface(self, V, F)

    def newton_stars(self, xyz, star_off, tets, centers, max_step=15, max_it=20, nthreads=1):
        X = _c(xyz, np.float64).reshape(-1, 3)
        O = _c(star_off, np.int32)
        T = _c(tets, np.int32).reshape(-1, 4)
        C = _c(centers, np.int32)
        ns = C.size
        out = np.empty((ns, 3))
        moved = np.empty(ns, np.uint8)
        self.L.two_newton_stars_batch(_p(X), _p(O), _p(T), _p(C), ns, max_step, max_it, _p(out),
                                      _p(moved), nthreads)
        return out, moved


    def smooth_stars(self, xyz, star_off, tets, centers, face_flags=None, kinds=None,
                     surface=None, boundary=None, eps2=0.0, sd=0.0, max_step=15, max_it=20,
                     nthreads=1):
        """One smoothing pass over independent stars (two_smooth_star): returns
        (positions [ns,3], status [ns] int8)."""
        X = _c(xyz, np.float64).reshape(-1, 3)
        O = _c(star_off, np.int32)
        T = _c(tets, np.int32).reshape(-1, 4)
        C = _c(centers, np.int32)
        FF = None if face_flags is None else _c(face_flags, np.uint8)
        K = None if kinds is None else _c(kinds, np.uint8)
        ns = C.size
        out = np.empty((ns, 3))
        st = np.empty(ns, np.int8)
        self.L.two_smooth_stars_batch(_p(X), _p(O), _p(T), _p(FF), _p(C), _p(K), ns,
                                      surface.h if surface is not None else None,
                                      boundary.h if boundary is not None else None,
                                      eps2, sd, max_step, max_it, _p(out), _p(st), nthreads)
        return out, st


    def collapse_check(self, xyz, off, tets, face_flags, v12, flags, surface=None,
                       boundary=None, eps2=0.0, sd=0.0, check_quality=True, soft_energy=-1.0,
                       nthreads=1):
        """Checks of candidate collapses v12[i] = (v1, v2) (two_collapse_check): codes [n]."""
        X = _c(xyz, np.float64).reshape(-1, 3)
        O = _c(off, np.int32)
        T = _c(tets, np.int32).reshape(-1, 4)
        FF = _c(face_flags, np.uint8)
        V = _c(v12, np.int32).reshape(-1, 2)
        FL = _c(flags, np.uint8)
        n = V.shape[0]
        out = np.empty(n, np.uint8)
        self.L.two_collapse_check_batch(_p(X), _p(O), _p(T), _p(FF), _p(V), _p(FL), n,
                                        surface.h if surface is not None else None,
                                        boundary.h if boundary is not None else None, eps2, sd,
                                        1 if check_quality else 0, soft_energy, _p(out), nthreads)
        return out


    def swap_check(self, xyz, v12, off, tets, budget=None):
        """Checks of candidate edge removals (two_swap_check): (result, config, spent)."""
        X = _c(xyz, np.float64).reshape(-1, 3)
        O = _c(off, np.int32)
        T = _c(tets, np.int32).reshape(-1, 4)
        V = _c(v12, np.int32).reshape(-1, 2)
        B = None if budget is None else _c(budget, np.int32)
        n = V.shape[0]
        res = np.empty(n, np.uint8)
        cfg = np.empty(n, np.int8)
        sp = np.empty(n, np.uint8)
        self.L.two_swap_check_batch(_p(X), _p(O), _p(T), _p(V), _p(B), n, _p(res), _p(cfg), _p(sp))
        return res, cfg, sp

    def dihedral_minmax(self, T12):
        """calTetQuality_AD of one tet (12 coordinates): (min, max) dihedral angle."""
        t = _c(T12, np.float64).reshape(12)
        a, b = ctypes.c_double(), ctypes.c_double()
        self.L.two_dihedral_minmax(_p(t), ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def dihedral_stats(self, xyz, tets, locked=None):
        """outputInfo's dihedral sweep: (out[4] = min, avg min, max, avg max; counts[7];
        per-tet mins; per-tet maxs)."""
        X = _c(xyz, np.float64).reshape(-1, 3)
        T = _c(tets, np.int32).reshape(-1, 4)
        L = None if locked is None else _c(locked, np.uint8)
        n = T.shape[0]
        out = np.zeros(4)
        cnt = np.zeros(7, np.int64)
        mins = np.empty(n)
        maxs = np.empty(n)
        self.L.two_dihedral_stats(_p(X), _p(T), n, _p(L), _p(out), _p(cnt), _p(mins), _p(maxs))
        return out, cnt, mins, maxs

    def energy_stats(self, xyz, tets, locked=None, thres=10.0):
        """(avg, max, second max, buckets[11]) of getAvgMaxEnergy / getMaxEnergy /
        getSecondMaxEnergy / getFilterEnergy's histogram."""
        X = _c(xyz, np.float64).reshape(-1, 3)
        T = _c(tets, np.int32).reshape(-1, 4)
        L = None if locked is None else _c(locked, np.uint8)
        a, m, m2 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        b = np.zeros(11, np.int64)
        self.L.two_energy_stats(_p(X), _p(T), T.shape[0], _p(L), thres, ctypes.byref(a),
                                ctypes.byref(m), ctypes.byref(m2), _p(b))
        return a.value, m.value, m2.value, b

    def filter_energy(self, buckets, thres=10.0):
        b = _c(buckets, np.int64)
        c = ctypes.c_int()
        e = self.L.two_filter_energy(_p(b), thres, ctypes.byref(c))
        return e, bool(c.value)


class OracleSurface:
    def __init__(self, o: Oracle, V, F):
        self.o = o
        self.V = _c(V, np.float64).reshape(-1, 3)
        self.F = _c(F, np.int32).reshape(-1, 3)
        self.h = o.L.two_surface_build(_p(self.V), self.V.shape[0], _p(self.F), self.F.shape[0])

    def __del__(self):
        try:
            self.o.L.two_surface_free(self.h)
        except Exception:
            pass

    def points_out(self, P, eps2, nthreads=1):
        X = _c(P, np.float64).reshape(-1, 3)
        out = np.empty(X.shape[0], np.uint8)
        self.o.L.two_points_out_batch(self.h, _p(X), X.shape[0], eps2, _p(out), nthreads)
        return out

    def point_out_brute(self, p, eps2) -> int:
        x = _c(p, np.float64)
        return self.o.L.two_point_out_brute(self.h, _p(x), eps2)

    def faces_out(self, tris, eps2, sd, nthreads=1):
        X = _c(tris, np.float64).reshape(-1, 9)
        out = np.empty(X.shape[0], np.uint8)
        self.o.L.two_faces_out_batch(self.h, _p(X), X.shape[0], eps2, sd, _p(out), nthreads)
        return out

    def nearest(self, P, nthreads=1):
        """(closest points [n,3], squared distances [n], input facet ids [n])."""
        X = _c(P, np.float64).reshape(-1, 3)
        n = X.shape[0]
        Q = np.empty((n, 3))
        D = np.empty(n)
        F = np.empty(n, np.int32)
        self.o.L.two_nearest_batch(self.h, _p(X), n, _p(Q), _p(D), _p(F), nthreads)
        return Q, D, F

    def nearest_brute(self, p):
        x = _c(p, np.float64)
        q = np.empty(3)
        d = ctypes.c_double()
        f = self.o.L.two_nearest_facet_brute(self.h, _p(x), _p(q), ctypes.byref(d))
        return q, d.value, int(f)


class RefLib:
    """The reference's own code (oracle/_ref/libtwref.so)."""

    def __init__(self):
        if not REF_SO.exists():
            if build_ref() is None:
                raise FileNotFoundError("oracle/_ref is not built (reference sources unavailable)")
        L = ctypes.CDLL(str(REF_SO))
        sig = {
            "twref_amips_batch_soa": ([_P, _I64, _P, _P, _P, _I], None),
            "twref_sample_triangle": ([_P, _D, _P, _I64], _I64),
            "twref_surface_build": ([_P, _I32, _P, _I32], _P),
            "twref_surface_free": ([_P], None),
            "twref_points_out": ([_P, _P, _I64, _D, _P, _I], None),
            "twref_faces_out": ([_P, _P, _I64, _D, _D, _P, _I], None),
            "twref_nearest": ([_P, _P, _I64, _P, _P, _I], None),
            "twref_energy_sweeps": ([_P, _P, _P, _I64, _D, _P, _P], None),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        self.L = L

    @staticmethod
    def available() -> bool:
        return REF_SO.exists() or (HERE / "_ref" / "src" / "amips_slice.inc").exists() or \
            (_recipe().reference_root() / "src").is_dir()

    def amips_batch_soa(self, T, nthreads=1, energy=True, jacobian=True, hessian=True):
        T = _c(T, np.float64)
        n = T.shape[1]
        E = np.empty(n) if energy else None
        J = np.empty((3, n)) if jacobian else None
        H = np.empty((9, n)) if hessian else None
        self.L.twref_amips_batch_soa(_p(T), n, _p(E), _p(J), _p(H), nthreads)
        return E, J, H

    def energy_sweeps(self, E, removed=None, locked=None, thres=10.0):
        """The reference's getAvgMaxEnergy / getMaxEnergy / getSecondMaxEnergy /
        getFilterEnergy over per-tet energies: (avg, max, max, second max, filter, clean_up)."""
        E = _c(E, np.float64)
        R = None if removed is None else _c(removed, np.uint8)
        L = None if locked is None else _c(locked, np.uint8)
        out = np.empty(5)
        c = ctypes.c_int()
        self.L.twref_energy_sweeps(_p(E), _p(R), _p(L), E.shape[0], thres, _p(out),
                                   ctypes.byref(c))
        return (*out.tolist(), bool(c.value))

    def sample_triangle(self, tri9, sd):
        t = _c(tri9, np.float64).reshape(9)
        n = self.L.twref_sample_triangle(_p(t), sd, None, 0)
        out = np.empty((max(n, 1), 3))
        self.L.twref_sample_triangle(_p(t), sd, _p(out), n)
        return out[:n]

    def surface(self, V, F):
        return RefSurface(self, V, F)


class RefSurface:
    def __init__(self, r: RefLib, V, F):
        self.r = r
        self.V = _c(V, np.float64).reshape(-1, 3)
        self.F = _c(F, np.int32).reshape(-1, 3)
        self.h = r.L.twref_surface_build(_p(self.V), self.V.shape[0], _p(self.F), self.F.shape[0])

    def __del__(self):
        try:
            self.r.L.twref_surface_free(self.h)
        except Exception:
            pass

    def points_out(self, P, eps2, nthreads=1):
        X = _c(P, np.float64).reshape(-1, 3)
        out = np.empty(X.shape[0], np.uint8)
        self.r.L.twref_points_out(self.h, _p(X), X.shape[0], eps2, _p(out), nthreads)
        return out

    def faces_out(self, tris, eps2, sd, nthreads=1):
        X = _c(tris, np.float64).reshape(-1, 9)
        out = np.empty(X.shape[0], np.uint8)
        self.r.L.twref_faces_out(self.h, _p(X), X.shape[0], eps2, sd, _p(out), nthreads)
        return out

    def nearest(self, P, nthreads=1):
        """(closest points [n,3], squared distances [n]) from the reference's tree."""
        X = _c(P, np.float64).reshape(-1, 3)
        n = X.shape[0]
        Q = np.empty((n, 3))
        D = np.empty(n)
        self.r.L.twref_nearest(self.h, _p(X), n, _p(Q), _p(D), nthreads)
        return Q, D
