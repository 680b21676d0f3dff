"""Certified FP32 mode: binary32 bulk with binary64 recomputation inside a
certified band.  Every decision must equal the plain FP64 path and the
oracle, on ordinary inputs and on inputs built to sit on the band's edges:
points at eps (1 +- k ulp) from a facet, sliver facets (never culled),
coordinates far from the origin (large binary32 rounding), tiny eps.
"""
import numpy as np
import pytest

import tetwild_gb300 as tw
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _both_modes(ctx, fn):
    ctx.set_precision(tw.TW_PRECISION_FP64)
    a = fn()
    ctx.set_precision(tw.TW_PRECISION_FP32_CERTIFIED)
    ctx.reset_stats()
    b = fn()
    st = ctx.stats()
    ctx.set_precision(tw.TW_PRECISION_FP64)
    return a, b, st


def test_certified_points_displaced_sphere(ctx, oracle):
    V, F = syn.displaced_sphere(seed=3)
    eps = 1e-3
    P = syn.envelope_points(V, F, 500_000, eps, seed=12)
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    a, b, st = _both_modes(ctx, lambda: ctx.envelope_points(P))
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=8)
    assert np.array_equal(a, want)
    assert np.array_equal(b, want)
    assert st["env_queries"] == len(P)
    # the FP32 lower bound decides most facets; FP64 only near the threshold
    assert st["env_facet_fp64"] < 0.6 * st["env_facet_tests"]


@pytest.mark.parametrize("offset", [0.0, 1000.0])
def test_certified_points_at_threshold(ctx, oracle, offset):
    V = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.0]]) + offset
    F = np.array([[0, 1, 2], [1, 3, 2]], np.int32)
    eps = 1e-3
    rng = np.random.default_rng(6)
    n = 4000
    xy = rng.random((n, 2)) * 1.2 - 0.1
    z = np.full(n, eps)
    for i in range(n):
        for _ in range(int(rng.integers(-4, 5))):
            z[i] = np.nextafter(z[i], np.inf if rng.random() < 0.5 else 0.0)
    P = np.c_[xy, z] + offset
    # edge and vertex regions at distance ~eps
    ang = rng.random(500) * 2 * np.pi
    Pv = np.c_[eps * np.cos(ang) * 0.999999, eps * np.sin(ang) * 0.999999, np.zeros(500)]
    Pv[:250] += [1.0, 1.0, 0.0]
    P = np.vstack([P, Pv + offset])
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    a, b, _ = _both_modes(ctx, lambda: ctx.envelope_points(P))
    want = oracle.surface(V, F).points_out(P, eps * eps)
    assert np.array_equal(a, want) and np.array_equal(b, want)
    assert 0 < want.sum() < len(P)


def test_certified_points_sliver_facets(ctx, oracle):
    rng = np.random.default_rng(13)
    # fan of slivers: long thin triangles with tiny angles, plus a degenerate one
    base = np.array([0.5, 0.5, 0.5])
    V = [base]
    F = []
    for k in range(200):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        e = np.cross(d, rng.normal(size=3))
        e /= np.linalg.norm(e)
        V.append(base + 0.3 * d)
        V.append(base + 0.3 * d + 10 ** rng.uniform(-9, -5) * e)
        F.append((0, 2 * k + 1, 2 * k + 2))
    V.append(base + [0.1, 0.1, 0.1])
    F.append((0, len(V) - 1, len(V) - 1))  # degenerate (repeated vertex)
    V = np.asarray(V)
    F = np.asarray(F, np.int32)
    eps = 2e-4
    P = base + rng.normal(size=(20000, 3)) * 0.15
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    a, b, _ = _both_modes(ctx, lambda: ctx.envelope_points(P))
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=4)
    assert np.array_equal(a, want) and np.array_equal(b, want)


def test_certified_faces(ctx, oracle):
    V, F = syn.displaced_sphere(seed=8, n_lon=200, n_rings=80)
    eps = 2e-3
    rng = np.random.default_rng(19)
    idx = rng.integers(0, len(F), 3000)
    A, B, C = V[F[idx, 0]], V[F[idx, 1]], V[F[idx, 2]]
    cen = (A + B + C) / 3
    nrm = np.cross(B - A, C - A)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    grow = rng.uniform(0.5, 3.0, (3000, 1))
    push = rng.uniform(-1.2, 1.2, (3000, 1)) * eps
    tris = np.hstack([cen + grow * (A - cen) + push * nrm, cen + grow * (B - cen) + push * nrm,
                      cen + grow * (C - cen) + push * nrm])
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    a, b, st = _both_modes(ctx, lambda: ctx.envelope_faces(tris))
    want = oracle.surface(V, F).faces_out(tris, eps * eps, eps, nthreads=8)
    assert np.array_equal(a, want) and np.array_equal(b, want)
    assert st["env_queries"] > len(tris)
