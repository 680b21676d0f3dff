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


def test_point_kernel_shapes_same_decisions(ctx, oracle):
    """Every launch shape of the grid point test (blocks of 128, 256, 384, 768) in both
    precision modes, ragged tails included (n not a multiple of 32), a batch below the
    sort threshold and a single point: the oracle's decisions."""
    V, F = syn.displaced_sphere(seed=4)
    eps = 1e-3
    P = syn.envelope_points(V, F, 300_007, eps, seed=14)
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=8)
    try:
        for shape in (128, 256, 384, 768):
            ctx.set_tuning(ctx.TUNE_POINT_BLOCK, shape)
            a, b, _ = _both_modes(ctx, lambda: ctx.envelope_points(P))
            assert np.array_equal(a, want), shape
            assert np.array_equal(b, want), shape
            # a batch below the sort threshold (input order) and a one-point batch
            small = P[:1000]
            a, b, _ = _both_modes(ctx, lambda: ctx.envelope_points(small))
            assert np.array_equal(a, want[:1000]) and np.array_equal(b, want[:1000])
            a, b, _ = _both_modes(ctx, lambda: ctx.envelope_points(P[:1]))
            assert a[0] == want[0] and b[0] == want[0]
    finally:
        ctx.set_tuning(ctx.TUNE_POINT_BLOCK, 384)


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


def _soup(n, size, seed):
    """n random triangles of edge ~size in every orientation inside the unit box."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3))
    V = (c + (rng.random((n, 3, 3)) - 0.5) * size).reshape(-1, 3)
    return V, np.arange(3 * n, dtype=np.int32).reshape(n, 3)


@pytest.mark.parametrize("cell,offset", [(0.05, 0.0), (0.1, 0.0), (0.2, 0.0), (1.0, 0.0),
                                         (0.1, 1000.0)])
def test_certified_grid_keeps_every_facet_within_reach(ctx, oracle, cell, offset):
    """Points just inside eps of a random point of a random facet (interior, edges and
    corners), in random directions: a facet dropped from a cell's list by the grid's
    separating-axis culling would turn such a point out.  The offset moves the soup far
    from the origin, where binary32 rounding of the culling is largest."""
    V, F = _soup(3000, 0.05, seed=21)
    V = V + offset
    eps = 2e-3
    rng = np.random.default_rng(22)
    n = 60000
    f = rng.integers(0, len(F), n)
    w = rng.random((n, 3)) ** 3          # many points near edges and corners
    w /= w.sum(1, keepdims=True)
    X = np.einsum("ij,ijk->ik", w, V[F[f]])
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = eps * np.where(rng.random(n) < 0.5, 1 - 1e-7, 1 + 1e-7)
    P = X + d * r[:, None]
    ctx.set_params(eps * eps, eps)
    ctx.set_tuning(tw.Context.TUNE_GRID_CELL, cell)
    try:
        ctx.surface_upload(V, F)
        a, b, _ = _both_modes(ctx, lambda: ctx.envelope_points(P))
    finally:
        ctx.set_tuning(tw.Context.TUNE_GRID_CELL, 0.2)
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=8)
    assert np.array_equal(a, want) and np.array_equal(b, want)
    assert want.sum() < len(P) // 2        # the inner half is in by construction


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


def _term_scales(T_soa):
    """Magnitudes of the terms that J and H sum (forward-error scale), per tet."""
    P = T_soa.T.reshape(-1, 4, 3)
    a = P[:, 0] - P[:, 3]
    b = (P[:, 0] - 2 * P[:, 1] + P[:, 3]) / np.sqrt(3)
    c = (P[:, 0] + P[:, 1] + P[:, 3] - 3 * P[:, 2]) / np.sqrt(6)
    N = (a * a).sum(1) + (b * b).sum(1) + (c * c).sum(1)
    D = np.einsum("ij,ij->i", a, np.cross(b, c))
    g = np.cross(b, c) + np.cross(c, a) / np.sqrt(3) + np.cross(a, b) / np.sqrt(6)
    gN = 2 * (a + b / np.sqrt(3) + c / np.sqrt(6))
    r = np.abs(D) ** (-2.0 / 3.0)
    ng, ngN = np.linalg.norm(g, axis=1), np.linalg.norm(gN, axis=1)
    sJ = r * (ngN + 2.0 / 3.0 * N / np.abs(D) * ng)
    sH = 3 * r + 4.0 / 3.0 * r / np.abs(D) * ngN * ng + 10.0 / 9.0 * N * r / D ** 2 * ng ** 2
    return sJ, sH


E_TOL32 = 1e-5  # certified relative energy error of the binary32 mode


@pytest.mark.parametrize("sigma", [0.1, 0.35])
def test_certified_amips_batch(ctx, sigma):
    T = syn.energy_batch(400_000, seed=31, sigma_rel=sigma)
    a, b, st = _both_modes(ctx, lambda: ctx.amips(T, tw.TW_ENERGY_QUALITY))
    assert np.array_equal(a["flip"], b["flip"])
    sent = a["E"] >= 1e50
    assert np.array_equal(sent, b["E"] >= 1e50)
    rel = np.abs(b["E"][~sent] - a["E"][~sent]) / np.abs(a["E"][~sent])
    assert rel.max() <= E_TOL32, rel.max()
    sJ, sH = _term_scales(T)
    ok = ~sent
    errJ = np.abs(b["J"] - a["J"]).max(0)[ok] / sJ[ok]
    errH = np.abs(b["H"] - a["H"]).max(0)[ok] / sH[ok]
    assert errJ.max() <= E_TOL32 and errH.max() <= E_TOL32, (errJ.max(), errH.max())
    assert st["amips_tets"] == T.shape[1]
    if sigma == 0.1:
        assert st["amips_fp64"] < 0.2 * st["amips_tets"]
    else:
        assert a["flip"].sum() > 0


def test_certified_amips_edge_cases(ctx):
    t = syn.REGULAR_TET.reshape(12)
    cases = [t, t.reshape(4, 3)[[1, 0, 2, 3]].reshape(12), np.zeros(12), np.r_[t[:9], t[:3]],
             np.r_[t[:9], 0.5, 0.2, 0.0], t * 1e-100, t * 1e100, t * 1e-12 + 0.5,
             t * 1e6, np.r_[t[:11], np.nan], np.r_[t[:11], np.inf]]
    T = np.ascontiguousarray(np.asarray(cases).T)
    a, b, _ = _both_modes(ctx, lambda: ctx.amips(T, tw.TW_ENERGY_QUALITY))
    assert np.array_equal(a["flip"], b["flip"])
    fa = np.isfinite(a["E"]) & (a["E"] < 1e50)
    assert np.array_equal(fa, np.isfinite(b["E"]) & (b["E"] < 1e50))
    assert np.all(np.abs(b["E"][fa] - a["E"][fa]) <= E_TOL32 * a["E"][fa])
    assert np.array_equal(a["E"][~fa], b["E"][~fa])


def test_certified_without_grid(ctx, oracle):
    """A facet whose box spans more than 2^16 grid cells leaves the surface without a grid:
    the certified point and face tests fall back to the tree walk (warp-shared candidates),
    with the same decisions."""
    Vs, Fs = syn.icosphere(3)
    big = np.array([[-50.0, -50.0, 3.0], [50.0, -50.0, 3.0], [0.0, 50.0, 3.0]])
    V = np.vstack([Vs, big])
    F = np.vstack([Fs, np.array([[len(Vs), len(Vs) + 1, len(Vs) + 2]])]).astype(np.int32)
    eps = 2e-3
    rng = np.random.default_rng(31)
    P = np.vstack([syn.envelope_points(Vs, Fs, 20000, eps, seed=32),
                   np.c_[rng.uniform(-40, 40, (5000, 2)), 3.0 + rng.uniform(-2 * eps, 2 * eps, 5000)]])
    ctx.set_params(eps * eps, eps / 2)
    ctx.surface_upload(V, F)
    a, b, _ = _both_modes(ctx, lambda: ctx.envelope_points(P))
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=8)
    assert np.array_equal(a, want) and np.array_equal(b, want)
    assert 0 < want.sum() < len(P)
    tri = np.hstack([Vs[Fs[:200, 0]], Vs[Fs[:200, 1]], Vs[Fs[:200, 2]]])
    tri = tri + rng.uniform(-1.5 * eps, 1.5 * eps, (len(tri), 1))
    fa, fb, _ = _both_modes(ctx, lambda: ctx.envelope_faces(tri))
    fw = oracle.surface(V, F).faces_out(tri, eps * eps, eps / 2, nthreads=8)
    assert np.array_equal(fa, fw) and np.array_equal(fb, fw)


def test_full_size_step_decisions(ctx, oracle):
    """The bench's step at its full size: all 10M point decisions around the 100k-facet
    displaced sphere in both precision modes, and the flips and energy sentinels of all
    4M certified AMIPS evaluations, against the oracle (energies within 1e-5 of FP64)."""
    from oracle.oracle import default_threads

    V, F = syn.displaced_sphere(seed=0)
    eps = 1e-3
    P = syn.envelope_points(V, F, 10_000_000, eps, seed=1)
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    a, b, _ = _both_modes(ctx, lambda: ctx.envelope_points(P))
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=default_threads())
    assert np.array_equal(a, want) and np.array_equal(b, want)
    T = syn.energy_batch(4_000_000, seed=3)
    ctx.set_precision(tw.TW_PRECISION_FP32_CERTIFIED)
    try:
        g = ctx.amips(T, tw.TW_ENERGY_QUALITY, True, False, False, True)
    finally:
        ctx.set_precision(tw.TW_PRECISION_FP64)
    E, _, _, Fl = oracle.amips_batch_soa(T, quality=True, jacobian=False, hessian=False,
                                         nthreads=default_threads())
    assert np.array_equal(g["flip"], Fl) and np.array_equal(g["E"] >= 1e50, E >= 1e50)
    fin = E < 1e50
    assert np.max(np.abs(g["E"][fin] - E[fin]) / E[fin]) <= 1e-5
