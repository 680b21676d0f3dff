"""GPU parity: every kernel, called through the C-ABI, against the CPU oracle.

Decisions (orientation signs, envelope in/out, Newton accept/reject and the
resulting positions) must be bit-identical.  Energies, gradients and
Hessians are compared bit for bit too: the device evaluates the same
operations in the same order as the oracle (no FP contraction), so the
1e-12 relative tolerance that the path allows is not even needed here; the
tests assert equality and, separately, report the relative error.
"""
import numpy as np
import pytest

import tetwild_gb300 as tw
from conftest import golden
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # plain FP64 tolerance of the path for E/J/H


def _same_or_both_nonfinite(a, b):
    fa, fb = np.isfinite(a), np.isfinite(b)
    return np.array_equal(fa, fb) and np.array_equal(a[fa], b[fb])


# ------------------------------------------------------------------ AMIPS ----
def test_amips_energy_batch_bitwise(ctx, oracle):
    T = syn.energy_batch(200_000, seed=1)
    g = ctx.amips(T, tw.TW_ENERGY_QUALITY)
    E, J, H, F = oracle.amips_batch_soa(T, quality=True, nthreads=8)
    assert np.array_equal(g["flip"], F)
    assert np.array_equal(g["E"], E)
    assert _same_or_both_nonfinite(g["J"], J)
    assert _same_or_both_nonfinite(g["H"], H)
    # sanity of the workload: ~5% near-degenerate (AMIPS energy > 3.5, the
    # optimum being 3); N(0, 0.1 edge) perturbations invert none
    assert 0.03 < (E > 3.5).mean() < 0.08


def test_amips_raw_mode_and_partial_outputs(ctx, oracle):
    T = syn.energy_batch(10_000, seed=2, sigma_rel=0.3)
    E, J, H, F = oracle.amips_batch_soa(T, quality=False, nthreads=4)
    g = ctx.amips(T, tw.TW_ENERGY_RAW, energy=True, jacobian=False, hessian=True, flip=False)
    assert set(g) == {"E", "H"}
    assert _same_or_both_nonfinite(g["E"], E)
    assert _same_or_both_nonfinite(g["H"], H)
    g2 = ctx.amips(T, tw.TW_ENERGY_RAW, energy=False, jacobian=True, hessian=False, flip=True)
    assert _same_or_both_nonfinite(g2["J"], J) and np.array_equal(g2["flip"], F)


def test_amips_golden_reference_tolerance(ctx):
    """Against the reference's own generated expressions (golden fixture): every
    tet, 1e-12 relative (the default energy form performs the reference's
    operations)."""
    g = golden("amips_ref.npz")
    T = np.ascontiguousarray(g["T"].T)
    out = ctx.amips(T, tw.TW_ENERGY_RAW, flip=False)
    rel = np.abs(out["E"] - g["E"]) / np.abs(g["E"])
    assert rel.max() <= REL_TOL


def test_amips_edge_cases(ctx, oracle):
    t = syn.REGULAR_TET.reshape(12)
    cases = [t, t.reshape(4, 3)[[1, 0, 2, 3]].reshape(12), np.zeros(12),
             np.r_[t[:9], t[:3]],                       # repeated vertex
             np.r_[t[:9], 0.5, 0.2, 0.0],               # coplanar
             t * 1e-100, t * 1e100, np.r_[t[:11], np.nan], np.r_[t[:11], np.inf]]
    T = np.ascontiguousarray(np.asarray(cases).T)
    g = ctx.amips(T, tw.TW_ENERGY_QUALITY)
    E, J, H, F = oracle.amips_batch_soa(T, quality=True)
    assert np.array_equal(g["flip"], F)
    assert np.array_equal(g["E"], E)
    assert _same_or_both_nonfinite(g["J"], J) and _same_or_both_nonfinite(g["H"], H)
    assert g["E"][0] == pytest.approx(3.0, abs=1e-14)
    assert np.all(g["E"][1:] == 1e50)


def test_amips_empty_and_odd_sizes(ctx, oracle):
    for n in (0, 1, 255, 257, 65537):
        T = syn.energy_batch(max(n, 1), seed=n)[:, :n].copy()
        g = ctx.amips(T, tw.TW_ENERGY_QUALITY)
        if n:
            E, J, H, F = oracle.amips_batch_soa(T, quality=True)
            assert np.array_equal(g["E"], E) and np.array_equal(g["flip"], F)
        else:
            assert g["E"].size == 0


# ------------------------------------------------------------ orientation ----
def test_orientation_adversarial_exact(ctx):
    gd = golden("orient_exact.npz")
    quads = gd["quads"]
    T = np.ascontiguousarray(quads.reshape(-1, 12).T)
    g = ctx.amips(T, tw.TW_ENERGY_QUALITY, jacobian=False, hessian=False)
    want_flip = (gd["signs"] != 1).astype(np.uint8)
    assert np.array_equal(g["flip"], want_flip)


def test_tet_quality_indexed(ctx, oracle):
    rng = np.random.default_rng(5)
    xyz = rng.random((5000, 3))
    tets = rng.integers(0, 5000, (40000, 4)).astype(np.int32)
    ctx.mesh_upload(xyz)
    E, F, N, st = ctx.tet_quality(tets)
    assert st == tw.TW_OK and not N.any()
    T = np.ascontiguousarray(xyz[tets].reshape(-1, 12).T)
    Eo, _, _, Fo = oracle.amips_batch_soa(T, quality=True, nthreads=4, jacobian=False, hessian=False)
    assert np.array_equal(F, Fo) and np.array_equal(E, Eo)
    # unrounded vertices: the call reports which tets need the host's exact path
    rounded = np.ones(5000, np.uint8)
    rounded[:10] = 0
    ctx.mesh_upload(xyz, rounded)
    E2, F2, N2, st2 = ctx.tet_quality(tets)
    assert st2 == tw.TW_NEEDS_EXACT_HOST
    assert np.array_equal(N2.astype(bool), (tets < 10).any(1))
    # vertex updates
    ids = np.arange(0, 5000, 7, dtype=np.int32)
    newx = rng.random((ids.size, 3))
    ctx.mesh_update_vertices(ids, newx)
    xyz2 = xyz.copy()
    xyz2[ids] = newx
    E3, F3, _, _ = ctx.tet_quality(tets)
    T3 = np.ascontiguousarray(xyz2[tets].reshape(-1, 12).T)
    Eo3, _, _, Fo3 = oracle.amips_batch_soa(T3, quality=True, jacobian=False, hessian=False)
    assert np.array_equal(E3, Eo3) and np.array_equal(F3, Fo3)
    with pytest.raises(tw.TetWildGpuError):
        ctx.tet_quality(np.array([[0, 1, 2, 5000]], np.int32))


# --------------------------------------------------------------- envelope ----
def test_envelope_points_golden(ctx):
    gd = golden("envelope_ref.npz")
    eps = float(gd["eps"])
    ctx.set_params(eps * eps, float(gd["sd"]))
    ctx.surface_upload(gd["V"], gd["F"])
    out = ctx.envelope_points(gd["P"])
    assert np.array_equal(out, gd["point_out"])


def test_envelope_faces_golden(ctx):
    gd = golden("envelope_ref.npz")
    eps = float(gd["eps"])
    ctx.set_params(eps * eps, float(gd["sd"]))
    ctx.surface_upload(gd["V"], gd["F"])
    out = ctx.envelope_faces(gd["faces"])
    assert np.array_equal(out, gd["face_out"])


def test_envelope_points_displaced_sphere(ctx, oracle):
    V, F = syn.displaced_sphere(seed=3)
    eps = 1e-3
    P = syn.envelope_points(V, F, 300_000, eps, seed=4)
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    out = ctx.envelope_points(P)
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=8)
    assert np.array_equal(out, want)
    assert 0.3 < out.mean() < 0.7


def test_envelope_points_at_threshold(ctx, oracle):
    """Points whose distance to a facet is eps * (1 +- k ulp)."""
    V = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.0]])
    F = np.array([[0, 1, 2], [1, 3, 2]], np.int32)
    eps = 1e-3
    rng = np.random.default_rng(6)
    xy = rng.random((2000, 2)) * 0.9 + 0.05
    z = np.full(2000, eps)
    for i in range(2000):
        for _ in range(int(rng.integers(-3, 4))):
            z[i] = np.nextafter(z[i], np.inf if rng.random() < 0.5 else 0.0)
    # edge and vertex regions too
    P = np.vstack([np.c_[xy, z], [[-eps, 0.5, 0.0]], [[1 + eps, 1 + 0.0, 0.0]],
                   [[0.0, 0.0, np.nextafter(eps, 1)]], [[0.5, 0.5, 0.0]]])
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    out = ctx.envelope_points(P)
    S = oracle.surface(V, F)
    want = S.points_out(P, eps * eps)
    brute = np.array([S.point_out_brute(p, eps * eps) for p in P], np.uint8)
    assert np.array_equal(want, brute)
    assert np.array_equal(out, want)
    assert 0 < out.sum() < len(P)


def test_envelope_single_facet_and_boundary_tree(ctx, oracle):
    V = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0]])
    F = np.array([[0, 1, 2]], np.int32)
    P = np.random.default_rng(7).normal(size=(5000, 3)) * 0.01 + [0.3, 0.3, 0.0]
    ctx.set_params(1e-4, 0.01)
    ctx.surface_upload(V, F, tw.TW_SURFACE_BOUNDARY)
    out = ctx.envelope_points(P, tw.TW_SURFACE_BOUNDARY)
    want = oracle.surface(V, F).points_out(P, 1e-4)
    assert np.array_equal(out, want)


def test_sample_triangle_device_matches_reference_golden(ctx):
    gd = golden("sample_ref.npz")
    sd = float(gd["sd"])
    for i, t in enumerate(gd["tris"]):
        want = gd["samples"][gd["offsets"][i]:gd["offsets"][i + 1]]
        got, cnt = ctx.sample_triangle(t, sd)
        assert cnt == len(want), i
        assert np.array_equal(got, want), i


def test_envelope_faces_vs_oracle(ctx, oracle):
    V, F = syn.displaced_sphere(seed=8, n_lon=200, n_rings=80)
    eps = 2e-3
    sd = eps
    rng = np.random.default_rng(9)
    idx = rng.integers(0, len(F), 3000)
    A, B, C = V[F[idx, 0]], V[F[idx, 1]], V[F[idx, 2]]
    cen = (A + B + C) / 3
    nrm = np.cross(B - A, C - A)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    grow = rng.uniform(0.5, 3.0, (3000, 1))
    push = rng.uniform(-1.2, 1.2, (3000, 1)) * eps
    tris = np.hstack([cen + grow * (A - cen) + push * nrm, cen + grow * (B - cen) + push * nrm,
                      cen + grow * (C - cen) + push * nrm])
    tris[:5] = np.array([0, 0, 0, 1, 1, 1, 2, 2, 2.0])  # degenerate: never out
    ctx.set_params(eps * eps, sd)
    ctx.surface_upload(V, F)
    out = ctx.envelope_faces(tris)
    want = oracle.surface(V, F).faces_out(tris, eps * eps, sd, nthreads=8)
    assert np.array_equal(out, want)
    assert not out[:5].any()
    assert 0.05 < out.mean() < 0.95


# ----------------------------------------------------------------- Newton ----
def test_newton_stars_bitwise(ctx, oracle):
    xyz, off, tets, cen = syn.star_batch(3000, seed=10)
    ctx.set_params(1e-6, 1e-3, 15, 20)
    ctx.mesh_upload(xyz)
    out, moved = ctx.newton_stars(off, tets, cen)
    want, wmoved = oracle.newton_stars(xyz, off, tets, cen, 15, 20, nthreads=8)
    assert np.array_equal(moved, wmoved)
    assert np.array_equal(out, want)
    assert moved.mean() > 0.5


def test_newton_stars_capped_backtracking(ctx, oracle):
    xyz, off, tets, cen = syn.star_batch(1000, seed=11, jitter_rel=0.3)
    ctx.set_params(1e-6, 1e-3, 1, 8)
    ctx.mesh_upload(xyz)
    out, moved = ctx.newton_stars(off, tets, cen)
    want, wmoved = oracle.newton_stars(xyz, off, tets, cen, 1, 8, nthreads=8)
    assert np.array_equal(moved, wmoved) and np.array_equal(out, want)


@pytest.mark.parametrize("mean_tets", [6.0, 24.0, 60.0])
def test_newton_every_launch_shape_bitwise(ctx, oracle, mean_tets):
    """Every launch shape (thread per star; 8, 16 or 32 lanes per star with the
    per-tet terms added in tet order) reproduces the oracle bit for bit, on
    stars smaller than, close to and larger than one lane group."""
    xyz, off, tets, cen = syn.star_batch(1200, seed=12 + int(mean_tets), mean_tets=mean_tets,
                                         lo=4, hi=96, jitter_rel=0.2)
    ctx.set_params(1e-6, 1e-3, 15, 20)
    ctx.mesh_upload(xyz)
    want, wmoved = oracle.newton_stars(xyz, off, tets, cen, 15, 20, nthreads=8)
    try:
        for shape in range(ctx.NEWTON_SHAPES):
            ctx.set_newton_shape(shape)
            out, moved = ctx.newton_stars(off, tets, cen)
            assert np.array_equal(moved, wmoved), shape
            assert np.array_equal(out, want), shape
    finally:
        ctx.set_newton_shape(5)


def test_newton_shape_rejects_unknown(ctx):
    with pytest.raises(tw.TetWildGpuError):
        ctx.set_newton_shape(ctx.NEWTON_SHAPES)
    with pytest.raises(tw.TetWildGpuError):
        ctx.set_newton_shape(-1)


def test_newton_device_autotune_and_graph_replay(ctx, oracle):
    """Device-pointer Newton step: autotuned shape, then captured in a CUDA
    graph and replayed; each replay rewrites the same outputs identically."""
    import torch

    xyz, off, tets, cen = syn.star_batch(2000, seed=21, mean_tets=24.0)
    ctx.set_params(1e-6, 1e-3, 1, 8)
    ctx.mesh_upload(xyz)
    want, wmoved = oracle.newton_stars(xyz, off, tets, cen, 1, 8, nthreads=8)
    dev = torch.device("cuda", 0)
    d_off = torch.from_numpy(off.astype(np.int32)).to(dev)
    d_tets = torch.from_numpy(tets.astype(np.int32).reshape(-1)).to(dev)
    d_cen = torch.from_numpy(cen.astype(np.int32)).to(dev)
    ns = int(cen.size)
    d_out = torch.empty(3 * ns, dtype=torch.float64, device=dev)
    d_mov = torch.empty(ns, dtype=torch.uint8, device=dev)
    args = (d_off.data_ptr(), d_tets.data_ptr(), d_cen.data_ptr(), ns, d_out.data_ptr(),
            d_mov.data_ptr())
    try:
        torch.cuda.synchronize()
        best, ms = ctx.newton_autotune_device(*args)
        assert 0 <= best < ctx.NEWTON_SHAPES and all(t > 0 for t in ms)
        assert np.array_equal(d_out.cpu().numpy().reshape(-1, 3), want)
        d_out.fill_(0.0)
        d_mov.fill_(7)
        torch.cuda.synchronize()
        ctx.capture_begin()
        ctx.newton_stars_device(*args)
        g = ctx.capture_end()
        for _ in range(2):
            g.launch()
            ctx.synchronize()
            assert np.array_equal(d_mov.cpu().numpy(), wmoved)
            assert np.array_equal(d_out.cpu().numpy().reshape(-1, 3), want)
            d_out.fill_(0.0)
            torch.cuda.synchronize()
        g.close()
    finally:
        ctx.set_newton_shape(5)
