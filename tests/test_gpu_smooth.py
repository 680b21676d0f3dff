"""GPU parity of the nearest-facet queries and of the smoothing pass
(smoothSingle / smoothSurface per-vertex bodies) against the CPU oracle.

Every status and every position must be bit-identical, in both precision
modes and for every launch shape of the Newton step.
"""
import numpy as np
import pytest

import tetwild_gb300 as tw
from conftest import golden
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

EPS = 1e-3


@pytest.fixture(scope="module")
def sphere():
    return syn.displaced_sphere(seed=0, n_lon=100, n_rings=50)


def test_nearest_points_vs_oracle(ctx, oracle, sphere):
    V, F = sphere
    rng = np.random.default_rng(3)
    P = syn.envelope_points(V, F, 30000, EPS, seed=4)
    P = np.vstack([P, P[:5000] + rng.normal(0, 0.03, (5000, 3)), rng.uniform(-2, 2, (2000, 3))])
    ctx.surface_upload(V, F)
    Q, D, Fi = ctx.nearest_points(P)
    Qo, Do, Fo = oracle.surface(V, F).nearest(P, nthreads=8)
    assert np.array_equal(D, Do)
    assert np.array_equal(Fi, Fo)
    assert np.array_equal(Q, Qo)


def test_nearest_points_reference_golden(ctx):
    g = golden("nearest_ref.npz")
    ctx.surface_upload(g["V"], g["F"])
    Q, D, _ = ctx.nearest_points(g["P"])
    assert np.array_equal(D, g["D"])
    diff = np.any(Q != g["Q"], axis=1)   # equal-distance ties only (see the oracle pins)
    assert diff.mean() < 0.02


def test_nearest_single_facet(ctx, oracle):
    V = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0]])
    F = np.array([[0, 1, 2]], np.int32)
    P = np.random.default_rng(0).uniform(-1, 2, (500, 3))
    ctx.surface_upload(V, F, tw.TW_SURFACE_BOUNDARY)
    Q, D, Fi = ctx.nearest_points(P, tw.TW_SURFACE_BOUNDARY)
    Qo, Do, Fo = oracle.surface(V, F).nearest(P)
    assert np.array_equal(Q, Qo) and np.array_equal(D, Do) and (Fi == 0).all()


def _mixed(sphere, n, seed):
    V, F = sphere
    return syn.mixed_star_batch(V, F, n, EPS, seed=seed, surface_fraction=0.6)


def _oracle_pass(oracle, sphere, batch, max_step, max_it, boundary=None):
    V, F = sphere
    xyz, off, tets, ff, cen, kinds = batch
    S = oracle.surface(V, F)
    B = oracle.surface(*boundary) if boundary is not None else S
    return oracle.smooth_stars(xyz, off, tets, cen, ff, kinds, surface=S, boundary=B,
                               eps2=EPS * EPS, sd=EPS / 2, max_step=max_step, max_it=max_it,
                               nthreads=8)


@pytest.mark.parametrize("precision", [tw.TW_PRECISION_FP64, tw.TW_PRECISION_FP32_CERTIFIED])
def test_smooth_pass_vs_oracle(ctx, oracle, sphere, precision):
    batch = _mixed(sphere, 3000, seed=5)
    xyz, off, tets, ff, cen, kinds = batch
    want, wst = _oracle_pass(oracle, sphere, batch, 1, 8)
    counts = np.bincount(wst, minlength=6)
    assert counts[2] > 500 and counts[4] > 20 and counts[5] > 100, counts
    ctx.set_params(EPS * EPS, EPS / 2, 1, 8)
    ctx.surface_upload(*sphere)
    ctx.mesh_upload(xyz)
    ctx.set_precision(precision)
    try:
        out, st = ctx.smooth_stars(off, tets, cen, ff, kinds)
    finally:
        ctx.set_precision(tw.TW_PRECISION_FP64)
    assert np.array_equal(st.astype(np.int8), wst)
    assert np.array_equal(out, want)


def _large_stars(sphere):
    """Eight surface stars of 400 tets with every face flagged a surface face: 600 faces
    through each centre.  Four stars of radius 2e-4 (inside the envelope: two pass every
    face), four of 4e-3."""
    V, F = sphere
    cp = V[np.random.default_rng(9).choice(len(V), 8, replace=False)]
    parts = [syn.star_batch(4, seed=9 + k, mean_tets=400, lo=400, hi=400, radius=r,
                            centres=cp[4 * k:4 * k + 4], jitter_rel=0.01)
             for k, r in enumerate((2e-4, 4e-3))]
    nv0 = len(parts[0][0])
    xyz = np.vstack([parts[0][0], parts[1][0]])
    off = np.concatenate([parts[0][1], parts[1][1][1:] + parts[0][1][-1]]).astype(np.int32)
    tets = np.vstack([parts[0][2], parts[1][2] + nv0]).astype(np.int32)
    cen = np.concatenate([parts[0][3], parts[1][3] + nv0]).astype(np.int32)
    ff = np.full(len(tets), 15, np.uint8)
    return xyz, off, tets, ff, cen, np.ones(len(cen), np.uint8)


def test_smooth_pass_large_stars(ctx, oracle, sphere):
    batch = _large_stars(sphere)
    xyz, off, tets, ff, cen, kinds = batch
    want, wst = _oracle_pass(oracle, sphere, batch, 1, 8)
    assert (wst == 2).sum() >= 1 and (wst == 5).sum() >= 1, wst
    ctx.set_params(EPS * EPS, EPS / 2, 1, 8)
    ctx.surface_upload(*sphere)
    ctx.mesh_upload(xyz)
    try:
        for precision in (tw.TW_PRECISION_FP64, tw.TW_PRECISION_FP32_CERTIFIED):
            ctx.set_precision(precision)
            out, st = ctx.smooth_stars(off, tets, cen, ff, kinds)
            assert np.array_equal(st.astype(np.int8), wst), precision
            assert np.array_equal(out, want), precision
    finally:
        ctx.set_precision(tw.TW_PRECISION_FP64)


def test_smooth_pass_every_launch_shape(ctx, oracle, sphere):
    batch = _mixed(sphere, 1500, seed=6)
    xyz, off, tets, ff, cen, kinds = batch
    want, wst = _oracle_pass(oracle, sphere, batch, 15, 20)
    ctx.set_params(EPS * EPS, EPS / 2, 15, 20)
    ctx.surface_upload(*sphere)
    ctx.mesh_upload(xyz)
    try:
        for shape in range(ctx.NEWTON_SHAPES):
            ctx.set_newton_shape(shape)
            out, st = ctx.smooth_stars(off, tets, cen, ff, kinds)
            assert np.array_equal(st.astype(np.int8), wst), shape
            assert np.array_equal(out, want), shape
    finally:
        ctx.set_newton_shape(5)


def test_smooth_boundary_stars_use_boundary_surface(ctx, oracle, sphere):
    V, F = sphere
    batch = list(_mixed(sphere, 1000, seed=7))
    kinds = batch[5].copy()
    sel = np.nonzero(kinds == 1)[0][::2]
    kinds[sel] = 2
    batch[5] = kinds
    # boundary surface: the northern half of the sphere
    Fb = F[V[F].mean(1)[:, 2] > 0]
    want, wst = _oracle_pass(oracle, sphere, batch, 1, 8, boundary=(V, Fb))
    xyz, off, tets, ff, cen, _ = batch
    ctx.set_params(EPS * EPS, EPS / 2, 1, 8)
    ctx.surface_upload(V, F)
    ctx.surface_upload(V, Fb, tw.TW_SURFACE_BOUNDARY)
    ctx.mesh_upload(xyz)
    out, st = ctx.smooth_stars(off, tets, cen, ff, kinds)
    assert np.array_equal(st.astype(np.int8), wst)
    assert np.array_equal(out, want)
    assert (wst[kinds == 2] == 2).any()


def test_smooth_boundary_without_boundary_surface_is_an_error(ctx, sphere):
    xyz, off, tets, ff, cen, kinds = _mixed(sphere, 50, seed=8)
    kinds = kinds.copy()
    kinds[-1] = 2
    ctx.surface_upload(*sphere)
    ctx.surface_upload(np.zeros((0, 3)), np.zeros((0, 3), np.int32), tw.TW_SURFACE_BOUNDARY)
    ctx.mesh_upload(xyz)
    with pytest.raises(tw.TetWildGpuError) as e:
        ctx.smooth_stars(off, tets, cen, ff, kinds)
    assert e.value.code == tw.TW_ERR_NO_SURFACE
    with pytest.raises(tw.TetWildGpuError):
        ctx.smooth_stars(off, tets, cen, None, kinds)


def test_smooth_device_graph_replay(ctx, oracle, sphere):
    """Device-pointer pass captured in a CUDA graph and replayed twice."""
    import torch

    batch = _mixed(sphere, 2000, seed=9)
    xyz, off, tets, ff, cen, kinds = batch
    want, wst = _oracle_pass(oracle, sphere, batch, 1, 8)
    ctx.set_params(EPS * EPS, EPS / 2, 1, 8)
    ctx.surface_upload(*sphere)
    ctx.mesh_upload(xyz)
    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in dict(off=off.astype(np.int32), tets=tets.astype(np.int32).reshape(-1),
                          ff=ff.astype(np.uint8), cen=cen.astype(np.int32),
                          kinds=kinds.astype(np.uint8)).items()}
    ns, nt = int(cen.size), int(len(tets))
    d_out = torch.empty(3 * ns, dtype=torch.float64, device=dev)
    d_st = torch.empty(ns, dtype=torch.uint8, device=dev)
    args = (d["off"].data_ptr(), d["tets"].data_ptr(), d["ff"].data_ptr(), d["cen"].data_ptr(),
            d["kinds"].data_ptr(), ns, nt, d_out.data_ptr(), d_st.data_ptr())
    torch.cuda.synchronize()
    ctx.smooth_stars_device(*args)      # sizes the scratch outside the capture
    ctx.synchronize()
    assert np.array_equal(d_st.cpu().numpy().astype(np.int8), wst)
    ctx.capture_begin()
    ctx.smooth_stars_device(*args)
    g = ctx.capture_end()
    for _ in range(2):
        d_out.fill_(0.0)
        d_st.fill_(255)
        torch.cuda.synchronize()
        g.launch()
        ctx.synchronize()
        assert np.array_equal(d_st.cpu().numpy().astype(np.int8), wst)
        assert np.array_equal(d_out.cpu().numpy().reshape(-1, 3), want)
    g.close()


def test_smooth_pass_full_size(ctx, oracle):
    """The bench's star batch at full size: 200,000 stars (half on the 100k-facet
    displaced sphere), Newton max_step 1 / max_it 8 — every status and position
    identical to the oracle in both precision modes."""
    from oracle.oracle import default_threads

    V, F = syn.displaced_sphere(seed=0)
    xyz, off, tets, ff, cen, kinds = syn.mixed_star_batch(V, F, 200_000, EPS, seed=11,
                                                          surface_fraction=0.5)
    S = oracle.surface(V, F)
    want, wst = oracle.smooth_stars(xyz, off, tets, cen, ff, kinds, surface=S, boundary=S,
                                    eps2=EPS * EPS, sd=EPS / 2, max_step=1, max_it=8,
                                    nthreads=default_threads())
    ctx.set_params(EPS * EPS, EPS / 2, 1, 8)
    ctx.surface_upload(V, F)
    ctx.mesh_upload(xyz)
    for precision in (tw.TW_PRECISION_FP64, tw.TW_PRECISION_FP32_CERTIFIED):
        ctx.set_precision(precision)
        try:
            out, st = ctx.smooth_stars(off, tets, cen, ff, kinds)
        finally:
            ctx.set_precision(tw.TW_PRECISION_FP64)
        assert np.array_equal(st.astype(np.int8), wst) and np.array_equal(out, want)
