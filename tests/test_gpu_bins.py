"""The point test's bin index (TW_TUNE_BIN_CELL): cubic bins listing their leaves with
a mask of the 8x8x8 fine cells each leaf reaches.  Every decision must equal the oracle's
and the hashed grid's (the index off), in both precision modes: for points at eps (1 -+
1e-7) of random facet points (a leaf dropped from a bin, or a fine-cell bit left clear,
turns such a point out), for every bin size from the 1/250-of-the-box floor to bins
larger than the facets, far from the origin, on a surface whose box is long and flat
(few bins on two axes), outside the box and far away, and with the queries unsorted."""
import numpy as np
import pytest

import tetwild_gb300 as tw
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _both_modes(ctx, fn):
    ctx.set_precision(tw.TW_PRECISION_FP64)
    a = fn()
    ctx.set_precision(tw.TW_PRECISION_FP32_CERTIFIED)
    b = fn()
    ctx.set_precision(tw.TW_PRECISION_FP64)
    return a, b


def _soup(n, size, seed, scale=(1.0, 1.0, 1.0)):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3)) * np.asarray(scale)
    V = (c + (rng.random((n, 3, 3)) - 0.5) * size).reshape(-1, 3)
    return V, np.arange(3 * n, dtype=np.int32).reshape(n, 3)


def _near_points(V, F, eps, n, seed):
    rng = np.random.default_rng(seed)
    f = rng.integers(0, len(F), n)
    w = rng.random((n, 3)) ** 3          # many points near edges and corners
    w /= w.sum(1, keepdims=True)
    X = np.einsum("ij,ijk->ik", w, V[F[f]])
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = eps * np.where(rng.random(n) < 0.5, 1 - 1e-7, 1 + 1e-7)
    return X + d * r[:, None]


def _check(ctx, oracle, V, F, P, eps, factors):
    """Every bin factor (0: the hashed grid), with the sort at its automatic size (a Morton
    prefix of the bins for small batches) and on the full bins."""
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=8)
    ctx.set_params(eps * eps, eps)
    try:
        for b in factors:
            ctx.set_tuning(tw.Context.TUNE_BIN_CELL, b)
            ctx.surface_upload(V, F)
            for sort in (1, 8):
                ctx.set_tuning(tw.Context.TUNE_SORT_POINTS, sort)
                a, c = _both_modes(ctx, lambda: ctx.envelope_points(P))
                assert np.array_equal(a, want), (b, sort)
                assert np.array_equal(c, want), (b, sort)
    finally:
        ctx.set_tuning(tw.Context.TUNE_BIN_CELL, 0.25)
        ctx.set_tuning(tw.Context.TUNE_SORT_POINTS, 1)
    return want


@pytest.mark.parametrize("offset", [0.0, 1000.0])
def test_bins_keep_every_facet_within_reach(ctx, oracle, offset):
    V, F = _soup(3000, 0.05, seed=41)
    V = V + offset
    eps = 2e-3
    P = _near_points(V, F, eps, 60000, seed=42)
    want = _check(ctx, oracle, V, F, P, eps, (0.0, 0.05, 0.25, 1.0, 4.0))
    assert want.sum() < len(P) // 2        # the inner half is in by construction


def test_bins_long_flat_surface(ctx, oracle):
    """A box 100 x 1 x 0.01: the bins are set by the long side (1/250 of it), so the other
    two axes get a few bins (one or two through the thin side)."""
    V, F = _soup(4000, 0.3, seed=43, scale=(100.0, 1.0, 0.01))
    eps = 5e-3
    P = _near_points(V, F, eps, 40000, seed=44)
    _check(ctx, oracle, V, F, P, eps, (0.0, 0.25, 2.0))


def test_bins_points_outside_and_far(ctx, oracle):
    """Points beyond every face of the box (within eps of the outer facets and farther),
    far away, and huge: the clamped bins and fine cells."""
    V, F = syn.icosphere(4)
    eps = 3e-3
    rng = np.random.default_rng(45)
    ring = syn.envelope_points(V, F, 20000, eps, seed=46)   # around the sphere
    axis = np.zeros((6 * 500, 3))
    for k in range(3):
        for s, sgn in enumerate((-1.0, 1.0)):
            blk = slice((2 * k + s) * 500, (2 * k + s + 1) * 500)
            axis[blk] = rng.normal(0, 0.02, (500, 3))
            axis[blk, k] = sgn * (1.0 + rng.uniform(-2 * eps, 2 * eps, 500))
    d = rng.normal(size=(2000, 3))
    far = d / np.linalg.norm(d, axis=1, keepdims=True) * 10.0 ** rng.uniform(0.5, 30, (2000, 1))
    P = np.vstack([ring, axis, far])
    want = _check(ctx, oracle, V, F, P, eps, (0.0, 0.25, 1.0))
    assert want[-2000:].all()
    assert 0 < want[:len(ring) + len(axis)].sum() < len(ring) + len(axis)


def test_bins_unsorted_and_sorted_coarse(ctx, oracle):
    """The same decisions with the queries in the caller's order and with a coarse sort
    (a Morton prefix of the bins)."""
    V, F = syn.displaced_sphere(seed=5)
    eps = 1e-3
    P = syn.envelope_points(V, F, 200_000, eps, seed=47)
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=8)
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    try:
        for knob in (0, 3, 5, 1):
            ctx.set_tuning(tw.Context.TUNE_SORT_POINTS, knob)
            a, c = _both_modes(ctx, lambda: ctx.envelope_points(P))
            assert np.array_equal(a, want), knob
            assert np.array_equal(c, want), knob
    finally:
        ctx.set_tuning(tw.Context.TUNE_SORT_POINTS, 1)


def test_bins_with_many_entries(ctx, oracle):
    """Bins 8x the facet extent on a dense soup: a bin lists more than 32 leaves, so its
    mask words are read in several groups of 32."""
    V, F = _soup(6000, 0.05, seed=48)
    eps = 2e-3
    P = _near_points(V, F, eps, 50000, seed=49)
    _check(ctx, oracle, V, F, P, eps, (8.0, 16.0))


def test_bin_knob_range(ctx):
    for bad in (0.01, -1.0, 100.0):
        with pytest.raises(tw.TetWildGpuError):
            ctx.set_tuning(tw.Context.TUNE_BIN_CELL, bad)
    ctx.set_tuning(tw.Context.TUNE_BIN_CELL, 0.25)


def test_points_in_bins_without_entries(ctx, oracle):
    """Points inside the sphere and around it, in bins that list no leaf: the binning pass
    decides them (out) and counts them as queries; the others take the sorted test."""
    V, F = syn.icosphere(4)
    eps = 2e-3
    rng = np.random.default_rng(50)

    def shell(n, r0, r1):
        d = rng.normal(size=(n, 3))
        return d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(r0, r1, (n, 1))

    P = np.vstack([syn.envelope_points(V, F, 100_000, eps, seed=51), shell(100_000, 0.0, 0.6),
                   shell(100_000, 1.3, 3.0)])
    P = P[rng.permutation(len(P))]
    want = oracle.surface(V, F).points_out(P, eps * eps, nthreads=8)
    ctx.set_params(eps * eps, eps)
    ctx.surface_upload(V, F)
    for prec in (tw.TW_PRECISION_FP64, tw.TW_PRECISION_FP32_CERTIFIED):
        ctx.set_precision(prec)
        ctx.reset_stats()
        try:
            got = ctx.envelope_points(P)
            st = ctx.stats()
        finally:
            ctx.set_precision(tw.TW_PRECISION_FP64)
        assert np.array_equal(got, want), prec
        assert st["env_queries"] == len(P)
    assert want.sum() >= 200_000          # every shell point, and part of the near ones


def test_bins_on_both_surfaces_and_eps_change(ctx, oracle):
    """The input and the boundary surface each get their own index; a new eps2 rebuilds
    both (an index built for another eps2 is never read)."""
    V, F = syn.icosphere(4)
    Vb, Fb = syn.torus(1.0, 0.3, 60, 20)
    P = np.vstack([syn.envelope_points(V, F, 60_000, 3e-3, seed=52),
                   syn.envelope_points(Vb, Fb, 60_000, 3e-3, seed=53)])
    ctx.set_params(1e-6, 1e-3)
    ctx.surface_upload(V, F, tw.TW_SURFACE_INPUT)
    ctx.surface_upload(Vb, Fb, tw.TW_SURFACE_BOUNDARY)
    for eps in (1e-3, 2.5e-3):
        ctx.set_params(eps * eps, eps)
        wi = oracle.surface(V, F).points_out(P, eps * eps, nthreads=8)
        wb = oracle.surface(Vb, Fb).points_out(P, eps * eps, nthreads=8)
        for prec in (tw.TW_PRECISION_FP64, tw.TW_PRECISION_FP32_CERTIFIED):
            ctx.set_precision(prec)
            try:
                gi = ctx.envelope_points(P, tw.TW_SURFACE_INPUT)
                gb = ctx.envelope_points(P, tw.TW_SURFACE_BOUNDARY)
            finally:
                ctx.set_precision(tw.TW_PRECISION_FP64)
            assert np.array_equal(gi, wi), (eps, prec)
            assert np.array_equal(gb, wb), (eps, prec)
        assert 0 < wi.sum() < len(P) and 0 < wb.sum() < len(P)
