"""GPU parity of the edge-collapse checks (EdgeCollapser::collapseAnEdge,
EdgeCollapser.cpp:284-446, with isCollapsable_epsilon :727-775) against the
oracle: every result code identical, in both precision modes."""
import math

import numpy as np
import pytest

import tetwild_gb300 as tw
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _candidates(m, rng, frac=1.0):
    xyz, tets, ff, kind = m["xyz"], m["tets"], m["face_flags"], m["kind"]
    off, ids = syn.vertex_stars(tets, len(xyz))
    E = set()
    for t in tets:
        for a in range(4):
            for b in range(4):
                if a != b:
                    E.add((int(t[a]), int(t[b])))
    E = np.array(sorted(E), np.int32)
    E = E[kind[E[:, 0]] != 3]
    if frac < 1.0:
        E = E[rng.random(len(E)) < frac]
    star_off = np.concatenate([[0], np.cumsum(off[E[:, 0] + 1] - off[E[:, 0]])]).astype(np.int32)
    st = np.concatenate([tets[ids[off[v]:off[v + 1]]] for v in E[:, 0]])
    sff = np.concatenate([ff[ids[off[v]:off[v + 1]]] for v in E[:, 0]])
    flags = ((kind[E[:, 0]] == 1) * tw.TW_CV_V1_SURFACE |
             (kind[E[:, 1]] == 1) * tw.TW_CV_V2_SURFACE).astype(np.uint8)
    return E, star_off, st, sff, flags


@pytest.mark.parametrize("precision", [tw.TW_PRECISION_FP64, tw.TW_PRECISION_FP32_CERTIFIED])
def test_collapse_checks_icosphere(ctx, oracle, precision):
    m = syn.icosphere_stage1_mesh()
    rng = np.random.default_rng(1)
    E, off, st, sff, flags = _candidates(m, rng)
    # a few v1s flagged unrounded, and one degenerate edge (v2 moved onto v1)
    flags = flags.copy()
    flags[rng.random(len(flags)) < 0.02] |= tw.TW_CV_V1_UNROUNDED
    xyz = m["xyz"].copy()
    eps_in = 1e-3 * m["diag"]
    eps = eps_in * (1.0 - 1.0 / math.sqrt(3.0))
    S = oracle.surface(m["V"], m["F"])
    ctx.set_params(eps * eps, eps_in, 15, 20)
    ctx.surface_upload(m["V"], m["F"])
    ctx.mesh_upload(xyz)
    ctx.set_precision(precision)
    try:
        for quality, soft in ((True, -1.0), (False, -1.0), (True, 6.0)):
            got = ctx.collapse_check(E, flags, off, st, sff, quality, soft)
            want = oracle.collapse_check(xyz, off, st, sff, E, flags, surface=S, boundary=S,
                                         eps2=eps * eps, sd=eps_in, check_quality=quality,
                                         soft_energy=soft, nthreads=8)
            assert np.array_equal(got, want), (quality, soft)
            counts = np.bincount(want, minlength=4)
            if quality and soft < 0:
                assert (counts > 0).all(), counts
            elif not quality:
                assert counts[2] == 0
    finally:
        ctx.set_precision(tw.TW_PRECISION_FP64)


def test_collapse_degenerate_edge_and_boundary(ctx, oracle):
    m = syn.icosphere_stage1_mesh(seed=3)
    rng = np.random.default_rng(2)
    E, off, st, sff, flags = _candidates(m, rng, frac=0.3)
    xyz = m["xyz"].copy()
    # v2 of the first candidate moved onto v1: a degenerate edge
    xyz[E[0, 1]] = xyz[E[0, 0]]
    flags = flags.copy()
    sel = rng.random(len(flags)) < 0.2
    flags[sel] |= tw.TW_CV_V1_BOUNDARY        # boundary v1 with a boundary surface
    V, F = m["V"], m["F"]
    Fb = F[V[F].mean(1)[:, 2] > 0.0]
    eps = 2e-3
    S, B = oracle.surface(V, F), oracle.surface(V, Fb)
    ctx.set_params(eps * eps, eps, 15, 20)
    ctx.surface_upload(V, F)
    ctx.surface_upload(V, Fb, tw.TW_SURFACE_BOUNDARY)
    ctx.mesh_upload(xyz)
    got = ctx.collapse_check(E, flags, off, st, sff)
    want = oracle.collapse_check(xyz, off, st, sff, E, flags, surface=S, boundary=B,
                                 eps2=eps * eps, sd=eps, nthreads=8)
    assert np.array_equal(got, want)


def test_energy_sweeps_vs_oracle(ctx, oracle):
    """getAvgMaxEnergy / getMaxEnergy / getSecondMaxEnergy / getFilterEnergy's
    histogram over the whole mesh: max, second max and buckets exact, the
    average within 1e-12 relative (the reference sums sequentially)."""
    m = syn.icosphere_stage1_mesh(seed=5)
    xyz = m["xyz"].copy()
    tets = m["tets"]
    rng = np.random.default_rng(4)
    # some inverted and near-flat tets for the sentinel and the upper buckets
    xyz += rng.normal(0.0, 0.02 * m["edge"], xyz.shape)
    locked = (rng.random(len(tets)) < 0.05).astype(np.uint8)
    ctx.mesh_upload(xyz)
    for lk in (None, locked):
        for thres in (10.0, 8.0):
            a, mx, m2, b = ctx.energy_stats(tets, lk, thres)
            ao, mxo, m2o, bo = oracle.energy_stats(xyz, tets, lk, thres)
            assert mx == mxo and m2 == m2o and np.array_equal(b, bo)
            assert abs(a - ao) <= 1e-12 * abs(ao)
            assert ctx.filter_energy(b, thres) == oracle.filter_energy(bo, thres)


def test_dihedral_sweep_vs_oracle(ctx, oracle):
    """calTetQuality_AD over the whole mesh and outputInfo's statistics: per-tet angles
    within 4 ulp (CUDA's acos against the host's), degenerate tets (0, pi) exactly,
    extremes within 4 ulp, means within 1e-12, threshold counts identical."""
    m = syn.icosphere_stage1_mesh(seed=6)
    xyz = m["xyz"].copy()
    tets = m["tets"].copy()
    rng = np.random.default_rng(9)
    xyz += rng.normal(0.0, 0.05 * m["edge"], xyz.shape)     # slivers and caps
    flat = rng.choice(len(tets), 20, replace=False)
    tets[flat, 3] = tets[flat, 2]                             # repeated vertex: degenerate
    locked = (rng.random(len(tets)) < 0.05).astype(np.uint8)
    ctx.mesh_upload(xyz)
    for lk in (None, locked):
        out, cnt, mins, maxs = ctx.dihedral_stats(tets, lk, per_tet=True)
        wout, wcnt, wmins, wmaxs = oracle.dihedral_stats(xyz, tets, lk)
        assert np.array_equal(mins[flat], np.zeros(20)) and np.all(maxs[flat] == math.pi)
        assert np.allclose(mins, wmins, rtol=4 * 2.0 ** -52, atol=1e-300)
        assert np.allclose(maxs, wmaxs, rtol=4 * 2.0 ** -52, atol=1e-300)
        assert np.array_equal(cnt, wcnt) and cnt[6] == (len(tets) - (lk.sum() if lk is not None else 0))
        assert abs(out[0] - wout[0]) <= 4 * 2.0 ** -52 * wout[0] + 1e-300
        assert abs(out[2] - wout[2]) <= 4 * 2.0 ** -52 * wout[2]
        assert abs(out[1] - wout[1]) <= 1e-12 * wout[1] and abs(out[3] - wout[3]) <= 1e-12 * wout[3]
    out, cnt, mins, maxs = ctx.dihedral_stats(tets[:0])
    assert cnt[6] == 0 and out[0] == 10.0 and out[2] == 0.0 and mins is None
