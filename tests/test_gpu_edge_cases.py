"""Empty batches through every batched entry point, in both precision modes:
empty results, no error, and the context still answers the next call (the
reference's loops simply run zero times)."""
import numpy as np
import pytest

import tetwild_gb300 as tw
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

MODES = [tw.TW_PRECISION_FP64, tw.TW_PRECISION_FP32_CERTIFIED]


@pytest.fixture(scope="module")
def setup():
    V, F = syn.icosphere(3)
    eps = 2e-3
    xyz, off, tets, ff, cen, kinds = syn.mixed_star_batch(V, F, 40, eps, seed=8)
    return V, F, eps, xyz, off, tets, ff, cen, kinds


@pytest.mark.parametrize("precision", MODES)
def test_empty_batches(ctx, oracle, setup, precision):
    V, F, eps, xyz, off, tets, ff, cen, kinds = setup
    ctx.set_params(eps * eps, eps / 2, 1, 8)
    ctx.surface_upload(V, F)
    ctx.mesh_upload(xyz)
    ctx.set_precision(precision)
    try:
        assert ctx.envelope_points(np.zeros((0, 3))).shape == (0,)
        assert ctx.envelope_faces(np.zeros((0, 9))).shape == (0,)
        Q, D, Fi = ctx.nearest_points(np.zeros((0, 3)))
        assert Q.shape == (0, 3) and D.shape == (0,) and Fi.shape == (0,)
        g = ctx.amips(np.zeros((12, 0)))
        assert g["E"].shape == (0,) and g["flip"].shape == (0,)
        E, Fl, N, st = ctx.tet_quality(np.zeros((0, 4), np.int32))
        assert E.shape == (0,) and st == tw.TW_OK
        pos, moved = ctx.newton_stars(np.zeros(1, np.int32), np.zeros((0, 4), np.int32),
                                      np.zeros(0, np.int32))
        assert pos.shape == (0, 3) and moved.shape == (0,)
        pos, status = ctx.smooth_stars(np.zeros(1, np.int32), np.zeros((0, 4), np.int32),
                                       np.zeros(0, np.int32), np.zeros(0, np.uint8),
                                       np.zeros(0, np.uint8))
        assert pos.shape == (0, 3) and status.shape == (0,)
        codes = ctx.collapse_check(np.zeros((0, 2), np.int32), np.zeros(0, np.uint8),
                                   np.zeros(1, np.int32), np.zeros((0, 4), np.int32),
                                   np.zeros(0, np.uint8))
        assert codes.shape == (0,)
        a, m, m2, buckets = ctx.energy_stats(np.zeros((0, 4), np.int32))
        wa, wm, wm2, wb = oracle.energy_stats(xyz, np.zeros((0, 4), np.int32))
        assert (np.isnan(a) and np.isnan(wa)) or a == wa      # 0 / 0, as the reference
        assert m == wm and m2 == wm2 and np.array_equal(buckets, wb)
        # the context still answers: one star batch against the oracle
        got, st2 = ctx.smooth_stars(off, tets, cen, ff, kinds)
        S = oracle.surface(V, F)
        want, wst = oracle.smooth_stars(xyz, off, tets, cen, ff, kinds, surface=S, boundary=S,
                                        eps2=eps * eps, sd=eps / 2, max_step=1, max_it=8)
        assert np.array_equal(st2.astype(np.int8), wst) and np.array_equal(got, want)
    finally:
        ctx.set_precision(tw.TW_PRECISION_FP64)


def test_server_empty_requests(setup):
    V, F, eps, xyz, off, tets, ff, cen, kinds = setup
    with tw.Server(0, 0, lanes=2) as srv:
        j = srv.job_open(V, F, eps * eps, eps / 2)
        srv.job_mesh(j, xyz)
        t1, out = srv.submit_points(j, np.zeros((0, 3)))
        t2, outf = srv.submit_faces(j, np.zeros((0, 9)))
        t3, res = srv.submit_amips(j, np.zeros((12, 0)))
        for t in (t1, t2, t3):
            srv.wait(t)
        assert out.shape == (0,) and outf.shape == (0,) and res[0].shape == (0,)
        t4, P_out = srv.submit_points(j, syn.envelope_points(V, F, 1000, eps, seed=2))
        srv.wait(t4)
        assert P_out.shape == (1000,)


def test_errors_leave_the_context_usable(ctx, oracle, setup):
    """Rejected calls report their error and the next call answers correctly: ids out of
    range in every index-based entry point, a face beyond the per-row sample bound (the
    kernel flags it before sampling), a query without a surface."""
    V, F, eps, xyz, off, tets, ff, cen, kinds = setup
    nv = len(xyz)
    with tw.Context(0) as c:
        with pytest.raises(tw.TetWildGpuError) as e:
            c.envelope_points(np.zeros((4, 3)))
        assert e.value.code == tw.TW_ERR_NO_SURFACE
        c.set_params(eps * eps, eps / 2, 1, 8)
        c.surface_upload(V, F)
        c.mesh_upload(xyz)
        bad = tets.copy()
        bad[-1, 2] = nv + 7
        calls = [
            lambda: c.tet_quality(bad),
            lambda: c.newton_stars(off, bad, cen),
            lambda: c.smooth_stars(off, bad, cen, ff, kinds),
            lambda: c.energy_stats(bad),
            lambda: c.collapse_check(np.array([[0, nv + 3]], np.int32), np.zeros(1, np.uint8),
                                     np.array([0, 1], np.int32), tets[:1], ff[:1]),
        ]
        for call in calls:
            with pytest.raises(tw.TetWildGpuError) as e:
                call()
            assert e.value.code == tw.TW_ERR_ARG
        # one face with edges of 1e4 at sampling distance eps/2: far beyond 4e6 samples a row
        huge = np.array([[0.0, 0, 0, 1e4, 0, 0, 0, 1e4, 0]])
        fine = np.hstack([V[F[:50, 0]], V[F[:50, 1]], V[F[:50, 2]]])
        for prec in MODES:
            c.set_precision(prec)
            with pytest.raises(tw.TetWildGpuError) as e:
                c.envelope_faces(np.vstack([fine, huge]))
            assert e.value.code == tw.TW_ERR_ARG and "sample bound" in str(e.value)
            assert np.array_equal(c.envelope_faces(fine),
                                  oracle.surface(V, F).faces_out(fine, eps * eps, eps / 2))
        got, st = c.smooth_stars(off, tets, cen, ff, kinds)
        S = oracle.surface(V, F)
        want, wst = oracle.smooth_stars(xyz, off, tets, cen, ff, kinds, surface=S, boundary=S,
                                        eps2=eps * eps, sd=eps / 2, max_step=1, max_it=8)
        assert np.array_equal(st.astype(np.int8), wst) and np.array_equal(got, want)


def test_reference_named_mirror(ctx, oracle, setup):
    """tetwild_gb300.LocalOperations / VertexSmoother: every method under its reference
    name answers as the oracle does."""
    V, F, eps, xyz, off, tets, ff, cen, kinds = setup
    ctx.set_params(eps * eps, eps / 2, 15, 20)
    ctx.surface_upload(V, F)
    ctx.surface_upload(V, F, tw.TW_SURFACE_BOUNDARY)
    ops = tw.LocalOperations(ctx, xyz)
    T = np.ascontiguousarray(xyz[tets].reshape(-1, 12))
    E, J, H, Fl = oracle.amips_batch_soa(T.T.copy(), quality=False)
    assert np.array_equal(ops.comformalAMIPSEnergy_new(T), E)
    assert np.array_equal(ops.comformalAMIPSJacobian_new(T), J.T)
    assert np.array_equal(ops.comformalAMIPSHessian_new(T), H.T)
    Eq, _, _, Fq = oracle.amips_batch_soa(T.T.copy(), quality=True)
    assert np.array_equal(ops.calTetQualities(tets), Eq)
    assert ops.isFlip(tets) == bool(Fq.any()) and ops.isTetFlip(tets[0]) == bool(Fq[0])
    S = oracle.surface(V, F)
    P = syn.envelope_points(V, F, 64, eps, seed=4)
    want = S.points_out(P, eps * eps)
    assert [ops.isPointOutEnvelop(p) for p in P] == [bool(w) for w in want]
    assert [ops.isPointOutBoundaryEnvelop(p) for p in P[:8]] == [bool(w) for w in want[:8]]
    tri = np.hstack([V[F[:6, 0]], V[F[:6, 1]], V[F[:6, 2]]])
    wf = S.faces_out(tri, eps * eps, eps / 2)
    assert [ops.isFaceOutEnvelop(t) for t in tri] == [bool(w) for w in wf]
    a, m = ops.getAvgMaxEnergy(tets)
    wa, wm, wm2, wb = oracle.energy_stats(xyz, tets)
    assert m == wm and abs(a - wa) <= 1e-12 * abs(wa)
    assert ops.getMaxEnergy(tets) == wm and ops.getSecondMaxEnergy(tets) == wm2
    assert ops.getFilterEnergy(tets) == oracle.filter_energy(wb)
    mins, maxs = ops.calTetQuality_AD(tets)
    _, _, wmins, wmaxs = oracle.dihedral_stats(xyz, tets)
    assert np.allclose(mins, wmins, rtol=4 * 2.0 ** -52) and np.allclose(maxs, wmaxs, rtol=4 * 2.0 ** -52)
    vs = tw.VertexSmoother(ctx, xyz)
    inner = np.nonzero(kinds == 0)[0]
    so = np.concatenate([[0], np.cumsum(np.diff(off)[inner])]).astype(np.int32)
    st = np.concatenate([tets[off[i]:off[i + 1]] for i in inner])
    pos, moved = vs.NewtonsMethod(so, st, cen[inner])
    wpos, wmoved = oracle.newton_stars(xyz, so, st, cen[inner])
    assert np.array_equal(pos, wpos) and np.array_equal(moved, wmoved)
