"""The small plain-method case: TetWild's query calls on the jittered icosphere
(subdivision 3, radius 1, N(0, 1e-3) radial jitter, -l 0.05, -e 1e-3 of the
bounding-box diagonal), replayed through the plain FP64 GPU kernels and the
oracle side by side.

The reference CLI cannot be built here (CGAL, geogram, libigl), so its call
log cannot be recorded; the stand-in is the query traffic of two smoothing
passes over a stage-1 mesh of the same input (``icosphere_stage1_mesh``):
every batch of stars (validity, Newton E/J/H, inversion checks, projection,
quality, face envelope), then the full-mesh calTetQualities sweep, the
envelope test of every surface face and of every surface vertex.  Every
result must be identical.
"""
import math

import numpy as np
import pytest

from tetwild_gb300 import synthetic as syn
from tetwild_gb300.smoothing import device_runner, smoothing_pass

pytestmark = pytest.mark.gpu


def _surface_faces(xyz, tets, ff):
    tris = set()
    for j in range(4):
        rows = np.nonzero((ff >> j) & 1)[0]
        for i in rows:
            tris.add(tuple(sorted(int(x) for x in np.delete(tets[i], j))))
    tris = np.array(sorted(tris), np.int64)
    return xyz[tris].reshape(-1, 9)


def test_icosphere_replay_plain_fp64(ctx, oracle):
    m = syn.icosphere_stage1_mesh()
    assert m["coverage"] == 1.0
    V, F, tets, ff, kind = m["V"], m["F"], m["tets"], m["face_flags"], m["kind"]
    eps_in = 1e-3 * m["diag"]
    sd = eps_in                                  # stage 1 (State.cpp:38)
    eps = eps_in * (1.0 - 1.0 / math.sqrt(3.0))   # State.cpp:39, sub_stage 1
    eps2 = eps * eps
    ctx.set_params(eps2, sd, 15, 20)
    ctx.set_precision(0)
    ctx.surface_upload(V, F)
    ctx.mesh_upload(m["xyz"])
    S = oracle.surface(V, F)

    def oracle_run(xyz, off, t, c, f, k):
        return oracle.smooth_stars(xyz, off, t, c, f, k, surface=S, boundary=S, eps2=eps2, sd=sd,
                                   max_step=15, max_it=20, nthreads=8)

    colour = syn.greedy_colouring(tets, len(m["xyz"]))
    xo = xg = m["xyz"]
    calls = 0
    for _ in range(2):
        xo, lo = smoothing_pass(xo, tets, ff, kind, oracle_run, colour)
        xg, lg = smoothing_pass(xg, tets, ff, kind, device_runner(ctx), colour)
        assert len(lo.batches) == len(lg.batches)
        for a, b in zip(lo.batches, lg.batches):
            assert np.array_equal(a["centers"], b["centers"])
            assert np.array_equal(a["status"].astype(np.int64), b["status"].astype(np.int64))
            assert np.array_equal(a["pos"], b["pos"])
        assert np.array_equal(xo, xg)
        counts = lg.status_counts()
        assert counts[2] > 100, counts
        calls += lg.stars
        # full-mesh sweeps on the new positions
        E, Fl, N, _ = ctx.tet_quality(tets)
        T = np.ascontiguousarray(xg[tets].reshape(-1, 12).T)
        Eo, _, _, Flo = oracle.amips_batch_soa(T, quality=True, nthreads=8, jacobian=False,
                                               hessian=False)
        assert np.array_equal(E, Eo) and np.array_equal(Fl, Flo)
        tris = _surface_faces(xg, tets, ff)
        assert np.array_equal(ctx.envelope_faces(tris), S.faces_out(tris, eps2, sd, nthreads=8))
        P = xg[kind == 1]
        assert np.array_equal(ctx.envelope_points(P), S.points_out(P, eps2, nthreads=8))
        calls += len(tets) + len(tris) + len(P)
    assert calls > 20000
