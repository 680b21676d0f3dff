"""The small plain-method case: TetWild's query calls on the jittered icosphere
(subdivision 3, radius 1, N(0, 1e-3) radial jitter, -l 0.05, -e 1e-3 of the
bounding-box diagonal), replayed through the plain FP64 GPU kernels and the
oracle side by side.

The reference CLI cannot be built here (CGAL, geogram, libigl), so its call
log cannot be recorded; the stand-in is the query traffic of two smoothing
passes over a stage-1 mesh of the same input (``icosphere_stage1_mesh``):
every batch of stars (validity, Newton E/J/H, inversion checks, projection,
quality, face envelope), then the full-mesh calTetQualities sweep, the
envelope test of every surface face and of every surface vertex; and the
checks of the other operators on every candidate of that mesh (checks only,
not applied): each edge split (EdgeSplitter::splitAnEdge, EdgeSplitter.cpp
:222-225: calTetQualities and isFlip of the new tets at the midpoint), each
edge collapse in both directions (EdgeCollapser::collapseAnEdge, :284-446,
with isCollapsable_epsilon :727-775) and each edge removal of a shell of 3,
4 or 5 tets (EdgeRemover::removeAnEdge_32 / _44 / _56, :125-600).  Every
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


def _edge_shells(tets):
    """{(a, b): sorted ids of the tets around the edge} over all edges, a < b."""
    shells = {}
    for i, t in enumerate(tets.tolist()):
        for x in range(4):
            for y in range(x + 1, 4):
                e = (min(t[x], t[y]), max(t[x], t[y]))
                shells.setdefault(e, []).append(i)
    return shells


def test_icosphere_operator_checks_plain_fp64(ctx, oracle):
    m = syn.icosphere_stage1_mesh()
    V, F, tets, ff, kind, xyz = m["V"], m["F"], m["tets"], m["face_flags"], m["kind"], m["xyz"]
    eps_in = 1e-3 * m["diag"]
    sd = eps_in
    eps = eps_in * (1.0 - 1.0 / math.sqrt(3.0))
    eps2 = eps * eps
    ctx.set_params(eps2, sd, 15, 20)
    ctx.set_precision(0)
    ctx.surface_upload(V, F)
    S = oracle.surface(V, F)
    shells = _edge_shells(tets)
    edges = sorted(shells)
    counts = {}

    # splits: the new tets of every edge with the midpoint appended as a vertex
    nv = len(xyz)
    mids = np.array([(xyz[a] + xyz[b]) / 2 for a, b in edges])
    big = np.vstack([xyz, mids])
    new_tets, owner = [], []
    for k, (a, b) in enumerate(edges):
        v = nv + k
        for ti in shells[(a, b)]:
            t = tets[ti].tolist()
            t1, t2 = list(t), list(t)
            t1[t1.index(b)] = v
            t2[t2.index(a)] = v
            new_tets += [t1, t2]
            owner += [k, k]
    new_tets = np.array(new_tets, np.int32)
    ctx.mesh_upload(big)
    E, Fl, N, _ = ctx.tet_quality(new_tets)
    T = np.ascontiguousarray(big[new_tets].reshape(-1, 12).T)
    Eo, _, _, Flo = oracle.amips_batch_soa(T, quality=True, nthreads=8, jacobian=False,
                                           hessian=False)
    assert np.array_equal(E, Eo) and np.array_equal(Fl, Flo)
    split_flip = np.zeros(len(edges), bool)
    np.logical_or.at(split_flip, np.array(owner), Fl.astype(bool))
    counts["split"] = (len(edges), int(split_flip.sum()))

    # collapses v1 -> v2 in both directions: the star of v1, vertex flags by kind
    ctx.mesh_upload(xyz)
    conn = [[] for _ in range(nv)]
    for i, t in enumerate(tets.tolist()):
        for v in t:
            conn[v].append(i)
    v12, flags, off, st_tets, st_ff = [], [], [0], [], []
    for a, b in edges:
        for v1, v2 in ((a, b), (b, a)):
            if kind[v1] == 3:
                continue                                   # locked box corners
            v12.append((v1, v2))
            flags.append((1 if kind[v1] == 1 else 0) | (4 if kind[v2] == 1 else 0))
            st_tets += [tets[i] for i in conn[v1]]
            st_ff += [ff[i] for i in conn[v1]]
            off.append(off[-1] + len(conn[v1]))
    v12 = np.array(v12, np.int32)
    flags = np.array(flags, np.uint8)
    off = np.array(off, np.int32)
    st_tets = np.array(st_tets, np.int32)
    st_ff = np.array(st_ff, np.uint8)
    got = ctx.collapse_check(v12, flags, off, st_tets, st_ff)
    want = oracle.collapse_check(xyz, off, st_tets, st_ff, v12, flags, surface=S, boundary=S,
                                 eps2=eps2, sd=sd, nthreads=8)
    assert np.array_equal(got, want)
    counts["collapse"] = np.bincount(want, minlength=4).tolist()

    # edge removals: every edge with a shell of 3, 4 or 5 tets, budgets 0 / 1 / 100
    cand = [e for e in edges if 3 <= len(shells[e]) <= 5]
    sv12 = np.array(cand, np.int32)
    soff = np.concatenate([[0], np.cumsum([len(shells[e]) for e in cand])]).astype(np.int32)
    stets = np.array([tets[i] for e in cand for i in shells[e]], np.int32)
    budget = np.random.default_rng(3).choice([0, 0, 1, 100], len(cand)).astype(np.int32)
    r, c, sp = ctx.swap_check(sv12, soff, stets, budget)
    ro, co, spo = oracle.swap_check(xyz, sv12, soff, stets, budget)
    assert np.array_equal(r, ro) and np.array_equal(sp, spo)
    ok = ro == 0
    assert np.array_equal(c[ok], co[ok])
    counts["swap"] = {k: np.bincount(ro[soff[1:] - soff[:-1] == k], minlength=4).tolist()
                      for k in (3, 4, 5)}
    print("operator checks:", counts)
    assert counts["split"][0] > 10000 and sum(counts["collapse"]) > 20000
    assert all(counts["swap"][k][0] > 0 for k in (3, 4, 5))
