"""Host logic of the smoothing pass (tetwild_gb300/smoothing.py), on CPU with the oracle as
the batch runner: stars in ascending tet order, a colouring in which no tet holds two
vertices of one colour, CSR star batches, and the claim the batching rests on.  The
reference's VertexSmoother::smooth (VertexSmoother.cpp:19-46) visits the vertices one at a
time, each seeing the moves before it; the stars of one colour share no centre, so running
them as one batch gives exactly the positions and statuses that visiting them one at a time
in the same order gives."""
import math

import numpy as np
import pytest

from tetwild_gb300 import synthetic as syn
from tetwild_gb300.smoothing import KIND_LOCKED, smoothing_pass, star_batch_of


@pytest.fixture(scope="module")
def mesh():
    return syn.icosphere_stage1_mesh(subdiv=2, seed=3)


def test_stars_list_every_tet_in_ascending_order(mesh):
    tets, nv = mesh["tets"], len(mesh["xyz"])
    off, ids = syn.vertex_stars(tets, nv)
    assert off[0] == 0 and off[-1] == 4 * len(tets)
    for v in range(nv):
        want = np.nonzero((tets == v).any(axis=1))[0]
        assert np.array_equal(ids[off[v]:off[v + 1]], want)


def test_colouring_separates_the_vertices_of_every_tet(mesh):
    tets = mesh["tets"]
    colour = syn.greedy_colouring(tets, len(mesh["xyz"]))
    c = np.sort(colour[tets], axis=1)
    assert (colour >= 0).all() and (np.diff(c, axis=1) > 0).all()


def test_star_batches_are_the_centres_stars(mesh):
    tets, ff, nv = mesh["tets"], mesh["face_flags"], len(mesh["xyz"])
    off, ids = syn.vertex_stars(tets, nv)
    centers = np.random.default_rng(0).choice(nv, 40, replace=False).astype(np.int32)
    star_off, st, sf = star_batch_of(centers, tets, ff, off, ids)
    assert star_off[0] == 0 and star_off[-1] == len(st) == len(sf)
    for i, c in enumerate(centers):
        rows = ids[off[c]:off[c + 1]]
        assert np.array_equal(st[star_off[i]:star_off[i + 1]], tets[rows])
        assert np.array_equal(sf[star_off[i]:star_off[i + 1]], ff[rows])
    e = star_batch_of(np.zeros(0, np.int32), tets, ff, off, ids)
    assert e[0].tolist() == [0] and len(e[1]) == 0


def test_colour_batches_equal_one_vertex_at_a_time(mesh, oracle):
    V, F, tets, ff, kind = mesh["V"], mesh["F"], mesh["tets"], mesh["face_flags"], mesh["kind"]
    eps_in = 1e-3 * mesh["diag"]
    sd = eps_in
    eps = eps_in * (1.0 - 1.0 / math.sqrt(3.0))
    eps2 = eps * eps
    S = oracle.surface(V, F)
    xyz = mesh["xyz"] + np.random.default_rng(4).normal(0.0, 0.1 * mesh["edge"],
                                                        mesh["xyz"].shape) * (kind == 0)[:, None]

    def stars(x, off, t, c, f, k):
        return oracle.smooth_stars(x, off, t, c, f, k, surface=S, boundary=S, eps2=eps2, sd=sd,
                                   max_step=15, max_it=20)

    def one_at_a_time(x, off, t, c, f, k):
        x = x.copy()
        pos = np.empty((len(c), 3))
        st = np.empty(len(c), np.int8)
        for i in range(len(c)):
            sl = slice(int(off[i]), int(off[i + 1]))
            p1, s1 = stars(x, np.array([0, off[i + 1] - off[i]], np.int32), t[sl], c[i:i + 1],
                           f[sl], k[i:i + 1])
            pos[i], st[i] = p1[0], s1[0]
            if s1[0] == 2:
                x[c[i]] = p1[0]
        return pos, st

    colour = syn.greedy_colouring(tets, len(xyz))
    xb, lb = smoothing_pass(xyz, tets, ff, kind, stars, colour)
    xs, ls = smoothing_pass(xyz, tets, ff, kind, one_at_a_time, colour)
    assert len(lb.batches) == len(ls.batches) > 2
    for a, b in zip(lb.batches, ls.batches):
        assert np.array_equal(a["centers"], b["centers"])
        assert np.array_equal(a["status"], b["status"]) and np.array_equal(a["pos"], b["pos"])
    assert np.array_equal(xb, xs)
    counts = lb.status_counts()
    assert counts[2] > 20, counts                       # vertices moved
    assert not np.isin(np.concatenate([b["centers"] for b in lb.batches]),
                       np.nonzero(kind == KIND_LOCKED)[0]).any()
    assert {b["phase"] for b in lb.batches} == {"single", "surface"}
