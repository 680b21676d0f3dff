"""GPU: operator candidates and their conflict-free batch built on the device
(tw_schedule_edges) on the icosphere stage-1 mesh, for splits and collapses, with and
without per-vertex scales: the batch equals the sequential greedy pass in priority order
(tests/schedule_ref.py), no two chosen operations share a tet, and each chosen
operation's checks (tw_collapse_check for collapses; calTetQualities and isFlip of the
new tets at the midpoint through tw_tet_quality for splits) equal the oracle's."""
import math

import numpy as np
import pytest

import tetwild_gb300 as tw
from schedule_ref import COLLAPSE, SPLIT, greedy_schedule
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mesh():
    return syn.icosphere_stage1_mesh()


@pytest.mark.parametrize("op", [SPLIT, COLLAPSE])
@pytest.mark.parametrize("scaled", [False, True])
def test_device_schedule_equals_greedy(ctx, oracle, mesh, op, scaled):
    xyz, tets, ff, kind = mesh["xyz"], mesh["tets"], mesh["face_flags"], mesh["kind"]
    L = 0.05 * mesh["diag"]
    scale = (np.random.default_rng(4).uniform(0.6, 1.4, len(xyz)) if scaled else None)
    ctx.mesh_upload(xyz)
    got, ncand = ctx.schedule_edges(tets, op, L * L, scale)
    want, wcand, their = greedy_schedule(xyz, tets, op, L * L, scale)
    assert ncand == wcand and np.array_equal(got, want)
    seen = set()
    for ts in their:
        assert seen.isdisjoint(ts)
        seen.update(ts)
    eps_in = 1e-3 * mesh["diag"]
    eps = eps_in * (1.0 - 1.0 / math.sqrt(3.0))
    ctx.set_params(eps * eps, eps_in, 15, 20)
    ctx.surface_upload(mesh["V"], mesh["F"])
    S = oracle.surface(mesh["V"], mesh["F"])
    if op == COLLAPSE:
        keep = kind[got[:, 0]] != 3                        # box corners stay
        v12 = got[keep]
        flags = ((kind[v12[:, 0]] == 1) * 1 | (kind[v12[:, 1]] == 1) * 4).astype(np.uint8)
        stars = [[] for _ in range(len(xyz))]
        for i, t in enumerate(tets.tolist()):
            for v in t:
                stars[v].append(i)
        off = np.concatenate([[0], np.cumsum([len(stars[a]) for a, _ in v12])]).astype(np.int32)
        st = np.array([tets[i] for a, _ in v12 for i in stars[a]], np.int32)
        sff = np.array([ff[i] for a, _ in v12 for i in stars[a]], np.uint8)
        r = ctx.collapse_check(v12, flags, off, st, sff)
        ro = oracle.collapse_check(xyz, off, st, sff, v12, flags, surface=S, boundary=S,
                                   eps2=eps * eps, sd=eps_in, nthreads=8)
        assert np.array_equal(r, ro)
        assert (ro == 0).sum() > 0
    else:
        nv = len(xyz)
        big = np.vstack([xyz, (xyz[got[:, 0]] + xyz[got[:, 1]]) / 2])
        new = []
        for k, (a, b) in enumerate(got.tolist()):
            for t in tets[np.isin(tets, [a, b]).sum(1) == 2]:
                t1, t2 = t.tolist(), t.tolist()
                t1[t1.index(b)] = nv + k
                t2[t2.index(a)] = nv + k
                new += [t1, t2]
        new = np.array(new, np.int32)
        ctx.mesh_upload(big)
        E, Fl, _, _ = ctx.tet_quality(new)
        T = np.ascontiguousarray(big[new].reshape(-1, 12).T)
        Eo, _, _, Flo = oracle.amips_batch_soa(T, quality=True, nthreads=8, jacobian=False,
                                               hessian=False)
        assert np.array_equal(E, Eo) and np.array_equal(Fl, Flo)


def test_schedule_edge_cases(ctx):
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]])
    ctx.mesh_upload(xyz)
    t = np.array([[0, 1, 2, 3]], np.int32)
    got, nc = ctx.schedule_edges(t, tw.TW_OP_SPLIT, 1.5)
    assert nc == 3 and len(got) == 1                     # the edges of length sqrt2, one tet
    assert np.array_equal(got[0], [1, 2])                # equal lengths in edge order
    got, nc = ctx.schedule_edges(t, tw.TW_OP_SPLIT, 10.0)
    assert nc == 0 and len(got) == 0
    got, nc = ctx.schedule_edges(t, tw.TW_OP_COLLAPSE, 10.0)
    assert nc == 12 and len(got) == 1                    # one tet: one operation
    with pytest.raises(tw.TetWildGpuError):
        ctx.schedule_edges(np.array([[0, 1, 2, 9]], np.int32), tw.TW_OP_SPLIT, 0.5)
    got, nc = ctx.schedule_edges(t, tw.TW_OP_SPLIT, 1.5)   # the context still works
    assert nc == 3
