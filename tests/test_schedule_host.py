"""CPU: the conflict-free operator batch (the greedy pass that tw_schedule_edges must
equal) on the icosphere stage-1 mesh: no two chosen operations share a tet, every
candidate left out shares a tet with an earlier chosen one, and the order is the
priority order (splits longest first, collapses shortest first)."""
import numpy as np
import pytest

from schedule_ref import COLLAPSE, SPLIT, edges_and_shells, greedy_schedule
from tetwild_gb300 import synthetic as syn


@pytest.fixture(scope="module")
def mesh():
    return syn.icosphere_stage1_mesh()


@pytest.mark.parametrize("op", [SPLIT, COLLAPSE])
def test_batch_is_conflict_free_and_maximal(mesh, op):
    xyz, tets = mesh["xyz"], mesh["tets"]
    L = 0.05 * mesh["diag"]
    taken, ncand, their = greedy_schedule(xyz, tets, op, L * L)
    assert ncand > 1000 and len(taken) > 100
    seen = {}
    for k, ts in enumerate(their):
        for t in ts:
            assert t not in seen, (k, seen.get(t))
            seen[t] = k
    # maximal: every candidate not taken meets a taken one
    edges, shells = edges_and_shells(tets)
    stars = [[] for _ in range(len(xyz))]
    for i, t in enumerate(tets.tolist()):
        for v in t:
            stars[v].append(i)
    taken_set = {tuple(x) for x in taken.tolist()}
    d = xyz[np.array(edges)[:, 0]] - xyz[np.array(edges)[:, 1]]
    w = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    for k, (a, b) in enumerate(edges):
        dirs = [(a, b)] if op == SPLIT else [(a, b), (b, a)]
        if not (w[k] > L * L if op == SPLIT else w[k] < L * L):
            continue
        for v1, v2 in dirs:
            if (v1, v2) in taken_set:
                continue
            ts = shells[(a, b)] if op == SPLIT else stars[v1]
            assert any(t in seen for t in ts), (v1, v2)
    # priority order
    lt = taken.astype(np.int64)
    dl = xyz[lt[:, 0]] - xyz[lt[:, 1]]
    wl = (dl[:, 0] * dl[:, 0] + dl[:, 1] * dl[:, 1]) + dl[:, 2] * dl[:, 2]
    assert np.all(np.diff(wl) <= 0) if op == SPLIT else np.all(np.diff(wl) >= 0)
