"""GPU: tw_swap_check (EdgeRemover::removeAnEdge_32 / _44 / _56 checks) against the oracle on
random shells of every size around their edge, with budgets (the remover's equal_buget),
rings the edge does not pierce, shells of 6 tets and tets not around the edge
(TW_SWAP_SIZE), an unrounded vertex (TW_SWAP_NEEDS_HOST, the call returns
TW_NEEDS_EXACT_HOST), an empty batch, and bad offsets and vertex ids (an error, after which
the context still answers)."""
import numpy as np
import pytest

import tetwild_gb300 as tw
from test_operator_checks import _shell

pytestmark = pytest.mark.gpu


def _batch(cases, seed):
    rng = np.random.default_rng(seed)
    xs, v12, off, tets, budget = [], [], [0], [], []
    base = 0
    for case in range(cases):
        k = int(rng.integers(3, 7))
        xyz, t = _shell(k, h=float(rng.uniform(0.2, 3.0)), jitter=float(rng.uniform(0, 0.4)),
                        radial=float(rng.uniform(0, 0.5)), seed=case,
                        zoff=rng.normal(0, float(rng.uniform(0, 0.8)), k))
        t = t[rng.permutation(k)] + base
        if case % 17 == 0:                      # a tet that is not around the edge
            t[0, t[0] == base + 1] = base + 2
        xs.append(xyz)
        v12.append((base, base + 1))
        tets += t.tolist()
        off.append(off[-1] + k)
        budget.append(int(rng.choice([0, 0, 1, 3])))
        base += len(xyz)
    return (np.vstack(xs), np.array(v12, np.int32), np.array(off, np.int32),
            np.array(tets, np.int32), np.array(budget, np.int32))


def test_swap_random_shells_vs_oracle(ctx, oracle):
    X, v12, off, tets, budget = _batch(600, seed=11)
    ctx.set_precision(tw.TW_PRECISION_FP64)
    ctx.mesh_upload(X)
    r, c, sp = ctx.swap_check(v12, off, tets, budget)
    ro, co, spo = oracle.swap_check(X, v12, off, tets, budget)
    assert np.array_equal(r, ro) and np.array_equal(sp, spo)
    ok = ro == 0
    assert np.array_equal(c[ok], co[ok])
    kinds = set(np.unique(ro).tolist())
    assert {0, 1, 2, 3} <= kinds, kinds


def test_swap_unrounded_empty_and_errors(ctx, oracle):
    X, v12, off, tets, budget = _batch(60, seed=12)
    rounded = np.ones(len(X), np.uint8)
    rounded[v12[5, 0]] = 0                      # an unrounded endpoint of shell 5
    ctx.mesh_upload(X, rounded)
    r, c, sp = ctx.swap_check(v12, off, tets, budget)
    ro, co, spo = oracle.swap_check(X, v12, off, tets, budget)
    assert r[5] == 4
    keep = np.arange(len(r)) != 5
    assert np.array_equal(r[keep], ro[keep])
    ctx.mesh_upload(X)
    e = ctx.swap_check(np.zeros((0, 2), np.int32), np.zeros(1, np.int32),
                       np.zeros((0, 4), np.int32))
    assert all(len(a) == 0 for a in e)
    bad_off = off.copy()
    bad_off[3] = bad_off[4] + 1                  # decreasing offsets
    with pytest.raises(tw.TetWildGpuError) as ex:
        ctx.swap_check(v12, bad_off, tets, budget)
    assert ex.value.code == tw.TW_ERR_ARG
    bad_tets = tets.copy()
    bad_tets[7, 2] = len(X) + 10                 # a vertex id out of range
    with pytest.raises(tw.TetWildGpuError):
        ctx.swap_check(v12, off, bad_tets, budget)
    r2, _, _ = ctx.swap_check(v12, off, tets, budget)   # the context still answers
    assert np.array_equal(r2, ro)
