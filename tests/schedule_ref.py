"""The conflict-free operator batch of tw_schedule_edges, restated as the sequential
greedy pass it must equal: candidates in priority order, each taken when none of its
tets belongs to a candidate taken before it."""
import numpy as np

SPLIT, COLLAPSE = 0, 1


def edges_and_shells(tets):
    """Unique edges (a < b) in ascending order and, per edge, the sorted ids of its tets."""
    shells = {}
    for i, t in enumerate(np.asarray(tets).tolist()):
        for x in range(4):
            for y in range(x + 1, 4):
                e = (min(t[x], t[y]), max(t[x], t[y]))
                shells.setdefault(e, []).append(i)
    edges = sorted(shells)
    return edges, shells


def greedy_schedule(xyz, tets, op, ideal_weight, scale=None):
    """((v1, v2) taken in priority order [m, 2], number of candidates, per taken candidate
    its tets)."""
    tets = np.asarray(tets)
    edges, shells = edges_and_shells(tets)
    stars = [[] for _ in range(len(xyz))]
    for i, t in enumerate(tets.tolist()):
        for v in t:
            stars[v].append(i)
    E = np.array(edges, np.int64).reshape(-1, 2)
    d = xyz[E[:, 0]] - xyz[E[:, 1]]
    w = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    s = np.ones(len(E)) if scale is None else (scale[E[:, 0]] + scale[E[:, 1]]) / 2.0
    thr = ideal_weight * s * s
    cands = []   # (weight, slot, v1, v2)
    for k, (a, b) in enumerate(edges):
        if op == SPLIT and w[k] > thr[k]:
            cands.append((w[k], 2 * k, a, b))
        elif op == COLLAPSE and w[k] < thr[k]:
            cands.append((w[k], 2 * k, a, b))
            cands.append((w[k], 2 * k + 1, b, a))
    if op == SPLIT:
        cands.sort(key=lambda c: (-c[0], c[1]))
    else:
        cands.sort(key=lambda c: (c[0], c[1]))
    used, taken, their = set(), [], []
    for _, slot, v1, v2 in cands:
        ts = shells[(min(v1, v2), max(v1, v2))] if op == SPLIT else stars[v1]
        if used.isdisjoint(ts):
            used.update(ts)
            taken.append((v1, v2))
            their.append(ts)
    return np.array(taken, np.int32).reshape(-1, 2), len(cands), their
