"""CPU tests of the oracle's edge-removal checks (EdgeRemover::removeAnEdge_32 / _44 / _56,
EdgeRemover.cpp:125-177, :277-369, :456-600): known answers on shells around a vertical
edge, the remover's equal-energy budget, and agreement with a second, independently written
restatement (below, in Python, over exact orientation signs and the oracle's pinned AMIPS
energies) on random shells.  The reference's operators cannot be compiled here (they need
its whole mesh state, CGAL and geogram), so these checks are pinned through their parts
(orientation, AMIPS) and by the two restatements agreeing."""
import numpy as np
import pytest

SUCCESS, FLIP, QUALITY, SIZE = 0, 1, 2, 3


def _shell(k, h=1.0, r=1.0, jitter=0.0, seed=0, zoff=None, radial=0.0):
    """The edge (0, 0, -h)-(0, 0, h) and k ring points around it; tets (v1, v2, p_i, p_i+1)
    oriented POSITIVE."""
    rng = np.random.default_rng(seed)
    ang = np.arange(k) * 2 * np.pi / k + rng.normal(0, jitter, k)
    rad = r * (1 + rng.uniform(-radial, radial, k))
    z = np.zeros(k) if zoff is None else np.asarray(zoff, float)
    ring = np.c_[rad * np.cos(ang), rad * np.sin(ang), z]
    xyz = np.vstack([[0, 0, -h], [0, 0, h], ring])
    tets = []
    for i in range(k):
        a, b = 2 + i, 2 + (i + 1) % k
        t = [0, 1, a, b]
        P = xyz[t]
        if np.linalg.det(np.c_[P[1] - P[0], P[2] - P[0], P[3] - P[0]].T) < 0:
            t = [0, 1, b, a]
        tets.append(t)
    return xyz, np.array(tets, np.int32)


def _check(oracle, xyz, tets, budget=0):
    r, c, s = oracle.swap_check(xyz, [[0, 1]], [0, len(tets)], tets, budget=[budget])
    return int(r[0]), int(c[0]), int(s[0])


def test_swap_known_answers(oracle):
    # removing a long edge helps, a short one hurts
    assert _check(oracle, *_shell(3, h=1.0))[:2] == (SUCCESS, 0)
    assert _check(oracle, *_shell(3, h=0.3))[0] == QUALITY
    assert _check(oracle, *_shell(5, h=3.0))[0] == SUCCESS
    assert _check(oracle, *_shell(5, h=1.0))[0] == QUALITY
    # a ring that the edge does not pierce: every configuration inverts a tet
    for k in (3, 4, 5):
        assert _check(oracle, *_shell(k, h=1.0, zoff=np.full(k, 1.5)))[0] == FLIP
    # shells of other sizes, and tets not around the edge
    assert _check(oracle, *_shell(6, h=3.0))[0] == SIZE
    xyz, t = _shell(4, h=3.0)
    t2 = t.copy()
    t2[1, t2[1] == 1] = 2
    assert _check(oracle, xyz, t2)[0] == SIZE


def test_swap_44_second_configuration_must_beat_the_first(oracle):
    """A square ring: both diagonals give the same max energy.  Without budget the
    second configuration is valid but not better than the first, which ends the removal
    (EdgeRemover.cpp:356-364); with budget it is accepted (equal) and taken."""
    xyz, t = _shell(4, h=3.0)
    assert _check(oracle, xyz, t, budget=0) == (QUALITY, 0, 0)
    assert _check(oracle, xyz, t, budget=5) == (SUCCESS, 1, 2)
    assert _check(oracle, xyz, t, budget=1) == (QUALITY, 0, 1)


# ---- the second restatement -------------------------------------------------------
def _orient(P):
    from fractions import Fraction as Fr

    p = [[Fr(float(x)) for x in v] for v in P]
    u = [p[1][k] - p[0][k] for k in range(3)]
    v = [p[2][k] - p[0][k] for k in range(3)]
    w = [p[3][k] - p[0][k] for k in range(3)]
    d = (u[0] * (v[1] * w[2] - v[2] * w[1]) - u[1] * (v[0] * w[2] - v[2] * w[0]) +
         u[2] * (v[0] * w[1] - v[1] * w[0]))
    return (d > 0) - (d < 0)


class _Restated:
    def __init__(self, oracle, xyz):
        self.o, self.xyz = oracle, xyz

    def flip(self, tets):
        return any(_orient(self.xyz[list(t)]) != 1 for t in tets)

    def qmax(self, tets):
        T = np.ascontiguousarray(self.xyz[np.asarray(tets)].reshape(-1, 12).T)
        E = self.o.amips_batch_soa(T, quality=True, jacobian=False, hessian=False)[0]
        return max(0.0, float(E.max()))

    @staticmethod
    def repl(t, a, b):
        t = list(t)
        t[t.index(a)] = b
        return t

    def check(self, shell, v1, v2, budget):
        st = {"budget": budget, "spent": 0}

        def better(nq, oq):
            if st["budget"] > 0:
                st["budget"] -= 1
                st["spent"] += 1
                return nq <= oq
            return nq < oq

        k = len(shell)
        if k not in (3, 4, 5) or any(v1 not in t or v2 not in t for t in shell):
            return SIZE, -1, 0
        oq = self.qmax(shell)
        if k == 3:
            vv = [x for x in shell[0] if x not in (v1, v2)]
            a, b = (shell[1], shell[2]) if vv[0] in shell[1] else (shell[2], shell[1])
            new = [self.repl(a, v1, vv[1]), self.repl(b, v2, vv[0])]
            if self.flip(new):
                return FLIP, -1, 0
            if not better(self.qmax(new), oq):
                return QUALITY, -1, st["spent"]
            return SUCCESS, 0, st["spent"]
        es = [[x for x in t if x not in (v1, v2)] for t in shell]
        nv, tid, vis = [es[0][0], es[0][1]], [0], [True] + [False] * (k - 1)
        for _ in range(k - 2):
            for j in range(k):
                if vis[j]:
                    continue
                if es[j][0] == nv[-1]:
                    vis[j] = True
                    nv.append(es[j][1])
                elif es[j][1] == nv[-1]:
                    vis[j] = True
                    nv.append(es[j][0])
                if vis[j]:
                    tid.append(j)
                    break
        tid.append(vis.index(False))
        if k == 4:
            valid, cfg = False, -1
            for i in range(2):
                a, b = nv[i], nv[2 + i]
                new = [self.repl(t, v2, b) if a in t else self.repl(t, v1, a) for t in shell]
                if self.flip(new):
                    continue
                nq = self.qmax(new)
                if not better(nq, oq):
                    return QUALITY, cfg, st["spent"]
                valid, oq, cfg = True, nq, i
            return (SUCCESS, cfg, st["spent"]) if valid else (FLIP, -1, st["spent"])
        ok = [True] * 5
        qs1 = {}
        for i in range(5):
            if not ok[(i + 1) % 5] and not ok[(i - 1) % 5]:
                continue
            t = shell[tid[i]]
            new = [self.repl(t, v1, nv[(i - 1) % 5]), self.repl(t, v2, nv[(i - 1) % 5])]
            if self.flip(new):
                ok[(i + 1) % 5] = ok[(i - 1) % 5] = False
                continue
            qs1[i] = new
        if not any(ok):
            return FLIP, -1, 0
        sel, tested = -1, False
        for i in range(5):
            if not ok[i]:
                continue
            t = shell[tid[(i + 2) % 5]]
            new = [self.repl(t, v1, nv[i]), self.repl(t, v2, nv[i])]
            if self.flip(new):
                continue
            tested = True
            nq = self.qmax(new + qs1[(i + 1) % 5] + qs1[(i - 1) % 5])
            if not better(nq, oq):
                continue
            oq, sel = nq, i
        if sel < 0:
            return (QUALITY if tested else FLIP), -1, st["spent"]
        return SUCCESS, sel, st["spent"]


def test_swap_agrees_with_second_restatement(oracle):
    rng = np.random.default_rng(7)
    seen = set()
    for case in range(240):
        k = int(rng.integers(3, 6))
        xyz, t = _shell(k, h=float(rng.uniform(0.2, 3.0)), jitter=float(rng.uniform(0, 0.4)),
                        radial=float(rng.uniform(0, 0.5)), seed=case,
                        zoff=rng.normal(0, float(rng.uniform(0, 0.8)), k))
        t = t[rng.permutation(k)]                          # the caller's order varies
        budget = int(rng.choice([0, 0, 1, 3]))
        got = _check(oracle, xyz, t, budget)
        want = _Restated(oracle, xyz).check([list(x) for x in t], 0, 1, budget)
        # the configuration index is meaningful only for a success
        if want[0] != SUCCESS:
            got, want = (got[0], got[2]), (want[0], want[2])
        assert got == want, (case, k, got, want)
        seen.add((k, got[0]))
    # every size reached success and at least one rejection
    for k in (3, 4, 5):
        assert (k, SUCCESS) in seen and ((k, QUALITY) in seen or (k, FLIP) in seen), seen
