"""Generates the golden fixtures in tests/golden/ from the reference's own code.

The reference ships no tests or fixtures, so the vectors come from running
its hot-path sources, compiled into oracle/_ref/libtwref.so by
oracle/ref/build_ref.py (needs the reference checkout), and from exact
rational arithmetic (Python fractions) for the orientation signs:

  amips_ref.npz     tets (AoS [n,12]) and the reference's
                    comformalAMIPS{Energy,Jacobian,Hessian}_new outputs
                    (LocalOperations.cpp:28-291)
  sample_ref.npz    triangles and the reference's sampleTriangle samples
                    (Common.cpp:143-228), concatenated with offsets
  envelope_ref.npz  a small displaced-sphere surface, query points and faces,
                    and the reference's isPointOutEnvelop /
                    isFaceOutEnvelop_sampling decisions
                    (LocalOperations.cpp:1034-1109 over mesh_AABB.cpp)
  orient_exact.npz  adversarial point quadruples and their exact
                    det[q-p, r-p, s-p] signs (CGAL::orientation convention)
  nearest_ref.npz   a small displaced-sphere surface, query points near and
                    far from it, and the closest points and squared
                    distances of the reference's
                    MeshFacetsAABBWithEps::nearest_facet (mesh_AABB.h:130)
  energy_sweeps_ref.npz
                    tets of three energy spreads (some inverted, some
                    locked) and the reference's getAvgMaxEnergy /
                    getMaxEnergy / getSecondMaxEnergy / getFilterEnergy
                    results over their calTetQualities energies
                    (LocalOperations.cpp:605-693) at three filter thresholds

Run: python tests/golden/make_golden.py [fixture names without .npz]
(all fixtures when no name is given)
"""
from __future__ import annotations

import sys
from fractions import Fraction
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle.oracle import Oracle, RefLib  # noqa: E402
from tetwild_gb300 import synthetic as syn  # noqa: E402


def exact_orient(p, q, r, s) -> int:
    P = [[Fraction(float(x)) for x in v] for v in (p, q, r, s)]
    u = [P[1][k] - P[0][k] for k in range(3)]
    v = [P[2][k] - P[0][k] for k in range(3)]
    w = [P[3][k] - P[0][k] for k in range(3)]
    det = (u[0] * (v[1] * w[2] - v[2] * w[1]) + u[1] * (v[2] * w[0] - v[0] * w[2]) +
           u[2] * (v[0] * w[1] - v[1] * w[0]))
    return (det > 0) - (det < 0)


def amips_cases(rng):
    T = syn.energy_batch(1500, seed=11).T.copy()          # benchmark distribution
    near = syn.energy_batch(300, seed=12, sigma_rel=0.35).T.copy()  # many near-flat / inverted
    scale = []
    for s in (1e-6, 1e-3, 1.0, 1e3):
        t = (syn.REGULAR_TET * s).reshape(12)
        scale.append(t)
        scale.append(t + rng.normal(0, 0.05 * s, 12))
    centred = syn.energy_batch(200, seed=13).T.copy()
    centred = (centred.reshape(-1, 4, 3) - centred.reshape(-1, 4, 3).mean(1, keepdims=True)).reshape(-1, 12)
    return np.vstack([T, near, np.asarray(scale), centred])


def triangle_cases(rng, sd):
    tris = []
    for _ in range(100):
        a = rng.random(3)
        L = rng.uniform(0.2 * sd, 20 * sd)
        b = a + L * rng.normal(size=3) / np.sqrt(3)
        c = a + L * rng.normal(size=3) / np.sqrt(3)
        tris.append(np.concatenate([a, b, c]))
    # right, obtuse, needle, equilateral, integer-N edge lengths
    e = np.array([0.0, 0.0, 0.0])
    tris.append(np.concatenate([e, [10 * sd, 0, 0], [0, 10 * sd, 0]]))
    tris.append(np.concatenate([e, [20 * sd, 0, 0], [19 * sd, 2 * sd, 0]]))
    tris.append(np.concatenate([e, [30 * sd, 0, 0], [15 * sd, 0.3 * sd, 0]]))
    tris.append(np.concatenate([e, [8 * sd, 0, 0], [4 * sd, 8 * sd * np.sqrt(3) / 2, 0]]))
    tris.append(np.concatenate([e, [4 * sd, 0, 0], [0, 3 * sd, 0]]))
    tris.append(np.concatenate([e, [0.5 * sd, 0, 0], [0, 0.4 * sd, 0]]))
    return np.asarray(tris)


def orient_cases(rng):
    quads = []
    for _ in range(300):
        quads.append(rng.normal(size=(4, 3)))
    # coplanar lattice points and 1-ulp perturbations
    for _ in range(300):
        base = rng.integers(-4, 5, size=(3, 3)).astype(float)
        a, b = rng.integers(-3, 4, 2).astype(float)
        p4 = base[0] + a * (base[1] - base[0]) + b * (base[2] - base[0])
        q = np.vstack([base, p4])
        k = rng.integers(0, 3)
        if k == 1:
            i, j = rng.integers(0, 4), rng.integers(0, 3)
            q[i, j] = np.nextafter(q[i, j], np.inf)
        elif k == 2:
            q = q * 1e-3 + 0.1
        quads.append(q)
    # near-coplanar with large offsets (cancellation in the differences)
    for _ in range(200):
        base = rng.normal(size=(3, 3)) * 1e-8 + 1e3
        w = rng.random(2)
        p4 = base[0] + w[0] * (base[1] - base[0]) + w[1] * (base[2] - base[0])
        quads.append(np.vstack([base, p4]))
    quads = np.asarray(quads)
    signs = np.array([exact_orient(*q) for q in quads], np.int8)
    return quads, signs


def make_nearest(ref):
    V, F = syn.displaced_sphere(seed=8, n_lon=40, n_rings=20)
    rng = np.random.default_rng(77)
    P = syn.envelope_points(V, F, 3000, 1e-2, seed=9)
    P = np.vstack([P, P[:1000] + rng.normal(0.0, 0.05, (1000, 3)),
                   rng.uniform(-2.0, 2.0, (500, 3))])
    Q, D = ref.surface(V, F).nearest(P)
    np.savez_compressed(HERE / "nearest_ref.npz", V=V, F=F, P=P, Q=Q, D=D)


SWEEP_SIGMAS = (0.1, 0.6, 2.0)
SWEEP_THRES = (1.0, 3.0, 10.0)


def make_sweeps(ref):
    """The sweeps' input is calTetQualities' energies (AMIPS energy, or the 1e50 sentinel for
    an inverted tet), stored as E: the oracle's reference form built with libm's pow, which
    is the reference's comformalAMIPSEnergy_new bit for bit (asserted below), with the
    oracle's exact orientation for the sentinel.  The results are the reference's sweeps
    over exactly these values."""
    o = Oracle(libm=True)
    n = 600
    Ts, Ls, Es, R = [], [], [], []
    for c, sigma in enumerate(SWEEP_SIGMAS):
        rng = np.random.default_rng(300 + c)
        T = syn.energy_batch(n, seed=310 + c, sigma_rel=sigma)
        flip = rng.random(n) < 0.03
        T[0:3, flip], T[3:6, flip] = T[3:6, flip].copy(), T[0:3, flip].copy()
        locked = (rng.random(n) < 0.1).astype(np.uint8)
        E = o.amips_batch_soa(T, quality=True, jacobian=False, hessian=False)[0]
        Er = ref.amips_batch_soa(T, jacobian=False, hessian=False)[0]
        live = E != 1e50
        assert np.array_equal(E[live], Er[live]) and (~live).any()
        rows = []
        for thres in SWEEP_THRES:
            a, m, _, m2, f, clean = ref.energy_sweeps(E, None, locked, thres)
            rows.append([a, m, m2, f, float(clean)])
        Ts.append(T)
        Ls.append(locked)
        Es.append(E)
        R.append(rows)
    np.savez_compressed(HERE / "energy_sweeps_ref.npz", T=np.stack(Ts), locked=np.stack(Ls),
                        E=np.stack(Es), sigmas=np.asarray(SWEEP_SIGMAS), thres=np.asarray(SWEEP_THRES),
                        results=np.asarray(R))


def main(names=None):
    rng = np.random.default_rng(2024)
    ref = RefLib()
    if names:
        if "nearest_ref" in names:
            make_nearest(ref)
        if "energy_sweeps_ref" in names:
            make_sweeps(ref)
        return
    make_nearest(ref)
    make_sweeps(ref)

    T = amips_cases(rng)
    E, J, H = ref.amips_batch_soa(T.T.copy())
    np.savez_compressed(HERE / "amips_ref.npz", T=T, E=E, J=J.T.copy(), H=H.T.copy())

    sd = 3.4641016151377544e-3 * 1.0
    tris = triangle_cases(rng, sd)
    samples, offs = [], [0]
    for t in tris:
        s = ref.sample_triangle(t, sd)
        samples.append(s)
        offs.append(offs[-1] + len(s))
    np.savez_compressed(HERE / "sample_ref.npz", tris=tris, sd=sd, samples=np.vstack(samples),
                        offsets=np.asarray(offs, np.int64))

    V, F = syn.displaced_sphere(seed=5, n_lon=40, n_rings=20)
    eps = 1e-2
    P = syn.envelope_points(V, F, 3000, eps, seed=6)
    S = ref.surface(V, F)
    pout = S.points_out(P, eps * eps)
    # faces: small triangles near the surface, half of them pushed outward
    idx = rng.integers(0, len(F), 200)
    A, B, C = V[F[idx, 0]], V[F[idx, 1]], V[F[idx, 2]]
    cen = (A + B + C) / 3
    nrm = np.cross(B - A, C - A)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    shrink = rng.uniform(0.3, 1.0, (200, 1))
    push = rng.uniform(-1.5, 1.5, (200, 1)) * eps
    faces = np.hstack([cen + shrink * (A - cen) + push * nrm, cen + shrink * (B - cen) + push * nrm,
                       cen + shrink * (C - cen) + push * nrm])
    fsd = eps
    fout = S.faces_out(faces, eps * eps, fsd)
    np.savez_compressed(HERE / "envelope_ref.npz", V=V, F=F, eps=eps, P=P, point_out=pout,
                        faces=faces, sd=fsd, face_out=fout)

    quads, signs = orient_cases(rng)
    np.savez_compressed(HERE / "orient_exact.npz", quads=quads, signs=signs)
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main(sys.argv[1:])
