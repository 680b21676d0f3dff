"""Pins the CPU oracle (oracle/tw_oracle.c) to the reference.

The reference has no tests or golden data of its own.  The oracle is pinned
against (a) fixtures produced by the reference's own code (tests/golden,
regenerated by tests/golden/make_golden.py from oracle/_ref), (b) the
reference's code run live when oracle/_ref can be built, and (c) exact
rational arithmetic and high-precision evaluation.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

from conftest import golden
from tetwild_gb300 import synthetic as syn


# ---------------------------------------------------------------- icbrt ----
def test_icbrt_close_to_exact(oracle):
    import mpmath

    mpmath.mp.prec = 200
    rng = np.random.default_rng(0)
    xs = list(10.0 ** rng.uniform(-300, 300, 3000)) + [5e-324, 1e-310, 2.2250738585072014e-308,
                                                        1.0, 8.0, 7.999999999999999, 1e308]
    worst = 0.0
    for x in xs:
        y = oracle.icbrt(float(x))
        exact = mpmath.mpf(x) ** (mpmath.mpf(-1) / 3)
        ulp = math.ulp(y)
        worst = max(worst, float(abs(mpmath.mpf(y) - exact) / ulp))
    assert worst <= 2.0, worst


def test_icbrt_special_values(oracle):
    assert oracle.icbrt(0.0) == math.inf
    assert oracle.icbrt(math.inf) == 0.0
    assert math.isnan(oracle.icbrt(math.nan))


# ---------------------------------------------------------------- AMIPS ----
# Two energy forms (two_set_energy_form): the reference form, the default,
# performs the reference's generated operations (LocalOperations.cpp:28-291)
# in its order and agrees with it to its rounding; the closed form evaluates
# the same function accurately.  Tolerance of the reference form against the
# reference's own routines: 1e-12 relative per entry of E, J and H.
REL_TOL = 1e-12
FORM_REFERENCE, FORM_CLOSED = 0, 1


def _aos_to_soa(T):
    return np.ascontiguousarray(np.asarray(T).T)


@pytest.fixture
def closed_form(oracle):
    oracle.set_energy_form(FORM_CLOSED)
    yield oracle
    oracle.set_energy_form(FORM_REFERENCE)


def test_default_form_is_reference(oracle):
    assert oracle.energy_form() == FORM_REFERENCE


def _within(a, b, tol):
    """Entry-wise |a - b| <= tol |b| (a zero reference entry must be matched exactly)."""
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b) <= tol * np.abs(b)


def test_amips_known_answers(oracle):
    for form, tol in ((FORM_CLOSED, 1e-14), (FORM_REFERENCE, REL_TOL)):
        oracle.set_energy_form(form)
        try:
            t = (syn.REGULAR_TET * 0.37 + np.array([3.0, -2.0, 5.0])).reshape(12)
            E, J, H, F = oracle.amips_batch_soa(_aos_to_soa([t]), quality=False)
            assert abs(E[0] - 3.0) < 3.0 * tol
            assert np.abs(J[:, 0]).max() < 1e-10 / 0.37
            # at the minimum the Hessian is symmetric positive definite (exactly
            # symmetric in the closed form; the generated expressions of H[1] and
            # H[3] round differently)
            Hm = H[:, 0].reshape(3, 3)
            assert np.all(_within(Hm, Hm.T, tol) | (np.abs(Hm - Hm.T) < tol * np.abs(Hm).max()))
            assert np.linalg.eigvalsh((Hm + Hm.T) / 2).min() > 0
            # either orientation gives 3 (README: range 3..inf)
            t2 = t.reshape(4, 3)[[0, 2, 1, 3]].reshape(12)
            E2, _, _, F2 = oracle.amips_batch_soa(_aos_to_soa([t2]), quality=False)
            assert abs(E2[0] - 3.0) < 3.0 * tol and F2[0] == 1 and F[0] == 0
        finally:
            oracle.set_energy_form(FORM_REFERENCE)


def test_amips_invariances(closed_form):
    oracle = closed_form
    T = syn.energy_batch(2000, seed=3).T
    E0 = oracle.amips_batch_soa(_aos_to_soa(T), quality=False)[0]
    Ts = T * 7.5
    E1 = oracle.amips_batch_soa(_aos_to_soa(Ts), quality=False)[0]
    perm = T.reshape(-1, 4, 3)[:, [1, 0, 3, 2]].reshape(-1, 12)
    E2 = oracle.amips_batch_soa(_aos_to_soa(perm), quality=False)[0]
    assert np.max(np.abs(E1 - E0) / E0) < 1e-12
    assert np.max(np.abs(E2 - E0) / E0) < 1e-12
    assert np.all(E0 >= 3.0 - 1e-12)


@pytest.mark.parametrize("form", [FORM_REFERENCE, FORM_CLOSED])
def test_amips_derivatives_match_finite_differences(oracle, form):
    oracle.set_energy_form(form)
    try:
        T = syn.energy_batch(50, seed=4).T
        E, J, H, _ = oracle.amips_batch_soa(_aos_to_soa(T), quality=False)
        h = 1e-7
        for i in range(0, 50, 7):
            for k in range(3):
                tp, tm = T[i].copy(), T[i].copy()
                tp[k] += h
                tm[k] -= h
                Ep, Jp, _, _ = oracle.amips_batch_soa(_aos_to_soa([tp]), quality=False)
                Em, Jm, _, _ = oracle.amips_batch_soa(_aos_to_soa([tm]), quality=False)
                fd = (Ep[0] - Em[0]) / (2 * h)
                assert abs(fd - J[k, i]) < 1e-5 * max(1.0, abs(E[i]) / 0.01)
                fdH = (Jp[:, 0] - Jm[:, 0]) / (2 * h)
                Hrow = H[:, i].reshape(3, 3)[:, k]
                assert np.max(np.abs(fdH - Hrow)) < 1e-4 * np.max(np.abs(Hrow))
    finally:
        oracle.set_energy_form(FORM_REFERENCE)


def _amips_cases_live():
    """The energy-batch distribution (regular tets of edge 0.01 in the unit
    cube, vertices perturbed by 0.1 edge) and a near-flat batch."""
    return np.hstack([syn.energy_batch(20000, seed=21),
                      syn.energy_batch(3000, seed=22, sigma_rel=0.35)])


def test_amips_reference_form_libm_bit_exact_golden():
    """With libm's pow (the TW_RF_LIBM build) the reference form performs
    exactly the reference's operations: bit-identical E, J and H on every
    fixture tet (the fixtures were made by the reference's own routines)."""
    from oracle.oracle import Oracle

    o = Oracle(libm=True)
    g = golden("amips_ref.npz")
    E, J, H, _ = o.amips_batch_soa(_aos_to_soa(g["T"]), quality=False)
    assert np.array_equal(E, g["E"])
    assert np.array_equal(J.T, g["J"])
    assert np.array_equal(H.T, g["H"])


def test_amips_reference_form_libm_bit_exact_live(reflib):
    from oracle.oracle import Oracle

    o = Oracle(libm=True)
    T = _amips_cases_live()
    Er, Jr, Hr = reflib.amips_batch_soa(T, nthreads=4)
    E, J, H, _ = o.amips_batch_soa(T, quality=False, nthreads=4)
    assert np.array_equal(E, Er) and np.array_equal(J, Jr) and np.array_equal(H, Hr)


def test_rf_pow_matches_libm(oracle):
    """rf_pow_m13 (icbrt times the exponent correction) against libm's
    pow(s, -0.333333333333333) over the double range: a few ulp."""
    rng = np.random.default_rng(5)
    xs = 10.0 ** rng.uniform(-300, 300, 20000)
    got = np.array([oracle.L.two_rf_pow_m13(float(x)) for x in xs])
    want = np.array([math.pow(float(x), -0.333333333333333) for x in xs])   # libm's pow
    rel = np.abs(got - want) / want
    assert rel.max() < 1e-15, rel.max()
    assert oracle.L.two_rf_pow_m13(0.0) == math.inf and oracle.L.two_rf_pow_m13(math.inf) == 0.0


def test_amips_matches_reference_golden(oracle):
    g = golden("amips_ref.npz")
    E, J, H, _ = oracle.amips_batch_soa(_aos_to_soa(g["T"]), quality=False)
    assert np.all(_within(E, g["E"], REL_TOL))
    assert np.all(_within(J.T, g["J"], REL_TOL))
    assert np.all(_within(H.T, g["H"], REL_TOL))


def test_amips_matches_reference_live(oracle, reflib):
    T = _amips_cases_live()
    Er, Jr, Hr = reflib.amips_batch_soa(T, nthreads=4)
    E, J, H, _ = oracle.amips_batch_soa(T, quality=False, nthreads=4)
    assert np.all(_within(E, Er, REL_TOL)), np.max(np.abs(E - Er) / np.abs(Er))
    assert np.all(_within(J, Jr, REL_TOL))
    assert np.all(_within(H, Hr, REL_TOL))


def _closed_form_tolerances(T):
    """Closed form against the reference: the reference's 15-digit
    coefficients (1.15470053837925 is not 2 * 0.577350269189626) make its
    result depend on the absolute position of the tet, and its terms on
    absolute coordinates cancel: an error of about 2e-15 |x| / edge on each
    row of the map, amplified by the conditioning edge^3 / |det| of the map.
    1e-12 relative at the origin, growing with |x|/edge * conditioning."""
    P = T.reshape(-1, 4, 3)
    edge = np.linalg.norm(P[:, 0] - P[:, 3], axis=1)
    far = np.abs(P).max(axis=(1, 2)) / np.maximum(edge, 1e-300)
    a = P[:, 0] - P[:, 3]
    b = (P[:, 0] - 2 * P[:, 1] + P[:, 3]) / np.sqrt(3)
    c = (P[:, 0] + P[:, 1] + P[:, 3] - 3 * P[:, 2]) / np.sqrt(6)
    D = np.einsum("ij,ij->i", a, np.cross(b, c))
    cond = np.maximum(1.0, edge ** 3 / np.maximum(np.abs(D), 1e-300))
    return 1e-12 + 5e-14 * far * cond


def _term_scales(T):
    """Magnitudes of the terms summed in J = r (gN - 2/3 N/D g) and
    H = 3r I - 2/3 r/D (gN g' + g gN') + 10/9 N r/D^2 g g'."""
    P = T.reshape(-1, 4, 3)
    a = P[:, 0] - P[:, 3]
    b = (P[:, 0] - 2 * P[:, 1] + P[:, 3]) / np.sqrt(3)
    c = (P[:, 0] + P[:, 1] + P[:, 3] - 3 * P[:, 2]) / np.sqrt(6)
    N = (a * a).sum(1) + (b * b).sum(1) + (c * c).sum(1)
    D = np.einsum("ij,ij->i", a, np.cross(b, c))
    g = np.cross(b, c) + np.cross(c, a) / np.sqrt(3) + np.cross(a, b) / np.sqrt(6)
    gN = 2 * (a + b / np.sqrt(3) + c / np.sqrt(6))
    r = np.abs(D) ** (-2.0 / 3.0)
    ng, ngN = np.linalg.norm(g, axis=1), np.linalg.norm(gN, axis=1)
    sJ = r * (ngN + 2.0 / 3.0 * N / np.abs(D) * ng)
    sH = 3 * r + 4.0 / 3.0 * r / np.abs(D) * ngN * ng + 10.0 / 9.0 * N * r / D ** 2 * ng ** 2
    return sJ, sH


def test_amips_closed_form_vs_reference(closed_form):
    oracle = closed_form
    g = golden("amips_ref.npz")
    T = g["T"]
    E, J, H, _ = oracle.amips_batch_soa(_aos_to_soa(T), quality=False)
    ok = np.isfinite(g["E"]) & (g["E"] < 1e8)
    tol = _closed_form_tolerances(T)
    relE = np.abs(E - g["E"]) / np.abs(g["E"])
    assert np.all(relE[ok] <= tol[ok]), relE[ok].max()
    sJ, sH = _term_scales(T)
    errJ = np.abs(J.T - g["J"]).max(1) / sJ
    errH = np.abs(H.T - g["H"]).max(1) / sH
    assert np.all(errJ[ok] <= 10 * tol[ok]), errJ[ok].max()
    assert np.all(errH[ok] <= 10 * tol[ok]), errH[ok].max()


def test_amips_closed_form_accurate(closed_form):
    """The closed form against a 60-digit evaluation of the same function."""
    import mpmath

    mpmath.mp.dps = 60
    oracle = closed_form
    T = syn.energy_batch(60, seed=23).T
    E = oracle.amips_batch_soa(_aos_to_soa(T), quality=False)[0]
    for i in range(T.shape[0]):
        p = [[mpmath.mpf(float(x)) for x in T[i, 3 * j:3 * j + 3]] for j in range(4)]
        s3, s6 = mpmath.sqrt(3), mpmath.sqrt(6)
        a = [p[0][k] - p[3][k] for k in range(3)]
        b = [(p[0][k] - 2 * p[1][k] + p[3][k]) / s3 for k in range(3)]
        c = [(p[0][k] + p[1][k] + p[3][k] - 3 * p[2][k]) / s6 for k in range(3)]
        N = sum(x * x for x in a + b + c)
        D = (a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
             a[2] * (b[0] * c[1] - b[1] * c[0]))
        exact = N * (D * D) ** (mpmath.mpf(-1) / 3)
        assert abs(float((E[i] - exact) / exact)) < 1e-14


# ---------------------------------------------------------- orientation ----
def test_orientation_matches_exact_golden(oracle):
    g = golden("orient_exact.npz")
    got = np.array([oracle.orient3d(*q) for q in g["quads"]], np.int8)
    assert np.array_equal(got, g["signs"])
    got_exact = np.array([oracle.orient3d_exact(*q) for q in g["quads"]], np.int8)
    assert np.array_equal(got_exact, g["signs"])


def _frac_orient(p, q, r, s):
    P = [[Fraction(float(x)) for x in v] for v in (p, q, r, s)]
    u = [P[1][k] - P[0][k] for k in range(3)]
    v = [P[2][k] - P[0][k] for k in range(3)]
    w = [P[3][k] - P[0][k] for k in range(3)]
    d = (u[0] * (v[1] * w[2] - v[2] * w[1]) + u[1] * (v[2] * w[0] - v[0] * w[2]) +
         u[2] * (v[0] * w[1] - v[1] * w[0]))
    return (d > 0) - (d < 0)


def test_orientation_random_vs_fraction(oracle):
    rng = np.random.default_rng(7)
    for _ in range(400):
        base = rng.normal(size=(3, 3)) * 10 ** rng.uniform(-6, 6)
        w = rng.random(2)
        p4 = base[0] + w[0] * (base[1] - base[0]) + w[1] * (base[2] - base[0])
        q = np.vstack([base, p4])
        i, j = rng.integers(0, 4), rng.integers(0, 3)
        for _ in range(rng.integers(0, 3)):
            q[i, j] = np.nextafter(q[i, j], np.inf)
        assert oracle.orient3d(*q) == _frac_orient(*q)


def test_collinear_exact(oracle):
    rng = np.random.default_rng(8)
    for _ in range(300):
        a = rng.integers(-5, 6, 3).astype(float) * 0.125
        d = rng.integers(-3, 4, 3).astype(float)
        b, c = a + d, a + 2.5 * d
        if rng.random() < 0.5:
            k = rng.integers(0, 3)
            c[k] = np.nextafter(c[k], np.inf)
        A = [Fraction(x) for x in a]
        B = [Fraction(x) for x in b]
        C = [Fraction(x) for x in c]
        u = [B[k] - A[k] for k in range(3)]
        v = [C[k] - A[k] for k in range(3)]
        cross = [u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]]
        assert oracle.collinear(a, b, c) == int(all(x == 0 for x in cross))


def test_quality_sentinel(oracle):
    t = syn.REGULAR_TET.reshape(12).copy()
    inv = t.reshape(4, 3)[[1, 0, 2, 3]].reshape(12)
    flat = t.copy()
    flat[11] = 0.0  # p3 on the plane of p0, p1, p2
    E, _, _, F = oracle.amips_batch_soa(_aos_to_soa([t, inv, flat]), quality=True)
    assert abs(E[0] - 3.0) < 1e-14 and F[0] == 0
    assert E[1] == 1e50 and F[1] == 1
    assert E[2] == 1e50 and F[2] == 1


# ------------------------------------------------------------- sampling ----
def test_sample_triangle_matches_reference_golden(oracle):
    g = golden("sample_ref.npz")
    sd = float(g["sd"])
    for i, t in enumerate(g["tris"]):
        want = g["samples"][g["offsets"][i]:g["offsets"][i + 1]]
        got = oracle.sample_triangle(t, sd)
        assert got.shape == want.shape, i
        assert np.array_equal(got, want), i


def test_sample_triangle_matches_reference_live(oracle, reflib):
    rng = np.random.default_rng(31)
    sd = 0.01
    for _ in range(300):
        a = rng.random(3)
        t = np.concatenate([a, a + rng.normal(size=3) * rng.uniform(0.001, 0.3),
                            a + rng.normal(size=3) * rng.uniform(0.001, 0.3)])
        assert np.array_equal(oracle.sample_triangle(t, sd), reflib.sample_triangle(t, sd))


# ------------------------------------------------------------- envelope ----
def test_point_envelope_matches_reference_golden(oracle):
    g = golden("envelope_ref.npz")
    eps2 = float(g["eps"]) ** 2
    S = oracle.surface(g["V"], g["F"])
    got = S.points_out(g["P"], eps2)
    assert np.array_equal(got, g["point_out"])
    brute = np.array([S.point_out_brute(p, eps2) for p in g["P"][:500]], np.uint8)
    assert np.array_equal(brute, g["point_out"][:500])


def test_face_envelope_matches_reference_golden(oracle):
    g = golden("envelope_ref.npz")
    eps2 = float(g["eps"]) ** 2
    S = oracle.surface(g["V"], g["F"])
    got = S.faces_out(g["faces"], eps2, float(g["sd"]))
    assert np.array_equal(got, g["face_out"])


def test_envelope_matches_reference_live(oracle, reflib):
    V, F = syn.displaced_sphere(seed=9, n_lon=80, n_rings=40)
    eps = 3e-3
    P = syn.envelope_points(V, F, 20000, eps, seed=10)
    a = oracle.surface(V, F).points_out(P, eps * eps, nthreads=4)
    b = reflib.surface(V, F).points_out(P, eps * eps, nthreads=4)
    assert np.array_equal(a, b)
    assert 0.3 < a.mean() < 0.7


def test_degenerate_face_is_not_out(oracle):
    V, F = syn.displaced_sphere(seed=9, n_lon=20, n_rings=10)
    S = oracle.surface(V, F)
    far = np.array([5.0, 5.0, 5.0, 6.0, 6.0, 6.0, 7.0, 7.0, 7.0])  # collinear, far away
    assert S.faces_out(far[None], 1e-6, 0.01)[0] == 0
    tri = np.array([5.0, 5.0, 5.0, 6.0, 6.0, 6.0, 7.0, 7.0, 7.5])
    assert S.faces_out(tri[None], 1e-6, 0.01)[0] == 1


# ------------------------------------------------------------------ QR ----
def test_qr_solve_matches_numpy(oracle):
    rng = np.random.default_rng(12)
    for _ in range(200):
        A = rng.normal(size=(3, 3))
        A = A @ A.T + 0.1 * np.eye(3)
        b = rng.normal(size=3)
        x = oracle.qr_solve3(A, b)
        assert np.allclose(x, np.linalg.solve(A, b), rtol=1e-10, atol=1e-12)


def test_qr_rank_deficient_gives_finite(oracle):
    A = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [1.0, 0.0, 1.0]])
    x = oracle.qr_solve3(A, np.array([1.0, 2.0, 1.0]))
    assert np.all(np.isfinite(x))
    assert np.allclose(A @ x, [1.0, 2.0, 1.0], atol=1e-12)


# --------------------------------------------------------------- Newton ----
def test_newton_star_decreases_energy(oracle):
    xyz, off, tets, cen = syn.star_batch(60, seed=14)
    out, moved = oracle.newton_stars(xyz, off, tets, cen)
    assert moved.sum() > 0
    for s in range(60):
        T = tets[off[s]:off[s + 1]]
        X = xyz.copy()
        before = oracle.amips_batch_soa(np.ascontiguousarray(X[T].reshape(-1, 12).T), quality=False)[0].sum()
        X[cen[s]] = out[s]
        after = oracle.amips_batch_soa(np.ascontiguousarray(X[T].reshape(-1, 12).T), quality=False)[0].sum()
        if moved[s]:
            assert after < before
        # never inverts a tet
        flips = oracle.amips_batch_soa(np.ascontiguousarray(X[T].reshape(-1, 12).T))[3]
        assert flips.sum() == 0 or not moved[s]


# -------------------------------------------------------- nearest facet ----
def _nearest_vs(Q, D, Qr, Dr):
    """Distances identical everywhere; closest points identical except where
    two facets tie at the same distance (the tie goes to a different facet)."""
    assert np.array_equal(D, Dr)
    diff = np.any(Q != Qr, axis=1)
    # ties happen where the closest feature is an edge shared by two facets
    # (computed once from each side) and are rarer the nearer the points
    assert diff.mean() < 0.02, diff.mean()
    if diff.any():
        # a tie: both points are at the same distance and agree to a few ulps
        err = np.abs(Q[diff] - Qr[diff]) / np.maximum(1.0, np.abs(Qr[diff]))
        assert err.max() <= 4.5e-16, err.max()
    return int(diff.sum())


def test_nearest_matches_reference_golden(oracle):
    g = golden("nearest_ref.npz")
    Q, D, Fi = oracle.surface(g["V"], g["F"]).nearest(g["P"], nthreads=4)
    _nearest_vs(Q, D, g["Q"], g["D"])
    assert (Fi >= 0).all() and (Fi < len(g["F"])).all()


def test_nearest_matches_reference_live(oracle, reflib):
    V, F = syn.displaced_sphere(seed=3, n_lon=100, n_rings=50)
    P = syn.envelope_points(V, F, 20000, 1e-3, seed=4)
    P = np.vstack([P, P[:5000] + np.random.default_rng(5).normal(0, 0.02, (5000, 3))])
    Q, D, _ = oracle.surface(V, F).nearest(P, nthreads=8)
    Qr, Dr = reflib.surface(V, F).nearest(P, nthreads=8)
    _nearest_vs(Q, D, Qr, Dr)


def test_nearest_tree_equals_brute_force(oracle):
    V, F = syn.displaced_sphere(seed=6, n_lon=30, n_rings=15)
    rng = np.random.default_rng(7)
    P = np.vstack([syn.envelope_points(V, F, 300, 1e-2, seed=8), rng.uniform(-1.5, 1.5, (100, 3))])
    S = oracle.surface(V, F)
    Q, D, Fi = S.nearest(P)
    for i in range(len(P)):
        q, d, f = S.nearest_brute(P[i])
        assert d == D[i] and f == Fi[i] and np.array_equal(q, Q[i])


# ------------------------------------------------------ smoothing pass ----
def test_smooth_interior_is_newton(oracle):
    """Interior stars: the pass equals NewtonsMethod wherever the star is valid."""
    xyz, off, tets, cen = syn.star_batch(300, seed=15, jitter_rel=0.25)
    out, st = oracle.smooth_stars(xyz, off, tets, cen, max_step=15, max_it=20, nthreads=4)
    want, moved = oracle.newton_stars(xyz, off, tets, cen, 15, 20, nthreads=4)
    valid = st != 0
    assert valid.mean() > 0.5
    assert np.array_equal(st[valid] == 2, moved[valid] == 1)
    m = st == 2
    assert np.array_equal(out[m], want[m])
    assert np.array_equal(out[~m], xyz[cen[~m]])


def test_smooth_surface_outcomes_are_consistent(oracle):
    """Surface stars: accepted positions lie on the surface (projection), keep
    every tet positive, lower the max energy and keep the one-ring surface
    faces in the envelope; rejected stars keep their old position."""
    V, F = syn.displaced_sphere(seed=0, n_lon=60, n_rings=30)
    eps = 1e-3
    xyz, off, tets, ff, cen = syn.surface_star_batch(V, F, 400, eps, seed=2)
    S = oracle.surface(V, F)
    kinds = np.ones(len(cen), np.uint8)
    out, st = oracle.smooth_stars(xyz, off, tets, cen, ff, kinds, surface=S, boundary=S,
                                  eps2=eps * eps, sd=eps / 2, max_step=1, max_it=8, nthreads=4)
    counts = np.bincount(st, minlength=6)
    assert counts[2] > 50 and counts[4] + counts[5] > 10, counts
    rej = st != 2
    assert np.array_equal(out[rej], xyz[cen[rej]])
    for i in np.nonzero(st == 2)[0][:60]:
        q, d, _ = S.nearest(out[i:i + 1])
        assert d[0] <= 1e-24
        T = tets[off[i]:off[i + 1]]
        X = xyz.copy()
        old = X[T].reshape(-1, 12)
        X[cen[i]] = out[i]
        new = X[T].reshape(-1, 12)
        qo = [oracle.L.two_tet_quality(np.ascontiguousarray(t).ctypes.data) for t in old]
        qn = [oracle.L.two_tet_quality(np.ascontiguousarray(t).ctypes.data) for t in new]
        assert max(qn) < max(qo) and max(qn) < 1e50
        tris = []
        for t in T:
            tri = X[[t[0], t[1], t[2]]]  # face opposite vertex 3 (the flagged one)
            tris.append(tri.reshape(9))
        assert not S.faces_out(np.asarray(tris), eps * eps, eps / 2).any()


@pytest.mark.parametrize("sigma", [0.1, 0.6, 2.0])
def test_energy_sweeps_match_reference_live(oracle, reflib, sigma):
    """getAvgMaxEnergy / getMaxEnergy / getSecondMaxEnergy / getFilterEnergy
    (LocalOperations.cpp:605-693, compiled from the reference) against the oracle's
    one-pass sweep, on tets whose energies spread over the filter's buckets, with
    inverted tets (the 1e50 sentinel) and locked tets."""
    rng = np.random.default_rng(40 + int(10 * sigma))
    n = 20000
    T = syn.energy_batch(n, seed=41, sigma_rel=sigma)
    flip = rng.random(n) < 0.02
    T[0:3, flip], T[3:6, flip] = T[3:6, flip].copy(), T[0:3, flip].copy()
    E = oracle.amips_batch_soa(T, quality=True, jacobian=False, hessian=False)[0]
    assert (E == 1e50).any()
    xyz = T.reshape(4, 3, n).transpose(2, 0, 1).reshape(-1, 3)
    tets = np.arange(4 * n, dtype=np.int32).reshape(n, 4)
    locked = (rng.random(n) < 0.1).astype(np.uint8)
    seen = set()
    for thres in (1.0, 3.0, 10.0):   # every branch of getFilterEnergy over the three batches
        a, m, m2, buckets = oracle.energy_stats(xyz, tets, locked, thres)
        f, clean = oracle.filter_energy(buckets, thres)
        ra, rm, rm_, rm2, rf, rclean = reflib.energy_sweeps(E, None, locked, thres)
        assert a == ra and m == rm == rm_ and m2 == rm2
        assert f == rf and clean == rclean
        seen.add((f, clean))
    assert len(seen) >= 2


def test_energy_sweeps_match_reference_golden(oracle):
    """getAvgMaxEnergy / getMaxEnergy / getSecondMaxEnergy / getFilterEnergy
    (LocalOperations.cpp:605-693): the oracle's one-pass sweep against the reference's
    results stored in energy_sweeps_ref.npz, bit for bit, over the filter branches the
    fixture's thresholds reach (inverted tets at the 1e50 sentinel, locked tets skipped).
    The fixture's energies are the reference's own; the sweep runs on the oracle's libm
    build, whose energies equal them bit for bit, and the default build's energies agree
    with them to 1e-12."""
    from oracle.oracle import Oracle

    Ed = oracle.amips_batch_soa(golden("energy_sweeps_ref.npz")["T"][0], quality=True,
                                jacobian=False, hessian=False)[0]
    assert np.all(_within(Ed, golden("energy_sweeps_ref.npz")["E"][0], REL_TOL))
    oracle = Oracle(libm=True)
    g = golden("energy_sweeps_ref.npz")
    n = g["T"].shape[2]
    tets = np.arange(4 * n, dtype=np.int32).reshape(n, 4)
    branches = set()
    for c in range(len(g["sigmas"])):
        T = g["T"][c]
        # the sweep input the reference ran over
        E = oracle.amips_batch_soa(T, quality=True, jacobian=False, hessian=False)[0]
        assert np.array_equal(E, g["E"][c])
        xyz = T.reshape(4, 3, n).transpose(2, 0, 1).reshape(-1, 3)
        for k, thres in enumerate(g["thres"]):
            a, m, m2, buckets = oracle.energy_stats(xyz, tets, g["locked"][c], float(thres))
            f, clean = oracle.filter_energy(buckets, float(thres))
            ra, rm, rm2, rf, rclean = g["results"][c, k]
            assert (a, m, m2, f, clean) == (ra, rm, rm2, rf, bool(rclean))
            branches.add((rf, bool(rclean)))
    assert len(branches) >= 3


def _dihedral_numpy(t):
    """Independent dihedral angles of one tet: pi minus the angle between the outward
    normals of the two faces meeting at each edge."""
    v = t.reshape(4, 3)
    n = []
    for i in range(4):
        o = [j for j in range(4) if j != i]
        nn = np.cross(v[o[1]] - v[o[0]], v[o[2]] - v[o[0]])
        if np.dot(nn, v[i] - v[o[0]]) > 0:
            nn = -nn
        n.append(nn / np.linalg.norm(nn))
    ang = [math.pi - math.acos(max(-1.0, min(1.0, float(np.dot(n[a], n[b])))))
           for a in range(4) for b in range(a + 1, 4)]
    return min(ang), max(ang)


def test_dihedral_known_answers(oracle):
    """calTetQuality_AD (LocalOperations.cpp:783-860): regular and corner tets, degenerate
    tets give (0, pi), tiny tets take the rescaled branch, and random tets agree with an
    independent computation from face normals."""
    reg = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], float).reshape(12)
    a, b = oracle.dihedral_minmax(reg)
    assert abs(a - math.acos(1 / 3)) < 1e-15 and abs(b - math.acos(1 / 3)) < 1e-15
    corner = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float).reshape(12)
    a, b = oracle.dihedral_minmax(corner)
    assert abs(a - math.acos(1 / math.sqrt(3))) < 1e-15 and abs(b - math.pi / 2) < 1e-15
    for bad in ([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]],      # flat
                [[0, 0, 0], [0, 0, 0], [0, 1, 0], [0, 0, 1]],      # repeated vertex
                [[0, 0, 0], [1, 0, 0], [2, 0, 0], [0, 0, 1]]):     # collinear face
        assert oracle.dihedral_minmax(np.array(bad, float).reshape(12)) == (0.0, math.pi)
    rng = np.random.default_rng(77)
    for k in range(300):
        t = rng.normal(size=12)
        if k % 3 == 0:
            t *= 1e-7                      # every nv component below 1e-5: rescaled
        a, b = oracle.dihedral_minmax(t)
        wa, wb = _dihedral_numpy(t)
        assert abs(a - wa) < 1e-9 and abs(b - wb) < 1e-9
        perm = rng.permutation(4)
        pa, pb = oracle.dihedral_minmax(t.reshape(4, 3)[perm].reshape(12))
        assert abs(pa - a) < 1e-12 and abs(pb - b) < 1e-12
