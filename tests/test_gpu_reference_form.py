"""GPU: the binary64 AMIPS evaluations against the reference's own routines.

The default energy form (TW_ENERGY_FORM_REFERENCE) performs the operations of
the reference's generated expressions (LocalOperations.cpp:28-291) in their
order, so the device agrees with the reference's compiled routines
(oracle/_ref) to its rounding: the tolerance is 1e-12 relative per entry of
E, J and H, with no allowance for position or conditioning.  The smoothing
pass decides with those energies; run against the oracle's libm build, whose
energies are the reference's bit for bit, it must take identical decisions
(every status, every moved flag).  The positions are continuous functions of
J and H, whose last bits follow pow (libm's against the device's; libm's pow
itself is not correctly rounded on ~0.07% of these arguments), and Newton's
3x3 solve and the surface projection amplify a one-ulp change by the
conditioning of the star: on the 200k-star batch the positions of the two
oracle builds differ by at most 6.8e-16 on 99% of the stars, 8.2e-15 on 99.9%
and 4.6e-10 on the worst (a surface star).  The test bounds that spread.
"""
import numpy as np
import pytest

import tetwild_gb300 as tw
from conftest import golden
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12   # binary64 E/J/H against the reference's routines, per entry
POS_TOL_999 = 1e-13   # positions, relative to max(1, |coordinate|): 99.9% of the stars
POS_TOL_MAX = 1e-9    # and every star
EPS = 1e-3


def _pos_err(a, b):
    return np.abs(a - b).max(axis=1) / np.maximum(1.0, np.abs(b).max(axis=1))


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    d = np.abs(a - b)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(d == 0, 0.0, d / np.abs(b))
    return r


def test_reference_form_full_energy_batch_vs_reference(ctx, reflib):
    """All 4M tets of the bench's energy batch: E, J, H against the reference's
    comformalAMIPS{Energy,Jacobian,Hessian}_new, 1e-12 relative per entry."""
    from oracle.oracle import default_threads

    T = syn.energy_batch(4_000_000, seed=0)
    g = ctx.amips(T, tw.TW_ENERGY_RAW, flip=False)
    Er, Jr, Hr = reflib.amips_batch_soa(T, nthreads=default_threads())
    rE, rJ, rH = _rel(g["E"], Er), _rel(g["J"], Jr), _rel(g["H"], Hr)
    print(f"max rel: E {rE.max():.3e}  J {rJ.max():.3e}  H {rH.max():.3e}")
    assert rE.max() <= REL_TOL and rJ.max() <= REL_TOL and rH.max() <= REL_TOL


def test_reference_form_golden(ctx):
    """Every tet of the reference's fixture (benchmark, near-flat, scaled from 1e-6 to
    1e3, origin-centred): 1e-12 relative per entry."""
    g = golden("amips_ref.npz")
    T = np.ascontiguousarray(g["T"].T)
    out = ctx.amips(T, tw.TW_ENERGY_RAW, flip=False)
    assert _rel(out["E"], g["E"]).max() <= REL_TOL
    assert _rel(out["J"], g["J"].T).max() <= REL_TOL
    assert _rel(out["H"], g["H"].T).max() <= REL_TOL


def test_closed_form_option_bitwise(ctx, oracle):
    """TW_ENERGY_FORM_CLOSED: bit for bit the oracle's closed form, in the batch and
    through the Newton step."""
    T = syn.energy_batch(200_000, seed=5)
    ctx.set_energy_form(tw.TW_ENERGY_FORM_CLOSED)
    oracle.set_energy_form(1)
    try:
        g = ctx.amips(T, tw.TW_ENERGY_QUALITY)
        E, J, H, F = oracle.amips_batch_soa(T, quality=True, nthreads=8)
        assert np.array_equal(g["E"], E) and np.array_equal(g["flip"], F)
        assert np.array_equal(g["J"], J) and np.array_equal(g["H"], H)
        xyz, off, tets, cen = syn.star_batch(2000, seed=6)
        ctx.mesh_upload(xyz)
        ctx.set_params(EPS * EPS, EPS / 2, 15, 20)
        out, moved = ctx.newton_stars(off, tets, cen)
        want, wmoved = oracle.newton_stars(xyz, off, tets, cen, 15, 20, nthreads=8)
        assert np.array_equal(out, want) and np.array_equal(moved, wmoved)
    finally:
        ctx.set_energy_form(tw.TW_ENERGY_FORM_REFERENCE)
        oracle.set_energy_form(0)
    # the two forms differ (by the reference's rounding), so the switch is live
    g2 = ctx.amips(T, tw.TW_ENERGY_QUALITY, jacobian=False, hessian=False, flip=False)
    assert not np.array_equal(g2["E"], E)


def test_smooth_pass_with_reference_energies(ctx):
    """The bench's 200k-star smoothing pass (half surface stars), both precision modes,
    against the oracle's libm build, whose AMIPS energies, gradients and Hessians are
    the reference's own bit for bit: every status identical, positions within the
    conditioning spread (module docstring)."""
    from oracle.oracle import Oracle, default_threads

    o = Oracle(libm=True)
    V, F = syn.displaced_sphere(seed=0)
    xyz, off, tets, ff, cen, kinds = syn.mixed_star_batch(V, F, 200_000, EPS, seed=11,
                                                          surface_fraction=0.5)
    S = o.surface(V, F)
    want, wst = o.smooth_stars(xyz, off, tets, cen, ff, kinds, surface=S, boundary=S,
                               eps2=EPS * EPS, sd=EPS / 2, max_step=1, max_it=8,
                               nthreads=default_threads())
    ctx.set_params(EPS * EPS, EPS / 2, 1, 8)
    ctx.surface_upload(V, F)
    ctx.mesh_upload(xyz)
    for precision in (tw.TW_PRECISION_FP64, tw.TW_PRECISION_FP32_CERTIFIED):
        ctx.set_precision(precision)
        try:
            out, st = ctx.smooth_stars(off, tets, cen, ff, kinds)
        finally:
            ctx.set_precision(tw.TW_PRECISION_FP64)
        n_status = int((st.astype(np.int8) != wst).sum())
        err = _pos_err(out, want)
        q = np.quantile(err, [0.5, 0.99, 0.999])
        print(f"precision {precision}: status mismatches {n_status}; position error "
              f"median {q[0]:.2e}, 99% {q[1]:.2e}, 99.9% {q[2]:.2e}, max {err.max():.2e} "
              f"({int((err > 0).sum())} stars not bit-identical)")
        assert n_status == 0
        assert q[2] <= POS_TOL_999 and err.max() <= POS_TOL_MAX


def test_newton_with_reference_energies(ctx):
    """NewtonsMethod at the reference's caps (15 steps, 20 halvings) on 20k interior
    stars against the oracle's libm build (the reference's energies bit for bit): the
    moved flags are identical.  Run to convergence, the line search compares the energy
    of a trial position (tets in stored order, VertexSmoother.cpp:606-614) against the
    energy at nearly the same point summed with each tet rotated (:640-651), a
    comparison that rounding decides, so a one-ulp change of pow flips some of those
    internal accept/reject steps: ~15% of the stars end up to ~1e-8 apart (measured on
    the CPU between the two oracle builds: 1.2e-8 at most)."""
    from oracle.oracle import Oracle, default_threads

    o = Oracle(libm=True)
    xyz, off, tets, cen = syn.star_batch(20_000, seed=7)
    ctx.mesh_upload(xyz)
    ctx.set_params(EPS * EPS, EPS / 2, 15, 20)
    out, moved = ctx.newton_stars(off, tets, cen)
    want, wmoved = o.newton_stars(xyz, off, tets, cen, 15, 20, nthreads=default_threads())
    err = _pos_err(out, want)
    print(f"moved flags identical: {np.array_equal(moved, wmoved)}, position error 99.9% "
          f"{np.quantile(err, 0.999):.2e}, max {err.max():.2e}")
    assert np.array_equal(moved, wmoved)
    assert err.max() <= 1e-7
