"""Device self-tests: the integer-arithmetic binary64 <-> binary32 conversions
that the certified mode uses instead of the FP64-pipe hardware conversions
must agree with the hardware bit for bit, and the bulk-copy kernel's bounded
mbarrier wait must give up (not hang) on a phase that never completes."""
import numpy as np
import pytest

import tetwild_gb300 as tw

pytestmark = pytest.mark.gpu


def test_integer_conversions_match_hardware(ctx):
    d2f_fail, f2d_fail = ctx.self_test(1 << 26)
    assert d2f_fail == 0
    assert f2d_fail == 0


def test_bounded_wait_gives_up_and_the_context_stays_usable(ctx, oracle):
    """The bulk-copy kernel's mbarrier wait: a phase no copy completes gives up after its
    poll limit (no hang, no fault), a phase fed by a bulk copy completes with the copied
    bytes, and the next bulk-staged AMIPS batch on the same context is exact."""
    import torch

    from tetwild_gb300 import synthetic as syn

    r = ctx.self_test_wait(1 << 12)
    assert r["timed_out"] and r["completed"] and r["copied"] == 1.5 and r["cycles"] > 0
    n = 64 * 256 * 2                        # device memory, even, >= 64 tiles: the bulk path
    T = syn.energy_batch(n, seed=9)
    dev = torch.device("cuda:0")
    dT = torch.from_numpy(T).to(dev)
    E = torch.empty(n, dtype=torch.float64, device=dev)
    Fl = torch.empty(n, dtype=torch.uint8, device=dev)
    ctx.set_precision(tw.TW_PRECISION_FP32_CERTIFIED)
    try:
        ctx.amips_device(dT.data_ptr(), n, tw.TW_ENERGY_QUALITY, E.data_ptr(), 0, 0, Fl.data_ptr())
        ctx.synchronize()
    finally:
        ctx.set_precision(tw.TW_PRECISION_FP64)
    We, _, _, Wf = oracle.amips_batch_soa(T, quality=True, jacobian=False, hessian=False)
    e = E.cpu().numpy()
    assert np.array_equal(Fl.cpu().numpy(), Wf)
    fin = We < 1e50
    assert np.array_equal(e >= 1e50, ~fin) and np.max(np.abs(e[fin] - We[fin]) / We[fin]) <= 1e-5
