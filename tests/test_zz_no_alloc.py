"""tw_amips_soa_noalloc: the AMIPS batch for callers that cannot let the
library allocate device memory (their own allocator owns the free HBM, or
they must not stall on cudaFree's device-wide synchronisation).

The entry point keeps its scratch in a fixed device array, so this checks,
through the C-ABI, that two calls in a row give exactly what the allocating
entry point tw_amips_soa gives (the second call smaller than the first, so
stale scratch from the first call would show), that the second call changes
the device's free memory by nothing, and that a batch over the fixed
capacity is refused.  The file sorts last so that a run stopping at the
first failure has already run every other test.
"""
import numpy as np
import pytest

import tetwild_gb300 as tw
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

CAPACITY = 65536  # TW_NOALLOC_MAX_TETS in include/tw_gb300.h


def _noalloc(lib, T, mode=tw.TW_ENERGY_QUALITY):
    n = T.shape[1]
    E, J, H = np.empty(n), np.empty((3, n)), np.empty((9, n))
    F = np.empty(n, np.uint8)
    st = lib.tw_amips_soa_noalloc(T.ctypes.data, n, mode, E.ctypes.data, J.ctypes.data,
                                  H.ctypes.data, F.ctypes.data, None)
    return st, E, J, H, F


def _same(a, b):
    fa, fb = np.isfinite(a), np.isfinite(b)
    return np.array_equal(fa, fb) and np.array_equal(a[fa], b[fb])


def test_noalloc_matches_allocating_entry_point_on_two_calls(ctx):
    import torch

    lib = tw.load_library()
    # first call: the full capacity, with inverted and flat tets mixed in
    T1 = np.ascontiguousarray(syn.energy_batch(CAPACITY, seed=101, sigma_rel=0.3))
    # second call: smaller, different tets (stale scratch would show up here)
    T2 = np.ascontiguousarray(syn.energy_batch(40_000, seed=202))
    for k, T in enumerate((T1, T2)):
        free_before = torch.cuda.mem_get_info()[0]
        st, E, J, H, F = _noalloc(lib, T)
        free_after = torch.cuda.mem_get_info()[0]
        assert st == tw.TW_OK
        if k == 1:
            assert free_after == free_before
        want = ctx.amips(T, tw.TW_ENERGY_QUALITY)
        assert np.array_equal(F, want["flip"])
        assert np.array_equal(E, want["E"])
        assert _same(J, want["J"]) and _same(H, want["H"])
    assert F.sum() == 0 and want["flip"].sum() == 0
    assert (E < 1e50).all()


def test_noalloc_refuses_batches_over_capacity():
    lib = tw.load_library()
    T = np.zeros((12, CAPACITY + 1))
    st, *_ = _noalloc(lib, T)
    assert st == tw.TW_ERR_TOO_LARGE
