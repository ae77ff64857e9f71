"""The allocation-free Gram-Schmidt entry point (tagi_mgs_dev_noalloc).

Some callers cannot allocate device memory during a call -- their device
memory belongs to another allocator or a fixed budget, or a cudaMalloc would
synchronize the device inside a latency-critical loop.  For them the library
offers an MGS variant whose scratch lives in a fixed device array.  These
tests call it through the C ABI and compare it with tagi_mgs_dev on calls
in a row (the shared scratch keeps the first call's contents), within the
1e-13 relative tolerance of the other MGS tests.  This file sorts last so a
run that stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_rejects_too_many_rows(native):
    """More than 128 earlier rows does not fit the fixed scratch: refused on the host."""
    L = native.lib()
    rc = L.tagi_mgs_dev_noalloc(None, None, None, 129, 10, 200, None)
    assert rc == native.TAGI_ERR_ARG
    assert b"128" in L.tagi_last_error_message()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1000, 300_001])
@pytest.mark.parametrize("m,targets", [(9, (5, 8)), (129, (0, 1, 128))])
def test_noalloc_matches_allocating_mgs_on_calls_in_a_row(native, n, m, targets):
    """Calls in a row on the shared scratch, each against tagi_mgs_dev on the
    same input: no earlier rows (0), one, and the largest count the scratch
    holds (128 rows of per-block partials); few points (fewer blocks than
    the scratch's 1024 block slots and than 4 per SM) and many."""
    import torch

    L = native.lib()
    rng = np.random.default_rng(42 + n + m)
    V0 = torch.as_tensor(rng.normal(size=(m, n)), dtype=torch.float64, device="cuda")
    W = torch.as_tensor(rng.uniform(0.2, 2.0, n), dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    Va, Vb = V0.clone(), V0.clone()
    for target in targets:
        Ua, Ub = Va[target].clone(), Vb[target].clone()
        native.check(L.tagi_mgs_dev(_ptr(Va), _ptr(Ua), _ptr(W), target, n, m, stream))
        native.check(L.tagi_mgs_dev_noalloc(_ptr(Vb), _ptr(Ub), _ptr(W), target, n, m, stream))
        torch.cuda.synchronize()
        ref, got = Ua.cpu().numpy(), Ub.cpu().numpy()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-13, target
        assert np.max(np.abs(Vb.cpu().numpy() - Va.cpu().numpy())) <= 1e-13
