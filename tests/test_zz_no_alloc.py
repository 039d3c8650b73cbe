"""The allocation-free determinant/inverse entry point.

Callers whose device memory belongs to another framework's allocator, or
that run where device allocation is forbidden, use
vsvb_det_factor_noalloc, whose scratch is a fixed device array instead of a
cudaMalloc.  This checks it through the C ABI against the allocating
vsvb_det_factor on the same inputs, for two calls in a row (the shared
scratch keeps the previous call's contents), and that oversized requests are
refused before any GPU work.  Collected last (test_zz_*) so a failing run
that stops at the first failure has already run everything else.
"""
import ctypes

import numpy as np
import pytest

from tests.gpu_helpers import built_lib, need_gpu

pytestmark = pytest.mark.gpu


def _call(fn, a):
    import torch
    nmat, n, _ = a.shape
    det = torch.full((nmat,), float("nan"), dtype=torch.float64, device="cuda")
    inv = torch.full_like(a, float("nan"))
    sing = torch.full((nmat,), -1, dtype=torch.int32, device="cuda")
    rc = fn(ctypes.c_void_p(a.data_ptr()), n, nmat, ctypes.c_void_p(det.data_ptr()), ctypes.c_void_p(inv.data_ptr()),
            ctypes.c_void_p(sing.data_ptr()), None)
    assert rc == 0
    return det.cpu().numpy(), inv.cpu().numpy(), sing.cpu().numpy()


def test_noalloc_matches_allocating_entry_point():
    need_gpu()
    built_lib()
    import torch
    from valence_gb300 import api
    L = api.lib()
    rng = np.random.default_rng(11)
    for call, n in enumerate((12, 7)):
        a = rng.standard_normal((64, n, n)) + 2 * np.eye(n)
        a[3, 2, :] = 0.25 * a[3, 5, :]  # one exactly singular block
        ta = torch.from_numpy(a).cuda()
        d0, i0, s0 = _call(L.vsvb_det_factor, ta)
        d1, i1, s1 = _call(L.vsvb_det_factor_noalloc, ta)
        assert np.array_equal(s0, s1), call
        assert np.allclose(d1, d0, rtol=1e-12, atol=1e-12 * np.abs(d0).max()), call
        assert np.allclose(i1, i0, rtol=1e-12, atol=1e-12), call
        assert s1[3] == 1 and np.all(s1[np.arange(64) != 3] == 0)


def test_noalloc_rejects_oversized_requests():
    need_gpu()
    built_lib()
    from valence_gb300 import api
    L = api.lib()
    null = ctypes.c_void_p(1)
    # 2 * 64 * 64 * 65 doubles > 4 MiB: refused before touching the (dummy) pointers
    rc = L.vsvb_det_factor_noalloc(null, 64, 65, null, null, null, None)
    assert rc == 8  # VSVB_ERR_TOO_LARGE
