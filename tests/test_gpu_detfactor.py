"""Batched Gauss-Jordan determinant/inverse (vsvb_det_factor) against
numpy float64, including an exactly singular block (rank deficiency of the
kind molecular symmetry produces in pi pairs)."""
import numpy as np
import pytest

from tests.gpu_helpers import built_lib, need_gpu

pytestmark = pytest.mark.gpu


def test_det_factor_matches_numpy():
    need_gpu()
    built_lib()
    import torch
    from valence_gb300 import api
    rng = np.random.default_rng(5)
    for n in (1, 3, 12, 40):
        a = rng.standard_normal((17, n, n)) + 2 * np.eye(n)
        if n > 2:
            a[4, 1, :] = 0.5 * a[4, 2, :]  # singular
        det, inv, sing = api.det_factor(torch.from_numpy(a).cuda())
        det, inv, sing = det.cpu().numpy(), inv.cpu().numpy(), sing.cpu().numpy()
        for m in range(len(a)):
            ref = np.linalg.det(a[m])
            if n > 2 and m == 4:
                # exactly singular: |det| is round-off against the Hadamard bound
                hadamard = np.prod(np.linalg.norm(a[m], axis=1))
                assert abs(det[m]) <= 1e-12 * hadamard
                assert sing[m] == 1
                assert np.all(inv[m] == 0.0)
            else:
                assert abs(det[m] - ref) <= 1e-11 * max(1.0, abs(ref)), (n, m, det[m], ref)
                assert sing[m] == 0
                assert np.allclose(inv[m], np.linalg.inv(a[m]), rtol=1e-9, atol=1e-11)
