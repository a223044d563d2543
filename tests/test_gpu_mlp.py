"""The warm-start network on the tcgen05 tensor cores: the MMA building block, then the
network's forward/backward against the numpy float64 oracle and the trained network's gain."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("K,N", [(16, 16), (96, 128), (128, 128), (128, 16), (64, 256)])
def test_tc_selftest(gpulib, K, N):
    import torch

    from ppafm_gb300 import _lib

    rng = np.random.default_rng(K * 1000 + N)
    A = torch.tensor(rng.standard_normal((128, K)), dtype=torch.bfloat16, device="cuda")
    B = torch.tensor(rng.standard_normal((N, K)), dtype=torch.bfloat16, device="cuda")
    D = torch.zeros((128, N), dtype=torch.float32, device="cuda")
    _lib.check(gpulib.ppgpu_tc_selftest(_lib.tptr(A), _lib.tptr(B), K, N, _lib.tptr(D), _lib.stream_handle()))
    _lib.check(gpulib.ppgpu_device_status(_lib.stream_handle()))
    ref = A.float().cpu().double().numpy() @ B.float().cpu().double().numpy().T
    got = D.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max() + 1e-4
