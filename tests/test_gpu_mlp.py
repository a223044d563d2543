"""The warm-start network on the tcgen05 tensor cores: the MMA building block, then the
network's forward/backward against the numpy float64 oracle and the trained network's gain."""

import numpy as np
import pytest

from oracle.mlp_oracle import IN as NIN

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


def _net(seed=3):
    import ctypes

    from ppafm_gb300 import _lib

    L = _lib.lib()
    h = ctypes.c_void_p()
    _lib.check(L.ppgpu_mlp_create(seed, ctypes.byref(h)))
    return L, h


def _params(L, h, which=0):
    from ppafm_gb300 import _lib

    n = L.ppgpu_mlp_nparams()
    out = np.zeros(n, dtype=np.float32)
    _lib.check(L.ppgpu_mlp_get(h, which, out.ctypes.data_as(_lib.POINTER(_lib.c_float))))
    return out


def _data(n, seed):
    import torch

    rng = np.random.default_rng(seed)
    X = rng.normal(0, 1, (n, NIN)).astype(np.float32)
    X[:, 81:90] *= 0.5
    X[:, 90:] = 0.0
    T = rng.normal(0, 0.5, (n, 4)).astype(np.float32)
    Xd = torch.tensor(X, dtype=torch.bfloat16, device="cuda")
    Td = torch.tensor(T, device="cuda")
    return X, T, Xd, Td


def test_mlp_forward_vs_oracle(gpulib):
    """bf16 network on the tensor cores against the float64 restatement with the same bf16
    roundings: max |dy| <= 1e-2 of max |y| (SiLU uses a hardware exp; a rounding flip of
    one bf16 activation moves an output by ~2^-9 of its scale)."""
    import torch

    from ppafm_gb300 import _lib
    from oracle import mlp_oracle as MO

    L, h = _net()
    X, T, Xd, Td = _data(512, 1)
    Y = torch.zeros((512, 16), device="cuda")
    _lib.check(L.ppgpu_mlp_forward(h, _lib.tptr(Xd), 512, _lib.tptr(Y), _lib.stream_handle()))
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))
    P = _params(L, h)
    ref = MO.forward(P, X)["y"]
    got = Y.cpu().numpy().astype(np.float64)
    assert np.abs(got[:, :3] - ref[:, :3]).max() <= 1e-2 * np.abs(ref[:, :3]).max()
    assert np.abs(got[:, 3:]).max() < 1e-6  # unused outputs: zero weights and bias
    L.ppgpu_mlp_destroy(h)


def test_mlp_gradients_vs_oracle(gpulib):
    """Gradients from the tensor-core forward/backward kernels against the float64
    restatement (same bf16 roundings): relative error of every parameter block's gradient
    <= 2e-2 in the 2-norm."""
    import ctypes

    import torch

    from ppafm_gb300 import _lib
    from oracle import mlp_oracle as MO

    L, h = _net(5)
    n = 512
    X, T, Xd, Td = _data(n, 2)
    idx = torch.randperm(n, generator=torch.Generator().manual_seed(0)).to(torch.int32).cuda()
    _lib.check(L.ppgpu_mlp_backward(h, _lib.tptr(Xd), _lib.tptr(Td), _lib.tptr(idx), n, _lib.stream_handle()))
    loss = ctypes.c_double()
    _lib.check(L.ppgpu_mlp_take_loss(h, ctypes.byref(loss), _lib.stream_handle()))
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))
    G = _params(L, h, 1).astype(np.float64)
    P = _params(L, h)
    ii = idx.cpu().numpy()
    lref, gref = MO.loss_and_grad(P, X[ii], T[ii])
    assert abs(loss.value - lref) <= 1e-2 * lref
    o = 0
    for name, shp in MO.SIZES:
        k = int(np.prod(shp))
        a, b = G[o : o + k], gref[o : o + k]
        o += k
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-7, name
    L.ppgpu_mlp_destroy(h)


def test_mlp_adam_step_vs_oracle(gpulib):
    import torch

    from ppafm_gb300 import _lib
    from oracle import mlp_oracle as MO

    L, h = _net(7)
    n = 256
    X, T, Xd, Td = _data(n, 3)
    idx = torch.arange(n, dtype=torch.int32, device="cuda")
    P0 = _params(L, h).astype(np.float64)
    _lib.check(L.ppgpu_mlp_backward(h, _lib.tptr(Xd), _lib.tptr(Td), _lib.tptr(idx), n, _lib.stream_handle()))
    G = _params(L, h, 1).astype(np.float64)
    _lib.check(L.ppgpu_mlp_adam(h, 1e-3, 1, _lib.stream_handle()))
    P1 = _params(L, h).astype(np.float64)
    ref, _, _ = MO.adam(P0, G, np.zeros_like(P0), np.zeros_like(P0), 1e-3, 1)
    assert np.abs(P1 - ref).max() < 1e-6
    assert np.abs(_params(L, h, 1)).max() == 0.0  # gradients cleared
    L.ppgpu_mlp_destroy(h)


def test_mlp_training_reduces_loss(gpulib):
    """A smooth synthetic target learned by the hand-written training kernels."""
    import ctypes

    import torch

    from ppafm_gb300 import _lib

    L, h = _net(11)
    n = 8192
    rng = np.random.default_rng(4)
    X = rng.normal(0, 1, (n, NIN)).astype(np.float32)
    X[:, 90:] = 0
    Wt = rng.normal(0, 0.3, (90, 3))
    T = np.zeros((n, 4), np.float32)
    T[:, :3] = np.tanh(X[:, :90] @ Wt)
    Xd = torch.tensor(X, dtype=torch.bfloat16, device="cuda")
    Td = torch.tensor(T, device="cuda")
    losses = []
    g = torch.Generator().manual_seed(1)
    for step in range(1, 301):
        idx = torch.randperm(n, generator=g)[:1024].to(torch.int32).cuda()
        _lib.check(L.ppgpu_mlp_backward(h, _lib.tptr(Xd), _lib.tptr(Td), _lib.tptr(idx), 1024, _lib.stream_handle()))
        _lib.check(L.ppgpu_mlp_adam(h, 1e-3, step, _lib.stream_handle()))
        v = ctypes.c_double()
        _lib.check(L.ppgpu_mlp_take_loss(h, ctypes.byref(v), _lib.stream_handle()))  # this step's loss
        if step in (1, 300):
            losses.append(v.value)
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))
    assert losses[1] < 0.2 * losses[0], losses
    L.ppgpu_mlp_destroy(h)
