"""Learned warm start for the batched relaxation (new here; the reference has no counterpart).

For every stroke and height, a small MLP reads the force grid around the probe (3x3x3
trilinear samples one grid step apart, 3 components each) and the displacement converged at
the height above, and proposes the displacement FIRE starts from.  Plain FIRE then runs to
the same |F| < convergence criterion as without the network, and a proposal whose force
residual is larger than the plain start's is discarded, so the network can only change how
many iterations a height takes.  Its training pairs come from plain FIRE itself
(``generate_pairs``); training and inference are the library's own tcgen05 kernels.

    net = WarmStartNet(seed=0)
    X, T = generate_pairs(heldout_systems, params, relax, stride=4)
    net.train(X, T, steps=30000, batch=8192, lr=5e-4)
    bp = BatchPipeline(systems, params, relax)
    bp.run_layered(net)            # or bp.run_layered() for plain FIRE in the same schedule
"""

import ctypes
import math

import numpy as np
import torch

from ._lib import check, lib, stream_handle, tptr

NIN, NOUT_ROW = 96, 16


class WarmStartNet:
    """The network's parameters (float32 master copy + Adam state) on the device."""

    def __init__(self, seed=0, loss_weights=(1.0, 1.0, 10.0)):
        self.handle = ctypes.c_void_p()
        check(lib().ppgpu_mlp_create(int(seed), ctypes.byref(self.handle)))
        self.nparams = lib().ppgpu_mlp_nparams()
        self.steps = 0
        self.set_loss_weights(loss_weights)

    def set_loss_weights(self, w):
        """Per-output weights of the squared error (x, y, z of the displacement change); the
        default weights z 10x: an error along the stiff radial spring costs the most iterations."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        check(lib().ppgpu_mlp_set_loss_weights(self.handle, w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))

    def _get(self, which):
        out = np.zeros(self.nparams, dtype=np.float32)
        check(lib().ppgpu_mlp_get(self.handle, which, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    @property
    def params(self):
        return self._get(0)

    @params.setter
    def params(self, P):
        P = np.ascontiguousarray(P, dtype=np.float32)
        if P.shape != (self.nparams,):
            raise ValueError(f"expected {self.nparams} parameters")
        check(lib().ppgpu_mlp_set(self.handle, P.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def save(self, path):
        np.savez(path, params=self.params, steps=self.steps)

    def load(self, path):
        d = np.load(path)
        self.params = d["params"]
        self.steps = int(d["steps"])

    def forward(self, X):
        """X: [n, 96] bf16 device tensor (n multiple of 128) -> [n, 16] float32."""
        n = X.shape[0]
        Y = torch.empty((n, NOUT_ROW), dtype=torch.float32, device=X.device)
        check(lib().ppgpu_mlp_forward(self.handle, tptr(X.contiguous()), n, tptr(Y), stream_handle()))
        return Y

    def train(self, X, T, steps=1000, batch=8192, lr=1e-3, seed=0, log_every=100, schedule="constant"):
        """Adam on the mean squared error of minibatches drawn uniformly from (X, T).
        schedule: "constant" or "cosine" (lr decays to 2 % of lr by the last step).
        Returns [(step, loss)] every log_every steps."""
        if schedule not in ("constant", "cosine"):
            raise ValueError(f"unknown schedule {schedule!r}")
        n = X.shape[0]
        batch = min(batch, (n // 128) * 128)
        if batch < 128:
            raise ValueError("need at least 128 training pairs")
        g = torch.Generator(device=X.device).manual_seed(seed)
        log = []
        L = lib()
        st = stream_handle()
        last = 0
        for s in range(steps):
            idx = torch.randint(0, n, (batch,), generator=g, device=X.device, dtype=torch.int32)
            check(L.ppgpu_mlp_backward(self.handle, tptr(X), tptr(T), tptr(idx), batch, st))
            self.steps += 1
            lr_s = lr if schedule == "constant" else lr * (0.02 + 0.98 * 0.5 * (1.0 + math.cos(math.pi * s / max(1, steps - 1))))
            check(L.ppgpu_mlp_adam(self.handle, float(lr_s), self.steps, st))
            if (s + 1) % log_every == 0 or s == steps - 1:
                v = ctypes.c_double()
                check(L.ppgpu_mlp_take_loss(self.handle, ctypes.byref(v), st))
                log.append((self.steps, v.value / (s + 1 - last)))  # mean over the steps since the last read
                last = s + 1
        return log

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            lib().ppgpu_mlp_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def generate_pairs(systems, parameters, relax=None, stride=4, tuning=None):
    """Training pairs from plain FIRE on `systems`: every stride-th stroke at every height.
    Returns (X [n, 96] bf16, T [n, 4] float32) device tensors (targets: 10/A times the change
    of the converged displacement from the height above)."""
    from .batch import BatchPipeline

    bp = BatchPipeline(systems, parameters, relax=relax, want_ppos=False, tuning=tuning)
    info = (ctypes.c_longlong * 2)()
    check(lib().ppgpu_batch_layer_info(bp.handle, info))
    nstrokes, nz = int(info[0]), int(info[1])
    ns = ((nstrokes + stride - 1) // stride) * nz
    X = torch.zeros((ns, NIN), dtype=torch.bfloat16, device="cuda")
    T = torch.full((ns, 4), float("nan"), dtype=torch.float32, device="cuda")
    bp.run_layered(None, record=(stride, X, T))
    torch.cuda.synchronize()
    ok = ~torch.isnan(T[:, 0])  # tile padding and missing heights are never written
    X, T = X[ok].contiguous(), T[ok].contiguous()
    bp.close()
    return X, T
