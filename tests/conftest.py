import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name + ".npz")))

    return load


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def gpulib():
    """Builds (if needed) and loads libppgpu.so; GPU tests only."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from ppafm_gb300 import _lib, build

    build.build()
    L = _lib.load()
    import ctypes

    buf = ctypes.create_string_buffer(128)
    _lib.check(L.ppgpu_device_info(buf, 128))
    return L


def rel_err(a, b, floor):
    """max over points of |a-b| / max(|b|, floor) with vector norms over the last axis."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.ndim >= 1 and a.shape[-1] == 3:
        d = np.linalg.norm(a - b, axis=-1)
        m = np.linalg.norm(b, axis=-1)
    else:
        d = np.abs(a - b)
        m = np.abs(b)
    return float(np.max(d / np.maximum(m, floor))) if d.size else 0.0
