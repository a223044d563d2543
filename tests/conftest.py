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


FF_TOL = 1e-5
FF_FLOOR = 1e-2
SUM_ULPS = 2.0**-20  # 16 float32 ulps (u = 2^-24)
SUM_CLAUSE_FRAC = 1e-3


def term_magnitudes(pts, Rs0, cLJs, kqq, Q):
    """sum_i |F_LJ,i(p)| + |Q| sum_i |F_el,i(p)| at points p (grid-origin frame), float64."""
    out = np.zeros(len(pts))
    kqq = np.zeros(len(Rs0)) if kqq is None else np.asarray(kqq)
    for k, p in enumerate(pts):
        d = p[None, :] - Rs0
        r2 = np.einsum("ij,ij->i", d, d) + 1e-8
        ir2 = 1.0 / r2
        ir6 = ir2**3
        flj = np.abs((12.0 * cLJs[:, 1] * ir6 - 6.0 * cLJs[:, 0]) * ir6 * ir2) * np.sqrt(r2)
        out[k] = flj.sum() + abs(Q) * (np.abs(kqq) * ir2).sum()
    return out


def check_ff(name, got, ref, coords, Rs0, cLJs, kqq, Q):
    """The float32 force-grid bar against a float64 reference (grids [..., 3]): every point
    within 1e-5 relative (|dF| <= 1e-5 max(|F|, 1e-2 eV/A)), except where that is finer than
    float32 resolves.  A float32 evaluation of a sum of pair terms carries an error of a few
    ulps of the terms' magnitudes sum_i |F_i|, so where the terms cancel (|F| << sum_i |F_i|:
    between atoms, and inside repulsive cores where the 10 eV/A clamp keeps only the
    direction of a large sum) a point passes at |dF| <= 2^-20 sum_i |F_i| (16 ulps); at most
    1 in 10^3 points may need that clause.  coords(idx) gives the grid-origin-frame positions
    of index tuples.  Prints the float32 error; returns the max relative error."""
    d = np.linalg.norm(got - ref, axis=-1)
    m = np.linalg.norm(ref, axis=-1)
    err = d / np.maximum(m, FF_FLOOR)
    over = np.argwhere(err > FF_TOL)
    worst_sum = 0.0
    if len(over):
        assert len(over) <= SUM_CLAUSE_FRAC * err.size, f"{name}: {len(over)} of {err.size} points beyond {FF_TOL} relative"
        S = term_magnitudes(coords(over), Rs0, cLJs, kqq, Q)
        ratio = d[tuple(over.T)] / (SUM_ULPS * S)
        worst_sum = float(ratio.max())
        assert worst_sum <= 1.0, f"{name}: a point beyond both 1e-5 relative and the float32 summation bound ({worst_sum:.2f} of it)"
    print(f"{name}: float32 max rel err {err.max():.2e}; {len(over)} of {err.size} points past 1e-5 (within {worst_sum:.2f} of the float32 summation bound)")
    return float(err.max())


def grid_coords(n, lvec):
    """coords(idx) of check_ff for a whole grid of size n and lattice lvec (origin + 3 rows)."""
    dc = np.asarray(lvec, dtype=np.float64)[1:4] / np.asarray(n)[:, None]
    return lambda idx: idx @ dc
