"""The no-allocation Lennard-Jones entry point (ppgpu_lj_grid_f64_noalloc).

Some callers cannot allocate device memory when they call the library: their own
allocator reserved the device memory up front, or they run latency-sensitive loops that
cannot take the device-wide synchronisation of cudaMalloc/cudaFree.  This entry point
stages its scratch in a fixed array inside the library instead.  The test calls it through
the C ABI with device buffers the test allocates beforehand, twice in a row on the same
grid (the second call accumulates a different atom set on top of the first, so stale
scratch from the first call would show), and compares with the drop-in getLennardJonesFF
(which allocates its own scratch) under the same tolerance as the other force-field tests.
The second pair of calls must leave the device's free memory (cudaMemGetInfo) unchanged,
and ppgpu_device_status must report no timeout.  The file is named to be collected last.
"""

import ctypes

import numpy as np
import pytest

from tests.conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-5
FLOOR = 1e-2


def _dropin(n, lvec, sets, with_E):
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import core

    FF, V = HL.setFF(None, with_E, n=n, lvec=lvec)
    for R, c in sets:
        core.getLennardJonesFF(np.ascontiguousarray(R), np.ascontiguousarray(c))
    core.deleteFF_Fpointer()
    core.deleteFF_Epointer()
    return FF, V


def _noalloc(L, n, lvec, sets, with_E):
    """Runs the calls on buffers allocated beforehand; returns (F, E, free bytes before the
    calls, free bytes after them)."""
    import torch

    from ppafm_gb300 import _lib

    nn = np.ascontiguousarray(n, dtype=np.int32)
    cell = np.ascontiguousarray(lvec[1:4], dtype=np.float64)
    F = torch.zeros((int(np.prod(nn)), 3), dtype=torch.float64, device="cuda")
    E = torch.zeros(int(np.prod(nn)), dtype=torch.float64, device="cuda") if with_E else None
    dev = [(torch.as_tensor(np.ascontiguousarray(R)).cuda(), torch.as_tensor(np.ascontiguousarray(c)).cuda()) for R, c in sets]
    torch.cuda.synchronize()  # every buffer exists before the calls
    free0 = torch.cuda.mem_get_info()[0]
    st = _lib.stream_handle()
    for (R, c), (Rd, cd) in zip(sets, dev):
        _lib.check(L.ppgpu_lj_grid_f64_noalloc(_lib.tptr(F), _lib.tptr(E), _lib.iptr(nn), _lib.dptr(cell), len(R), _lib.tptr(Rd), _lib.tptr(cd), st))
    _lib.check(L.ppgpu_device_status(st))  # synchronises; no bounded wait gave up
    free1 = torch.cuda.mem_get_info()[0]
    return F.cpu().numpy().reshape(tuple(nn) + (3,)), (E.cpu().numpy().reshape(tuple(nn)) if with_E else None), free0, free1


@pytest.mark.parametrize("shape", ["planes", "columns"])
def test_noalloc_matches_dropin_twice(gpulib, shape):
    rng = np.random.default_rng(17)
    if shape == "planes":  # whole (y, z) planes per chunk
        n = np.array([40, 36, 30], np.int32)
        lvec = np.array([[0.0, 0, 0], [8.0, 0, 0], [0.5, 7.2, 0], [0, 0, 6.0]])
    else:  # a y-z plane larger than the chunk: runs of z columns
        n = np.array([3, 700, 400], np.int32)
        lvec = np.array([[0.0, 0, 0], [0.6, 0, 0], [0, 70.0, 0], [0, 0, 40.0]])
    L = lvec[1:4].diagonal()
    sets = []
    for na in (57, 23):
        R = np.column_stack([rng.uniform(0, L[0], na), rng.uniform(0, L[1], na), rng.uniform(0, L[2], na)])
        c = np.column_stack([rng.uniform(10, 60, na), rng.uniform(1e4, 8e4, na)])
        sets.append((R, c))
    F0, E0 = _dropin(n, lvec, sets, True)
    F1, E1, _, _ = _noalloc(gpulib, n, lvec, sets, True)
    ok = np.linalg.norm(F0, axis=-1) < 1e30
    assert rel_err(F1[ok], F0[ok], FLOOR) < TOL
    assert rel_err(E1[ok], E0[ok], FLOOR) < 1e-4
    # repeat the pair of calls: the shared scratch keeps the last call's contents, and the
    # calls (device code loaded by the first pair) take no device memory
    F2, _, free0, free1 = _noalloc(gpulib, n, lvec, sets, False)
    assert rel_err(F2[ok], F0[ok], FLOOR) < TOL
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes across the calls"


def test_noalloc_rejects_oversized_requests(gpulib):
    import torch

    from ppafm_gb300 import _lib

    L = gpulib
    n = np.array([4, 4, 4], np.int32)
    cell = np.eye(3) * 3.0
    F = torch.zeros((64, 3), dtype=torch.float64, device="cuda")
    R = torch.zeros((1, 3), dtype=torch.float64, device="cuda")
    c = torch.zeros((1, 2), dtype=torch.float64, device="cuda")
    st = L.ppgpu_lj_grid_f64_noalloc(_lib.tptr(F), None, _lib.iptr(n), _lib.dptr(cell), 32769, _lib.tptr(R), _lib.tptr(c), _lib.stream_handle())
    assert st == _lib.PPGPU_ERR_ARG and "atoms" in _lib.last_error()
    big = np.array([1, 1, 300000], np.int32)
    st = L.ppgpu_lj_grid_f64_noalloc(_lib.tptr(F), None, _lib.iptr(big), _lib.dptr(cell), 1, _lib.tptr(R), _lib.tptr(c), _lib.stream_handle())
    assert st == _lib.PPGPU_ERR_ARG
