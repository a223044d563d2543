"""The C ABI's error behaviour, on the CPU: each call below is rejected (or, for empty work,
accepted) before the library touches a GPU -- the device API with PPGPU_ERR_ARG (1), the
drop-in symbols called before the state they need with PPGPU_ERR_STATE (3) -- and a message
naming the problem in ppgpu_last_error: what a caller binding include/ppgpu.h relies on.
Pointers that the checks do not dereference are placeholders."""

import ctypes

import numpy as np
import pytest

PPGPU_OK, PPGPU_ERR_ARG = 0, 1


@pytest.fixture(scope="module")
def L():
    from ppafm_gb300 import _lib, build

    build.build()
    return _lib.load()


def _msg(L):
    return L.ppgpu_last_error().decode()


def _ip(a):
    return np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))


CELL = np.eye(3) * 10.0
FAKE = ctypes.c_void_p(0x1000)  # 16-byte aligned placeholder, never dereferenced by the checks


def _ff(L, FE=FAKE, n=(8, 8, 8), cell=CELL, i0=(0, 0, 0), ns=(8, 8, 8), atoms=FAKE, natoms=4, ncharged=2, mode=2, kind=0, Qs=None, QZs=None):
    n = np.asarray(n, np.int32)
    cellv = np.ascontiguousarray(cell, dtype=np.float64)
    return L.ppgpu_ff_subgrid(FE, _ip(n), _dp(cellv), _ip(i0), _ip(ns), atoms, natoms, ncharged, mode, kind, 0.0, 0.0, None if Qs is None else _dp(Qs), None if QZs is None else _dp(QZs), 0, None)


def test_force_field_argument_checks(L):
    assert L.ppgpu_ff_grid(FAKE, None, _dp(CELL), FAKE, 1, 0, 0, 0, 0.0, 0.0, None, None, 0, None) == PPGPU_ERR_ARG
    assert "null n" in _msg(L)
    assert _ff(L, FE=None) == PPGPU_ERR_ARG and "null argument" in _msg(L)
    assert _ff(L, natoms=2, ncharged=3) == PPGPU_ERR_ARG and "atom counts" in _msg(L)
    assert _ff(L, atoms=None) == PPGPU_ERR_ARG and "null atoms" in _msg(L)
    assert _ff(L, FE=ctypes.c_void_p(0x1004)) == PPGPU_ERR_ARG and "16-byte aligned" in _msg(L)
    assert _ff(L, i0=(0, 4, 0), ns=(8, 8, 8)) == PPGPU_ERR_ARG and "axis 1" in _msg(L)
    assert _ff(L, n=(8, 8, 0)) == PPGPU_ERR_ARG and "axis 2" in _msg(L)
    assert _ff(L, mode=7) == PPGPU_ERR_ARG and "mode 7" in _msg(L)
    assert _ff(L, mode=1, kind=3) == PPGPU_ERR_ARG and "kind 3" in _msg(L)
    assert _ff(L, mode=3) == PPGPU_ERR_ARG and "Qs, QZs" in _msg(L)
    singular = np.array([[1.0, 0, 0], [2.0, 0, 0], [0, 0, 1.0]])
    assert _ff(L, cell=singular) == PPGPU_ERR_ARG and "singular" in _msg(L)


def _scan(L, FE=FAKE, n=(8, 8, 8), nx=4, ny=4, nz=10, nw=0, W=None, df=None, fzs=FAKE, xs=FAKE):
    prm = np.zeros(16)
    return L.ppgpu_relax_scan(FE, _ip(n), _dp(CELL), _dp(prm), nx, ny, nz, xs, FAKE, FAKE, None, fzs, None, None, nw, None if W is None else _dp(W), df, None, None)


def test_relaxation_argument_checks(L):
    assert _scan(L, FE=None) == PPGPU_ERR_ARG and "null argument" in _msg(L)
    assert _scan(L, xs=None) == PPGPU_ERR_ARG and "null argument" in _msg(L)
    assert _scan(L, nx=-1) == PPGPU_ERR_ARG and "negative sizes" in _msg(L)
    # Δf needs 1 <= nw <= min(64, nz), its weights and fzs
    assert _scan(L, df=FAKE, nw=0, W=np.ones(1)) == PPGPU_ERR_ARG and "df needs" in _msg(L)
    assert _scan(L, df=FAKE, nw=11, W=np.ones(11)) == PPGPU_ERR_ARG and "df needs" in _msg(L)
    assert _scan(L, df=FAKE, nw=3, W=None) == PPGPU_ERR_ARG
    assert _scan(L, df=FAKE, nw=3, W=np.ones(3), fzs=None) == PPGPU_ERR_ARG
    # an empty scan is no work
    assert _scan(L, nx=0) == PPGPU_OK and _scan(L, nz=0) == PPGPU_OK


def test_lanes_per_stroke_and_spline_checks(L):
    assert L.ppgpu_set_relax_tps(3) == PPGPU_ERR_ARG and "not in" in _msg(L)
    out = np.zeros(1, np.int32)
    assert L.ppgpu_get_relax_tps(-1, _ip(out)) == PPGPU_ERR_ARG
    assert L.ppgpu_set_relax_tps(0) == PPGPU_OK
    assert L.ppgpu_get_relax_tps(1000, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == PPGPU_OK
    assert L.ppgpu_set_tip_spline(-1, None, None) == PPGPU_ERR_ARG and "negative" in _msg(L)
    assert L.ppgpu_set_tip_spline(1, _dp([1.0]), _dp([0.0, 0.0])) == PPGPU_ERR_ARG and "at least 2" in _msg(L)


def test_pack_atoms_checks(L):
    out = np.zeros(12, np.float32)
    nch = np.zeros(1, np.int32)
    assert L.ppgpu_pack_atoms(-1, None, None, None, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), _ip(nch)) == PPGPU_ERR_ARG
    assert L.ppgpu_pack_atoms(1, None, None, None, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), _ip(nch)) == PPGPU_ERR_ARG
    assert L.ppgpu_pack_atoms(0, None, None, None, None, None) == PPGPU_OK


def test_no_allocation_entry_point_limits(L):
    """The entry point that allocates nothing rejects what its fixed array cannot hold: more
    than 32768 atoms, or a z column longer than its 2^18-point chunk; with no output grid it
    does nothing."""
    n = np.array([8, 8, 8], np.int32)
    assert L.ppgpu_lj_grid_f64_noalloc(FAKE, None, None, _dp(CELL), 1, FAKE, FAKE, None) == PPGPU_ERR_ARG
    assert L.ppgpu_lj_grid_f64_noalloc(FAKE, None, _ip(n), _dp(CELL), 32769, FAKE, FAKE, None) == PPGPU_ERR_ARG
    assert "32768" in _msg(L)
    assert L.ppgpu_lj_grid_f64_noalloc(FAKE, None, _ip(n), _dp(CELL), 4, None, None, None) == PPGPU_ERR_ARG
    assert "null atom arrays" in _msg(L)
    assert L.ppgpu_lj_grid_f64_noalloc(FAKE, None, _ip([4, 4, (1 << 18) + 1]), _dp(CELL), 4, FAKE, FAKE, None) == PPGPU_ERR_ARG
    assert "chunk" in _msg(L)
    assert L.ppgpu_lj_grid_f64_noalloc(None, None, _ip(n), _dp(CELL), 4, FAKE, FAKE, None) == PPGPU_OK
    assert L.ppgpu_last_status() == PPGPU_OK


DROPIN_SCRIPT = r"""
import ctypes, numpy as np, sys
sys.path.insert(0, sys.argv[1])
from ppafm_gb300 import _lib, core
L = _lib.load()
ip = lambda a: np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(ctypes.POINTER(ctypes.c_int))
dp = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
rT = np.zeros((2, 2, 3, 3)); rs = np.zeros_like(rT); fs = np.zeros_like(rT)
out = []
# before setGridN / setGridCell: the relaxation and the force fields report a state error
L.relaxTipStrokes_omp(2, 2, 1, 1, 3, dp(rT), dp(rs), dp(fs), None)
out.append((L.ppgpu_last_status(), L.ppgpu_last_error().decode()))
L.getLennardJonesFF(1, dp(np.zeros(3)), dp(np.ones(2)))
out.append((L.ppgpu_last_status(), L.ppgpu_last_error().decode()))
core.setGridN([8, 8, 8]); core.setGridCell(np.eye(3) * 8.0)
# grid set, no force-field pointer: the relaxation still refuses; a force field with nothing to
# store does nothing (the reference computes and stores nothing either)
L.relaxTipStrokes_omp(2, 2, 1, 1, 3, dp(rT), dp(rs), dp(fs), None)
out.append((L.ppgpu_last_status(), L.ppgpu_last_error().decode()))
L.getLennardJonesFF(1, dp(np.zeros(3)), dp(np.ones(2)))
out.append((L.ppgpu_last_status(), ""))
# the Python wrappers turn the status into an exception
try:
    core.relaxTipStrokes_omp(rT, rs, fs)
    out.append("no exception")
except _lib.PPGPUError as e:
    out.append("raised: " + str(e))
print(repr(out))
"""


def test_dropin_state_errors():
    """The drop-in symbols are void like the reference's; called before the state they need
    (grid shape and cell, the borrowed force-field pointer) they do nothing and report
    PPGPU_ERR_STATE (3) through ppgpu_last_status, which the Python wrappers raise.  Run in a
    fresh process: the drop-in state is process-global."""
    import ast
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", DROPIN_SCRIPT, root], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = ast.literal_eval(r.stdout.strip().splitlines()[-1])
    assert out[0][0] == 3 and "setGridN/setGridCell" in out[0][1]
    assert out[1][0] == 3 and "setGridN/setGridCell" in out[1][1]
    assert out[2][0] == 3 and "setFF_Fpointer" in out[2][1]
    assert out[3][0] == PPGPU_OK
    assert out[4].startswith("raised:") and "setFF_Fpointer" in out[4]
