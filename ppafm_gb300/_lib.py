"""ctypes loader for libppgpu.so (the library's C ABI is declared in include/ppgpu.h).

Mirrors the reference's loader (ppafm/cpp_utils.py:36-57): the shared library is found
next to the package, built on demand when PPAFM_GB300_REBUILD=1, and bound once.  There is
no fallback: if the library cannot be loaded, importing the device entry points raises.
"""

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_longlong, c_ulonglong, c_void_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libppgpu.so")

PPGPU_OK = 0
PPGPU_ERR_ARG = 1
PPGPU_ERR_CUDA = 2
PPGPU_ERR_STATE = 3
PPGPU_ERR_DEVICE_TIMEOUT = 4
PPGPU_ERR_NO_DEVICE = 5

FF_LJ, FF_COULOMB, FF_LJC, FF_QZS = 0, 1, 2, 3
FF_WITH_E, FF_ACCUMULATE, FF_F64 = 1, 2, 4
FFT_F64 = 1
ATOM_FLOATS = 12
RELAX_NPARAM = 15
AFM_NPARAM = 28

# Every exported symbol of include/ppgpu.h with (argtypes, restype).
_dp = POINTER(c_double)
_ip = POINTER(c_int)
SIGNATURES = {
    # drop-in symbols (ProbeParticle.cpp:319-701)
    "setGridN": ([_ip], None),
    "setGridCell": ([_dp], None),
    "setFF_Fpointer": ([_dp], None),
    "setFF_Epointer": ([_dp], None),
    "deleteFF_Fpointer": ([], None),
    "deleteFF_Epointer": ([], None),
    "setRelax": ([c_int, c_double, c_double, c_double], None),
    "setFIRE": ([c_double, c_double, c_double], None),
    "setTip": ([c_double, c_double, _dp, _dp], None),
    "getLennardJonesFF": ([c_int, _dp, _dp], None),
    "getCoulombFF": ([c_int, _dp, _dp, c_int], None),
    "relaxTipStroke": ([c_int, c_int, c_int, _dp, _dp, _dp, c_void_p], c_int),
    "relaxTipStrokes_omp": ([c_int, c_int, c_int, c_int, c_int, _dp, _dp, _dp, c_void_p], c_int),
    "ppgpu_last_iterations": ([], c_longlong),
    # status
    "ppgpu_last_error": ([], c_char_p),
    "ppgpu_last_status": ([], c_int),
    "ppgpu_device_status": ([c_void_p], c_int),
    "ppgpu_device_info": ([c_char_p, c_int], c_int),
    # device API
    "ppgpu_pack_atoms": ([c_int, _dp, _dp, _dp, POINTER(c_float), _ip], c_int),
    "ppgpu_ff_grid": ([c_void_p, _ip, _dp, c_void_p, c_int, c_int, c_int, c_int, c_double, c_double, _dp, _dp, c_int, c_void_p], c_int),
    "ppgpu_ff_subgrid": ([c_void_p, _ip, _dp, _ip, _ip, c_void_p, c_int, c_int, c_int, c_int, c_double, c_double, _dp, _dp, c_int, c_void_p], c_int),
    "ppgpu_relax_strokes": ([c_void_p, _ip, _dp, _dp, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p], c_int),
    "ppgpu_relax_scan": ([c_void_p, _ip, _dp, _dp, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, _dp, c_void_p, c_void_p, c_void_p, c_int, _dp, c_void_p, c_void_p, c_void_p], c_int),
    "ppgpu_set_tip_spline": ([c_int, _dp, _dp], c_int),
    "ppgpu_set_relax_tps": ([c_int], c_int),
    "ppgpu_get_relax_tps": ([c_longlong, _ip], c_int),
    "ppgpu_relax_afm": ([c_void_p, _ip, _dp, _dp, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_int, _dp, c_void_p, c_void_p, c_void_p], c_int),
    "ppgpu_fz2df": ([c_void_p, c_longlong, c_int, c_int, _dp, c_double, c_void_p, c_void_p], c_int),
    "ppgpu_clamp_grid": ([c_void_p, c_longlong, c_double, c_void_p], c_int),
    "ppgpu_interp_grid": ([c_void_p, _ip, _dp, _dp, c_void_p, _ip, _dp, _dp, _dp, _dp, c_void_p], c_int),
    "ppgpu_grad_fd": ([c_void_p, _ip, _dp, _dp, c_void_p, c_int, c_void_p], c_int),
    "ppgpu_grad_potential_grid": ([c_void_p, _ip, _dp, _dp, c_void_p, _ip, _dp, _dp, _dp, c_void_p], c_int),
    "ppgpu_tip_charges_field": ([c_void_p, _ip, _dp, _dp, _dp, _dp, c_void_p, c_int, c_void_p], c_int),
    "ppgpu_interp_tip_grid": ([c_void_p, _ip, _dp, _dp, c_void_p, _ip, _dp, c_void_p], c_int),
    "ppgpu_scalar_clamp": ([c_void_p, c_void_p, c_longlong, c_double, c_double, c_int, c_double, c_void_p], c_int),
    "ppgpu_scalar_add_mult": ([c_void_p, c_void_p, c_void_p, c_longlong, c_double, c_void_p], c_int),
    "ppgpu_scalar_sums": ([c_void_p, c_longlong, c_void_p, c_void_p], c_int),
    "ppgpu_scalar_power": ([c_void_p, c_void_p, c_longlong, c_double, c_double, c_void_p], c_int),
    "ppgpu_axpby_grid": ([c_void_p, c_void_p, c_double, c_void_p, c_double, c_longlong, c_void_p], c_int),
    "ppgpu_grid_from_f64": ([c_void_p, c_void_p, c_void_p, c_longlong, c_void_p], c_int),
    "ppgpu_grid_to_f64": ([c_void_p, c_void_p, c_void_p, c_longlong, c_int, c_void_p], c_int),
    "ppgpu_ffma_peak": ([c_void_p, c_int, POINTER(c_longlong), c_void_p], c_int),
    "ppgpu_fft_create": ([_ip, c_int, POINTER(c_void_p)], c_int),
    "ppgpu_fft_destroy": ([c_void_p], c_int),
    "ppgpu_fft_potential2forces": ([c_void_p, c_void_p, c_void_p, _dp, c_double, c_int, c_void_p, c_void_p], c_int),
    "ppgpu_fft_probe_density": ([c_void_p, c_void_p, _dp, c_double, _dp, c_void_p], c_int),
    "ppgpu_fft_density_power": ([c_void_p, c_void_p, c_double, c_int, c_void_p], c_int),
    "ppgpu_fft_poisson": ([c_void_p, c_void_p, _dp, c_void_p, c_void_p], c_int),
    "ppgpu_fft_correlate": ([c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p], c_int),
    "ppgpu_gaussian_density": ([c_void_p, _ip, _dp, c_int, c_void_p, c_int, c_void_p], c_int),
    "ppgpu_lj_grid_f64_noalloc": ([c_void_p, c_void_p, _ip, _dp, c_int, c_void_p, c_void_p, c_void_p], c_int),
    "ppgpu_batch_create": ([c_void_p, c_int, _dp, c_double, c_double, c_int, _dp, _ip, POINTER(c_void_p)], c_int),
    "ppgpu_batch_run": ([c_void_p, c_void_p], c_int),
    "ppgpu_batch_info": ([c_void_p, POINTER(c_longlong)], c_int),
    "ppgpu_batch_iterations": ([c_void_p, POINTER(c_ulonglong), c_void_p], c_int),
    "ppgpu_batch_destroy": ([c_void_p], c_int),
    "ppgpu_batch_set_wait": ([c_void_p, c_double, c_int], c_int),
    "ppgpu_set_ff_block": ([c_int], c_int),
    "ppgpu_batch_run_layered": ([c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p], c_int),
    "ppgpu_batch_layer_info": ([c_void_p, POINTER(c_longlong)], c_int),
    "ppgpu_tc_selftest": ([c_void_p, c_void_p, c_int, c_int, c_void_p, c_void_p], c_int),
    "ppgpu_mlp_create": ([c_ulonglong, POINTER(c_void_p)], c_int),
    "ppgpu_mlp_destroy": ([c_void_p], c_int),
    "ppgpu_mlp_nparams": ([], c_int),
    "ppgpu_mlp_get": ([c_void_p, c_int, POINTER(c_float)], c_int),
    "ppgpu_mlp_set": ([c_void_p, POINTER(c_float)], c_int),
    "ppgpu_mlp_forward": ([c_void_p, c_void_p, c_int, c_void_p, c_void_p], c_int),
    "ppgpu_mlp_backward": ([c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p], c_int),
    "ppgpu_mlp_adam": ([c_void_p, c_double, c_int, c_void_p], c_int),
    "ppgpu_mlp_take_loss": ([c_void_p, POINTER(c_double), c_void_p], c_int),
    "ppgpu_mlp_views": ([c_void_p, POINTER(c_void_p)], c_int),
    "ppgpu_mlp_set_loss_weights": ([c_void_p, _dp], c_int),
}


class BatchJob(ctypes.Structure):
    """ppgpu_batch_job of include/ppgpu.h."""

    _fields_ = [
        ("FE", c_void_p),
        ("atoms", c_void_p),
        ("natoms", c_int),
        ("ncharged", c_int),
        ("n", c_int * 3),
        ("cell", c_double * 9),
        ("nx", c_int),
        ("ny", c_int),
        ("nz", c_int),
        ("xs", _dp),
        ("ys", _dp),
        ("zs", _dp),
        ("pos_offset", c_double * 3),
        ("fzs", c_void_p),
        ("ppos", c_void_p),
        ("df", c_void_p),
        ("iters", c_void_p),
    ]

_lib = None


class PPGPUError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"libppgpu error {status}: {msg}")
        self.status = status


def load(path=None):
    """Loads and binds libppgpu.so; raises if it is missing or incomplete."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIB_PATH
    if os.environ.get("PPAFM_GB300_REBUILD") == "1" or not os.path.exists(path):
        from . import build as _build

        _build.build(force=os.environ.get("PPAFM_GB300_REBUILD") == "1")
    L = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(L, name)  # AttributeError if the library lacks a declared symbol
        fn.argtypes = args
        fn.restype = res
    if path == LIB_PATH:
        _lib = L
    return L


def lib():
    return load()


def last_error():
    return lib().ppgpu_last_error().decode()


def check(status):
    """Raises PPGPUError for a non-zero status of a ppgpu_* call."""
    if status != PPGPU_OK:
        raise PPGPUError(status, last_error())


def check_state():
    """Raises if the last drop-in (void) call recorded an error."""
    st = lib().ppgpu_last_status()
    if st != PPGPU_OK:
        raise PPGPUError(st, last_error())


def dptr(a):
    """double* of a contiguous float64 numpy array (or None)."""
    return None if a is None else a.ctypes.data_as(_dp)


def iptr(a):
    return None if a is None else a.ctypes.data_as(_ip)


def tptr(t):
    """Device address of a torch tensor (or None)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
