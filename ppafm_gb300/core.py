"""Drop-in replacement of ppafm/core.py over libppgpu.so.

Same function names, arguments and array conventions as the reference's ctypes layer
(ppafm/core.py:33-324): float64 C-contiguous numpy arrays, process-global grid/tip/
relaxation state, force fields accumulated into the array registered with
``setFF_Fpointer``.  The work runs on the GPU; arrays stay host numpy arrays.

Differences from the reference, all deliberate:
  * ``setRelax`` takes ``convF2`` as documented (the reference wrapper references an
    undefined name, ppafm/core.py:97-98);
  * a failed call raises ``PPGPUError`` instead of printing or exiting.
"""

import ctypes
import weakref

import numpy as np

from . import common as PPU
from ._lib import PPGPUError, check_state, dptr, iptr, lib

__all__ = [
    "setGridN",
    "setGridCell",
    "setFF_Fpointer",
    "setFF_Epointer",
    "deleteFF_Fpointer",
    "deleteFF_Epointer",
    "setRelax",
    "setFIRE",
    "setTip",
    "getLennardJonesFF",
    "getCoulombFF",
    "relaxTipStroke",
    "relaxTipStrokes_omp",
    "SplineParameters",
    "last_iterations",
    "PPGPUError",
]


def _f64(a, ndim, name):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or a.ndim != ndim or not a.flags["C_CONTIGUOUS"]:
        raise TypeError(f"{name}: expected a C-contiguous float64 array with {ndim} dimensions")
    return a


def setGridN(n):
    """core.py:38 -> ProbeParticle.cpp:358."""
    n = np.array(n, dtype=np.int32).copy()
    lib().setGridN(iptr(n))
    check_state()


def setGridCell(cell):
    """core.py:48 -> ProbeParticle.cpp:365 (last three rows of a 3x3 or 4x3 lvec)."""
    cell = np.array(np.asarray(cell)[-3:, 0:3], copy=True, dtype=np.float64)
    lib().setGridCell(dptr(cell))
    check_state()


def setFF_Fpointer(gridF):
    """core.py:59-61: borrows gridF [nx,ny,nz,3]; the pointer is dropped when gridF dies."""
    _f64(gridF, 4, "setFF_Fpointer")
    lib().setFF_Fpointer(dptr(gridF))
    weakref.finalize(gridF, deleteFF_Fpointer)


def setFF_Epointer(gridE):
    """core.py:69-71."""
    _f64(gridE, 3, "setFF_Epointer")
    lib().setFF_Epointer(dptr(gridE))
    weakref.finalize(gridE, deleteFF_Epointer)


def deleteFF_Fpointer():
    lib().deleteFF_Fpointer()


def deleteFF_Epointer():
    lib().deleteFF_Epointer()


def setRelax(maxIters=1000, convF2=1.0e-8, dt=0.1, damping=0.1):
    """ProbeParticle.cpp:322 (also sets FIRE's dtmax = dt and acoef0 = damping)."""
    lib().setRelax(int(maxIters), float(convF2), float(dt), float(damping))
    check_state()


def setFIRE(finc=1.1, fdec=0.5, falpha=0.99):
    lib().setFIRE(float(finc), float(fdec), float(falpha))
    check_state()


def setTip(lRadial=None, kRadial=None, rPP0=None, kSpring=None, parameters=None):
    """core.py:115-129: stiffness in eV/A^2 (negative), defaults from ``parameters``
    (r0Probe, krad, klat)."""
    if lRadial is None:
        lRadial = parameters.r0Probe[2]
    if kRadial is None:
        kRadial = parameters.krad / -PPU.eVA_Nm
    if rPP0 is None:
        rPP0 = np.array((parameters.r0Probe[0], parameters.r0Probe[1], 0.0))
    if kSpring is None:
        kSpring = np.array((parameters.klat, parameters.klat, 0.0)) / -PPU.eVA_Nm
    rPP0 = np.ascontiguousarray(rPP0, dtype=np.float64)
    kSpring = np.ascontiguousarray(kSpring, dtype=np.float64)
    lib().setTip(float(lRadial), float(kRadial), dptr(rPP0), dptr(kSpring))
    check_state()


def getLennardJonesFF(Rs, cLJs):
    """core.py:193-195: gridF (+ gridE) += LJ force field of atoms Rs [n,3] with (c6,c12)."""
    _f64(Rs, 2, "Rs")
    _f64(cLJs, 2, "cLJs")
    lib().getLennardJonesFF(len(Rs), dptr(Rs), dptr(cLJs))
    check_state()


def getCoulombFF(Rs, kQQs, kind=0):
    """core.py:270-272: kQQs = Q * CoulombConst per atom; kind 0/1/2 = s/pz/dz2 tip."""
    _f64(Rs, 2, "Rs")
    _f64(kQQs, 1, "kQQs")
    lib().getCoulombFF(len(Rs), dptr(Rs), dptr(kQQs), int(kind))
    check_state()


class SplineParameters(ctypes.Structure):
    """Radial tip spline (core.py:132-155, TIP::SplineParams): knots xs and per knot the radial
    force and its slope, ydys [n, 2]."""

    _fields_ = [("rff_n", ctypes.c_int), ("rff_xs", ctypes.POINTER(ctypes.c_double)), ("rff_ydys", ctypes.POINTER(ctypes.c_double))]

    def __init__(self, xs, ydys):
        super().__init__()
        self.np_rff_xs = np.ascontiguousarray(xs, dtype=np.double)
        self.np_rff_ydys = np.ascontiguousarray(ydys, dtype=np.double)
        self.rff_n = len(self.np_rff_xs)
        self.rff_xs = np.ctypeslib.as_ctypes(self.np_rff_xs)
        self.rff_ydys = np.ctypeslib.as_ctypes(self.np_rff_ydys.reshape(-1))

    @classmethod
    def from_file(cls, file_path):
        d = np.genfromtxt(file_path)
        return cls(d[:, 0], d[:, 1:])


def _spline_ptr(tip_spline):
    if tip_spline is None:
        return None
    if not isinstance(tip_spline, ctypes.Structure):
        raise TypeError("tip_spline must be a SplineParameters structure (or None)")
    return ctypes.cast(ctypes.pointer(tip_spline), ctypes.c_void_p)


def relaxTipStroke(rTips, rs, fs, probeStart=1, relaxAlg=1, tip_spline=None):
    """core.py:312-314: one stroke [nstep,3]; returns the iteration sum.  tip_spline: a
    SplineParameters (ctypes structure of the same layout) replacing the radial spring."""
    for a, nm in ((rTips, "rTips"), (rs, "rs"), (fs, "fs")):
        _f64(a, 2, nm)
    r = lib().relaxTipStroke(int(probeStart), int(relaxAlg), len(rTips), dptr(rTips), dptr(rs), dptr(fs), _spline_ptr(tip_spline))
    check_state()
    return r


def relaxTipStrokes_omp(rTips, rs, fs, probeStart=1, relaxAlg=1, tip_spline=None):
    """core.py:322-324: all strokes of rTips [nx,ny,nz,3]; returns 0 like the reference."""
    for a, nm in ((rTips, "rTips"), (rs, "rs"), (fs, "fs")):
        _f64(a, 4, nm)
    nx, ny, nz, _ = rTips.shape
    r = lib().relaxTipStrokes_omp(nx, ny, int(probeStart), int(relaxAlg), nz, dptr(rTips), dptr(rs), dptr(fs), _spline_ptr(tip_spline))
    check_state()
    return r


def last_iterations():
    """Total FIRE iterations of the last relaxTipStroke(s) call."""
    return lib().ppgpu_last_iterations()
