"""CPU oracle for the probe-particle AFM hot path -- TEST INFRASTRUCTURE ONLY.

This module is the checker of the CUDA library in ``ppafm_gb300``.  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may import it; the
product path never does.

It has two halves:

* ctypes bindings to ``oracle/libpporacle.so`` (``pp_oracle.c``), the FP64 C restatement
  of the reference C++ core and the FP32 restatement of its OpenCL kernels;
* numpy restatements of the reference's Python-side arithmetic: the Fz->df weights and
  convolution (``ppafm/common.py:333-430``), periodic-image replication
  (``common.py:608-628, 728-776``), Lennard-Jones mixing (``common.py:851-892``), scan
  grids (``common.py:922-946``), the force clamp (``ppafm/io.py:766-778``), the FFT
  density-overlap route (``ppafm/fieldFFT.py:32-319``) and the AFMulator point-charge
  pipeline (``ppafm/ocl/AFMulator.py:211-479``, ``ppafm/ocl/relax.py:43-87``).

Pinning: the FP64 C functions are compared bit-for-bit with the reference library compiled
from its own sources (``oracle/_ref``, built by ``oracle/Makefile`` where the reference
checkout exists), and the numpy functions against golden vectors produced by the reference
package itself (``tests/golden``).  The AFMulator (OpenCL) restatement cannot be run against
the reference here (no OpenCL runtime); its parity is unpinned except where it shares
arithmetic with the pinned CPU functions.
"""

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_longlong

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpporacle.so")
REF_PATH = os.path.join(HERE, "_ref", "ProbeParticle_lib.so")

# ppafm/common.py:20-21
eVA_Nm = 16.0217662
CoulombConst = 14.399645

_lib = None


def build():
    """Compile the C restatement (``make -C oracle``)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = POINTER(c_double)
        fp = POINTER(c_float)
        ip = POINTER(c_int)
        L.oc_ff_subgrid.argtypes = [ip, dp, ip, ip, c_int, dp, dp, c_int, dp, dp, c_int]
        L.oc_lj_grid.argtypes = [ip, dp, c_int, dp, dp, dp, dp, c_int]
        L.oc_coulomb_grid.argtypes = [ip, dp, c_int, dp, dp, c_int, dp, dp, c_int]
        L.oc_relax_strokes.argtypes = [ip, dp, dp, dp, c_int, c_int, c_int, c_int, dp, dp, dp, ip, ip, c_int, c_int, dp, dp]
        L.oc_fz2df.argtypes = [c_longlong, c_int, dp, c_int, dp, c_double, dp, c_int]
        L.oc_afm_ff_qzs.argtypes = [ip, fp, fp, fp, fp, c_int, fp, fp, fp, fp, fp, c_int]
        L.oc_afm_relax_tilted.argtypes = [fp, ip, fp, c_int, fp, c_int, fp, fp, fp, fp, fp, fp, fp, ip, c_int]
        L.oc_afm_convolve_z.argtypes = [c_int, c_int, c_int, fp, fp, fp, c_int]
        L.oc_grid_setup.argtypes = [ip, dp, dp, dp]
        L.oc_num_threads.restype = c_int
        _lib = L
    return _lib


def _p(a, ctype):
    return a.ctypes.data_as(POINTER(ctype))


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _c32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def num_threads():
    return lib().oc_num_threads()


# ----------------------------------------------------------------- FP64 grid sampling


def grid_setup(n, cell):
    """(dCell, diCell) of GridShape::setCell (Grid.h:29-36)."""
    n = _i32(n)
    cell = _c64(cell).reshape(3, 3)
    d = np.zeros(9)
    di = np.zeros(9)
    lib().oc_grid_setup(_p(n, c_int), _p(cell, c_double), _p(d, c_double), _p(di, c_double))
    return d.reshape(3, 3), di.reshape(3, 3)


def lj_grid(n, cell, Rs, cLJs, gridF=None, gridE=None, nthreads=0):
    """getLennardJonesFF (ProbeParticle.cpp:508-513): returns gridF += F, gridE += E."""
    n = _i32(n)
    cell = _c64(cell).reshape(3, 3)
    Rs = _c64(Rs)
    cLJs = _c64(cLJs)
    if gridF is None:
        gridF = np.zeros(tuple(n) + (3,))
    ep = _p(gridE, c_double) if gridE is not None else None
    lib().oc_lj_grid(_p(n, c_int), _p(cell, c_double), len(Rs), _p(Rs, c_double), _p(cLJs, c_double), _p(gridF, c_double), ep, nthreads)
    return gridF, gridE


def coulomb_grid(n, cell, Rs, kQQs, kind=0, gridF=None, gridE=None, nthreads=0):
    """getCoulombFF (ProbeParticle.cpp:540-554)."""
    n = _i32(n)
    cell = _c64(cell).reshape(3, 3)
    Rs = _c64(Rs)
    kQQs = _c64(kQQs)
    if gridF is None:
        gridF = np.zeros(tuple(n) + (3,))
    ep = _p(gridE, c_double) if gridE is not None else None
    lib().oc_coulomb_grid(_p(n, c_int), _p(cell, c_double), len(Rs), _p(Rs, c_double), _p(kQQs, c_double), kind, _p(gridF, c_double), ep, nthreads)
    return gridF, gridE


def ff_subgrid(n, cell, i0, ns, Rs, coefs, kind, nthreads=0, with_E=False):
    """A sub-box [i0, i0+ns) of the LJ (kind=-1) or Coulomb (kind 0/1/2) grid."""
    n = _i32(n)
    i0 = _i32(i0)
    ns = _i32(ns)
    cell = _c64(cell).reshape(3, 3)
    Rs = _c64(Rs)
    coefs = _c64(coefs)
    gridF = np.zeros(tuple(ns) + (3,))
    gridE = np.zeros(tuple(ns)) if with_E else None
    ep = _p(gridE, c_double) if gridE is not None else None
    lib().oc_ff_subgrid(_p(n, c_int), _p(cell, c_double), _p(i0, c_int), _p(ns, c_int), len(Rs), _p(Rs, c_double), _p(coefs, c_double), kind, _p(gridF, c_double), ep, nthreads)
    return gridF, gridE


# ------------------------------------------------------------------- FP64 relaxation


def tip_params(lRadial, kRadial, rPP0, kSpring):
    """TIP::makeConsistent (ProbeParticle.cpp:64-69) applied to setTip's arguments."""
    rPP0 = np.array(rPP0, dtype=np.float64).copy()
    if abs(kRadial) > 1e-8:
        rPP0[2] = -np.sqrt(lRadial * lRadial - rPP0[0] * rPP0[0] - rPP0[1] * rPP0[1])
    return dict(lRadial=float(lRadial), kRadial=float(kRadial), rPP0=rPP0, kSpring=np.array(kSpring, dtype=np.float64))


def relax_param_vector(tip, maxIters=1000, convF2=1e-8, dt=0.1, damping=0.1, finc=1.1, fdec=0.5, falpha=0.99):
    v = np.zeros(15)
    v[0:7] = [maxIters, convF2, dt, damping, finc, fdec, falpha]
    v[7] = tip["lRadial"]
    v[8] = tip["kRadial"]
    v[9:12] = tip["rPP0"]
    v[12:15] = tip["kSpring"]
    return v


def relax_strokes(n, cell, gridF, params, rTips, probeStart=1, relaxAlg=1, nthreads=0, spline=None):
    """relaxTipStrokes_omp (ProbeParticle.cpp:682-701) over strokes laid out as
    rTips[..., nstep, 3] (every leading index is one stroke).  spline = (xs [n], ydys [n, 2])
    replaces the radial spring by forceRSpline.  Returns (rs, fs, itrsum per stroke,
    iterations per step)."""
    n = _i32(n)
    cell = _c64(cell).reshape(3, 3)
    gridF = _c64(gridF)
    params = _c64(params)
    rTips = _c64(rTips)
    shp = rTips.shape
    nstep = shp[-2]
    nstroke = int(np.prod(shp[:-2]))
    rs = np.zeros(shp)
    fs = np.zeros(shp)
    sums = np.zeros(nstroke, dtype=np.int32)
    iters = np.zeros(shp[:-1], dtype=np.int32)
    sx = sy = None
    ns = 0
    if spline is not None:
        sx = _c64(spline[0])
        sy = _c64(spline[1]).reshape(-1)
        ns = len(sx)
    lib().oc_relax_strokes(_p(n, c_int), _p(cell, c_double), _p(gridF, c_double), _p(params, c_double), probeStart, relaxAlg, nstroke, nstep, _p(rTips, c_double), _p(rs, c_double), _p(fs, c_double), _p(sums, c_int), _p(iters, c_int), nthreads, ns, None if sx is None else _p(sx, c_double), None if sy is None else _p(sy, c_double))
    return rs, fs, sums, iters


# ------------------------------------------------------------------- Fz -> df (numpy)


def get_df_weight(Amp, dz=0.1):
    """Discretised Giessibl kernel (common.py:333-392)."""
    n = int(np.ceil(Amp / dz))
    w = np.zeros(n + 1)
    f = np.zeros(n + 1)
    f2 = np.zeros(n + 1)
    t = np.linspace(-1 + 2 * n * dz / Amp, -1, n + 1)
    if n > 1:
        f[1:-1] = np.sqrt(1 - t[1:-1] * t[1:-1])
        f2[1:-1] = (np.arccos(-t[1:-1]) - t[1:-1] * f[1:-1]) / 2.0
    f2[0] = np.pi / 2
    df = f[:-1] - f[1:]
    df2 = f2[:-1] - f2[1:]
    w[1:] = t[:-1] * df + df2
    w[:-1] -= t[1:] * df + df2
    return w / (np.pi * dz)


def get_simple_df_weight(n=10, dz=0.1):
    """Simpler kernel used by AFMulator (common.py:395-418)."""
    n = int(n)
    if n < 2:
        n = 2
    t = np.linspace(-1 + 0.5 / n, 1 - 0.5 / n, n - 1)
    f = np.sqrt(1 - t * t)
    w = np.zeros(n)
    w[:-1] = f
    w[1:] -= f
    t = np.linspace(-1, 1, n)
    w0 = np.sum(t * w)
    return w / (w0 * n * dz)


def Fz2df(F, dz, k0, f0, amplitude=1.0, units=16.0217656, nthreads=0):
    """common.py:421-430 -- 'valid' np.convolve along z, scaled by units*f0/k0."""
    W = get_df_weight(amplitude, dz=dz)
    F = _c64(F)
    nz = F.shape[-1]
    nout = nz - len(W) + 1
    out = np.zeros(F.shape[:-1] + (nout,))
    lib().oc_fz2df(int(np.prod(F.shape[:-1])), nz, _p(F, c_double), len(W), _p(_c64(W), c_double), units * f0 / k0, _p(out, c_double), nthreads)
    return out


def Fz2df_numpy(F, dz, k0, f0, amplitude=1.0, units=16.0217656):
    W = get_df_weight(amplitude, dz=dz)
    return np.apply_along_axis(lambda m: np.convolve(m, W, mode="valid"), axis=2, arr=F) * units * f0 / k0


# ------------------------------------------------------------- atoms, LJ, scan grids


def PBCAtoms(Zs, Rs, Qs, avec, bvec, na=1, nb=1):
    """In-plane periodic images, i outer, j inner, atoms innermost (common.py:608-628)."""
    Zs_, Rs_, Qs_ = [], [], []
    for i in range(-na, na + 1):
        for j in range(-nb, nb + 1):
            for ia in range(len(Zs)):
                Zs_.append(Zs[ia])
                Rs_.append((Rs[ia][0] + i * avec[0] + j * bvec[0], Rs[ia][1] + i * avec[1] + j * bvec[1], Rs[ia][2]))
                Qs_.append(Qs[ia])
    return np.array(Zs_), np.array(Rs_, dtype=np.float64), np.array(Qs_, dtype=np.float64)


def PBCAtoms3D_np(Zs, Rs, Qs, cLJs, lvec, npbc=(1, 1, 1)):
    """3-D images with the home cell first, FP32 (common.py:728-776)."""
    lvec = np.asarray(lvec, dtype=np.float64)
    natom = len(Zs)
    mtot = (2 * npbc[0] + 1) * (2 * npbc[1] + 1) * (2 * npbc[2] + 1)
    Zs_ = np.empty(mtot * natom, np.int32)
    xyz = np.empty((mtot * natom, 3), np.float32)
    qs = np.empty(mtot * natom, np.float32)
    cl = np.empty((mtot * natom, 2), np.float32)
    Zs_[:natom], xyz[:natom], qs[:natom], cl[:natom] = Zs, Rs, Qs, cLJs
    i0 = natom
    for ia in range(-npbc[0], npbc[0] + 1):
        for ib in range(-npbc[1], npbc[1] + 1):
            for ic in range(-npbc[2], npbc[2] + 1):
                if ia == 0 and ib == 0 and ic == 0:
                    continue
                s = ia * lvec[0] + ib * lvec[1] + ic * lvec[2]
                Zs_[i0 : i0 + natom] = Zs
                xyz[i0 : i0 + natom] = Rs + s[None, :]
                qs[i0 : i0 + natom] = Qs
                cl[i0 : i0 + natom] = cLJs
                i0 += natom
    return Zs_, xyz, qs, cl


def getAtomsLJ(iZprobe, iZs, FFparams):
    """c6 = 2*eps*R^6, c12 = eps*R^12 with R = r0_i + r0_j, eps = sqrt(e_i e_j) (common.py:851-868).
    FFparams: array [Z-1] -> (rmin, epsilon, alpha)."""
    cLJs = np.zeros((len(iZs), 2))
    for i, z in enumerate(iZs):
        Rij = FFparams[iZprobe - 1][0] + FFparams[z - 1][0]
        Eij = np.sqrt(FFparams[iZprobe - 1][1] * FFparams[z - 1][1])
        cLJs[i, 0] = 2 * Eij * (Rij**6)
        cLJs[i, 1] = Eij * (Rij**12)
    return cLJs


def getAtomsREA(iZprobe, iZs, FFparams, alphaFac=-1.0):
    """common.py:880-892."""
    REAs = np.zeros((len(iZs), 4))
    i = iZprobe - 1
    for ii, z in enumerate(iZs):
        j = z - 1
        REAs[ii, 0] = FFparams[i][0] + FFparams[j][0]
        REAs[ii, 1] = np.sqrt(FFparams[i][1] * FFparams[j][1])
        REAs[ii, 2] = FFparams[j][2] * alphaFac
    return REAs


def REA2LJ(cREAs):
    """common.py:871-877."""
    cLJs = np.zeros((len(cREAs), 2))
    R6 = cREAs[:, 0] ** 6
    cLJs[:, 0] = 2 * cREAs[:, 1] * R6
    cLJs[:, 1] = cREAs[:, 1] * (R6**2)
    return cLJs


def prepareScanGrids(scanMin, scanMax, scanStep, r0Probe):
    """common.py:922-946."""
    xTips = np.arange(scanMin[0], scanMax[0] + 0.5 * scanStep[0], scanStep[0])
    yTips = np.arange(scanMin[1], scanMax[1] + 0.5 * scanStep[1], scanStep[1])
    zTips = np.arange(scanMin[2], scanMax[2] + 0.5 * scanStep[2], scanStep[2])
    lvecScan = np.array(
        [
            [scanMin[0] + r0Probe[0], scanMin[1] + r0Probe[1], scanMin[2] - r0Probe[2]],
            [scanMax[0] - scanMin[0], 0.0, 0.0],
            [0.0, scanMax[1] - scanMin[1], 0.0],
            [0.0, 0.0, scanMax[2] - scanMin[2]],
        ]
    )
    return xTips, yTips, zTips, lvecScan


def limit_vec_field(FF, Fmax=100.0):
    """In-place clamp |F| <= Fmax preserving direction (io.py:766-778)."""
    FR = np.sqrt(FF[..., 0] ** 2 + FF[..., 1] ** 2 + FF[..., 2] ** 2)
    mask = FR > Fmax
    for k in range(3):
        FF[..., k][mask] *= Fmax / FR[mask]
    return FF


def scan_tips(xTips, yTips, zTips, origin):
    """rTips of relaxedScan3D_omp (HighLevel.py:104-117): z descending, origin removed."""
    nx, ny, nz = len(xTips), len(yTips), len(zTips)
    rTips = np.zeros((nx, ny, nz, 3))
    rTips[:, :, :, 0] = (xTips - origin[0])[:, None, None]
    rTips[:, :, :, 1] = (yTips - origin[1])[None, :, None]
    rTips[:, :, :, 2] = (zTips - origin[2])[::-1][None, None, :]
    return rTips


def relaxed_scan(n, cell, gridF, params, xTips, yTips, zTips, origin, nthreads=0, spline=None):
    """relaxedScan3D_omp + the origin handling of perform_relaxation (HighLevel.py:104-124,
    162-172): returns fzs [nx,ny,nz] and PPpos [nx,ny,nz,3], ascending z, and iterations."""
    rTips = scan_tips(xTips, yTips, zTips, origin)
    rs, fs, sums, iters = relax_strokes(n, cell, gridF, params, rTips, nthreads=nthreads, spline=spline)
    rs = rs[:, :, ::-1, :].copy() + np.asarray(origin)[None, None, None, :]
    fzs = fs[:, :, ::-1, 2].copy()
    return fzs, rs, iters[:, :, ::-1].copy()


# ------------------------------------------------------------- FFT route (numpy FP64)


def getMGrid(dims, dd):
    """Rolled frequency-index coordinate grids (fieldFFT.py:32-49)."""
    XYZ = np.mgrid[0 : dims[0], 0 : dims[1], 0 : dims[2]].astype(float)
    out = []
    for ax in range(3):
        sh = dims[ax] // 2
        sh_ = sh + (1.0 if dims[ax] % 2 != 0 else 0.0)
        out.append(dd[ax] * np.roll(XYZ[ax] - sh_, sh, axis=ax))
    return out


def _normalized_basis(lvec):
    s = np.asarray(lvec, dtype=np.float64)[1:4]
    return s / np.linalg.norm(s, axis=1)[:, None]


def grid_dd(lvec, nDim):
    s = np.asarray(lvec, dtype=np.float64)[1:4]
    return tuple(np.linalg.norm(s[k]) / nDim[k] for k in range(3))


def getProbeDensity(lvec, X, Y, Z, dd, sigma=0.7, multipole_dict=None):
    """Normalised Gaussian tip density with optional multipoles, tilt 0 (fieldFFT.py:99-118)."""
    mat = _normalized_basis(lvec).T
    rx = X * mat[0, 0] + Y * mat[0, 1] + Z * mat[0, 2]
    ry = X * mat[1, 0] + Y * mat[1, 1] + Z * mat[1, 2]
    rz = X * mat[2, 0] + Y * mat[2, 1] + Z * mat[2, 2]
    radial = np.exp(-(rx**2 + ry**2 + rz**2) / (2 * sigma**2))
    radial /= np.sum(radial) * np.abs(np.linalg.det(mat)) * dd[0] * dd[1] * dd[2]
    if multipole_dict is None:
        return radial
    rho = np.zeros(radial.shape)
    for kind, coef in multipole_dict.items():
        x, y, z = rx / sigma, ry / sigma, rz / sigma
        harm = {
            "s": 1.0,
            "px": x,
            "py": y,
            "pz": z,
            "dz2": 0.25 * (2 * z**2 - x**2 - y**2),
            "dx2": 0.25 * (2 * x**2 - y**2 - z**2),
            "dy2": 0.25 * (2 * y**2 - x**2 - z**2),
            "dxy": x * y,
            "dxz": x * z,
            "dyz": y * z,
        }.get(kind, 0.0)
        rho += radial * coef * harm
    return rho


def potential2forces_mem(V, lvec, nDim, sigma=0.7, rho=None, multipole=None, doForce=True, doPot=False):
    """E and F of the cross-correlation of V with the tip density (fieldFFT.py:268-319)."""
    dims = nDim
    dd = grid_dd(lvec, dims)
    X, Y, Z = getMGrid(dims, dd)
    if rho is None:
        rho = getProbeDensity(lvec, X, Y, Z, dd, sigma=sigma, multipole_dict=multipole)
    LmatInv = np.linalg.inv(_normalized_basis(lvec))
    detLmatInv = np.abs(np.linalg.det(LmatInv))
    dz = [1 / (dims[k] * dd[k] * dd[k]) for k in range(3)]
    zeta = [LmatInv[a, 0] * dz[0] * X + LmatInv[a, 1] * dz[1] * Y + LmatInv[a, 2] * dz[2] * Z for a in range(3)]
    convFFT = np.fft.fftn(V) * np.conj(np.fft.fftn(rho))
    E = Fx = Fy = Fz = None
    if doPot:
        E = np.real(np.fft.ifftn(convFFT * (dd[0] * dd[1] * dd[2]) / detLmatInv))
    if doForce:
        convFFT = convFFT * (-2 * np.pi * 1j * (dd[0] * dd[1] * dd[2]) / detLmatInv)
        Fx = np.real(np.fft.ifftn(zeta[0] * convFFT))
        Fy = np.real(np.fft.ifftn(zeta[1] * convFFT))
        Fz = np.real(np.fft.ifftn(zeta[2] * convFFT))
    return Fx, Fy, Fz, E


def handle_negative_density(rho):
    """cli/conv_rho.py:18-22."""
    q = rho.sum()
    rho[rho < 0] = 0
    rho *= q / rho.sum()
    return rho


def poisson_hartree(rho_charge, lvec):
    """Hartree potential V (eV per unit charge) of a periodic charge density (e/A^3) on a
    general cell: V_k = 4*pi*k_e*rho_k/|G|^2 with G = sum_j m_j b_j (b_j the reciprocal
    basis, 2*pi included, m_j numpy's FFT frequency indices), zero mean.
    No reference counterpart (ppafm has no Poisson solver); pinned by a Gaussian-charge
    known answer instead."""
    n = rho_charge.shape
    cell = np.asarray(lvec, dtype=np.float64)[1:4]
    B = 2 * np.pi * np.linalg.inv(cell).T  # rows b_j, a_i . b_j = 2 pi delta_ij
    m = [np.fft.fftfreq(n[k], d=1.0 / n[k]) for k in range(3)]
    M0, M1, M2 = np.meshgrid(m[0], m[1], m[2], indexing="ij")
    G = M0[..., None] * B[0] + M1[..., None] * B[1] + M2[..., None] * B[2]
    G2 = np.sum(G * G, axis=-1)
    rk = np.fft.fftn(rho_charge)
    with np.errstate(divide="ignore", invalid="ignore"):
        Vk = 4 * np.pi * CoulombConst * rk / G2
    Vk[0, 0, 0] = 0
    return np.real(np.fft.ifftn(Vk))


def gaussian_density(n, lvec, atoms):
    """Sum of normalised 3-D Gaussians on the periodic grid (minimum-image distance):
    rho(p) = sum_i w_i exp(-|p - R_i|^2 / (2 s_i^2)) / ((2 pi)^1.5 s_i^3), grid point
    p = (i/n0) a + (j/n1) b + (k/n2) c; atoms rows (x, y, z relative to the origin, s, w).
    Terms with |p - R_i|^2 / (2 s_i^2) >= 40 (below 5e-18 of the peak) are left out, so each
    atom touches only the grid box around it.  Synthetic-input generator of the
    density-overlap workload (no reference counterpart: the reference reads densities from
    files)."""
    n = tuple(int(x) for x in n)
    cell = np.asarray(lvec, dtype=np.float64)[1:4]
    inv = np.linalg.inv(cell)
    colnorm = np.linalg.norm(inv, axis=0)  # |fractional step| per unit distance along each axis
    rho = np.zeros(n)
    for x, y, z, s, w in np.asarray(atoms, dtype=np.float64):
        fa = np.array([x, y, z]) @ inv
        rc = np.sqrt(80.0) * s
        idx = []
        for k in range(3):
            h = rc * colnorm[k] * n[k]
            if 2 * h + 3 >= n[k]:
                idx.append(np.arange(n[k]))
            else:
                c = fa[k] * n[k]
                idx.append(np.arange(int(np.floor(c - h)) - 1, int(np.ceil(c + h)) + 2) % n[k])
        F = np.stack(np.meshgrid(*[idx[k] / n[k] for k in range(3)], indexing="ij"), axis=-1)
        g = F - fa
        g -= np.rint(g)
        d = g @ cell
        t = np.sum(d * d, axis=-1) / (2 * s * s)
        val = np.where(t < 40.0, w * np.exp(-t) / ((2 * np.pi) ** 1.5 * s**3), 0.0)
        np.add.at(rho, np.ix_(idx[0], idx[1], idx[2]), val)
    return rho


# -------------------------------------------------- AFMulator point-charge (OpenCL, FP32)

VALID_SIZES = np.array([16, 32, 64, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048])


def get_lvec(scan_window, pad=(3.0, 3.0, 5.0), tipR0=(0.0, 0.0, 3.0), pixPerAngstrome=10):
    """AFMulator.py:702-719."""
    pad = np.array(pad)
    tipR0 = np.array(tipR0)
    center = (np.array(scan_window[0]) + np.array(scan_window[1])) / 2
    box = (np.array(scan_window[1]) - np.array(scan_window[0])) + 2 * pad
    nDim = (pixPerAngstrome * box).round().astype(np.int32)
    nDim = np.array([VALID_SIZES[VALID_SIZES >= d][0] for d in nDim])
    box = nDim / pixPerAngstrome
    origin = center - box / 2 - tipR0
    return np.array([origin, [box[0], 0, 0], [0, box[1], 0], [0, 0, box[2]]])


def genFFSampling(lvec, pixPerAngstrome=10):
    """common.py:967-977."""
    return np.array([int(round(pixPerAngstrome * np.sqrt(np.dot(lvec[k], lvec[k])))) for k in (1, 2, 3)], np.int32)


def afm_ff_qzs(nDim, lvec, xyzs, qs, cLJs, Qs, QZs, nthreads=0):
    """evalLJC_QZs_noPos over the AFMulator grid; FE [nz,ny,nx,4] x-fastest."""
    nDim = _i32(nDim)
    lvec = np.asarray(lvec, dtype=np.float64)
    p0 = _c32(lvec[0])
    dl = [_c32(lvec[1 + k] / nDim[k]) for k in range(3)]
    atoms = _c32(np.concatenate([xyzs, np.asarray(qs).reshape(-1, 1)], axis=1))
    cl = _c32(cLJs)
    FE = np.zeros((nDim[2], nDim[1], nDim[0], 4), np.float32)
    lib().oc_afm_ff_qzs(_p(nDim, c_int), _p(p0, c_float), _p(dl[0], c_float), _p(dl[1], c_float), _p(dl[2], c_float), len(atoms), _p(atoms, c_float), _p(cl, c_float), _p(_c32(Qs), c_float), _p(_c32(QZs), c_float), _p(FE, c_float), nthreads)
    return FE


def interp_at(arr, lvec_in, nout, origin_out, step_out, rot=np.eye(3), rot_center=np.zeros(3)):
    """Periodic trilinear interpolation of a grid onto rotated grid points (interp_at +
    linearInterpB, ppafm/ocl/cl/FF.cl:34-72, 1010-1046), in float32 like the kernel; output
    [nout0, nout1, nout2], C order."""
    arr = np.asarray(arr, np.float32)
    n = np.array(arr.shape)
    lvec_in = np.asarray(lvec_in, np.float64)
    T = np.linalg.inv(lvec_in[1:] / n[:, None]).T.astype(np.float32)
    f32 = np.float32
    i, j, k = np.meshgrid(*[np.arange(m, dtype=np.float32) for m in nout], indexing="ij")
    so = np.asarray(step_out, np.float32)
    o = np.asarray(origin_out, np.float32)
    pos = [o[c] + i * so[0, c] + j * so[1, c] + k * so[2, c] for c in range(3)]
    rc = np.asarray(rot_center, np.float32)
    R = np.asarray(rot, np.float32)
    d = [pos[c] - rc[c] for c in range(3)]
    pos = [rc[c] + (R[c, 0] * d[0] + R[c, 1] * d[1] + R[c, 2] * d[2]) for c in range(3)]
    return _lerp_b(arr, lvec_in[0], T, pos)


def interp_tip_at(arr, lvec_in, shape_new, lvec_new):
    """TipDensity.interp_at (interp_tip_at, ppafm/ocl/cl/FF.cl:1049-1093), float32 like the
    kernel: output indices past the middle wrap to negative positions i*a' + j*b' + k*c'; zero
    where a fractional coordinate (pos . rows of inv(input cell), the reference's form) exceeds
    0.5 in magnitude, else the periodic interpolation of the input about origin 0."""
    arr = np.asarray(arr, np.float32)
    n = np.array(arr.shape)
    lvec_in = np.asarray(lvec_in, np.float64)
    lvec_new = np.asarray(lvec_new, np.float64)
    T = np.linalg.inv(lvec_in[1:] / n[:, None]).T.astype(np.float32)
    Linv = np.linalg.inv(lvec_in[1:]).astype(np.float32)
    so = (lvec_new[1:] / np.array(shape_new)[:, None]).astype(np.float32)
    idx = []
    for a in range(3):
        i = np.arange(shape_new[a])
        i = np.where(i > shape_new[a] // 2, i - shape_new[a], i)
        idx.append(i.astype(np.float32))
    i, j, k = np.meshgrid(*idx, indexing="ij")
    pos = [i * so[0, c] + j * so[1, c] + k * so[2, c] for c in range(3)]
    frac = [Linv[a, 0] * pos[0] + Linv[a, 1] * pos[1] + Linv[a, 2] * pos[2] for a in range(3)]
    out = _lerp_b(arr, np.zeros(3), T, pos)
    out[(np.abs(frac[0]) > 0.5) | (np.abs(frac[1]) > 0.5) | (np.abs(frac[2]) > 0.5)] = 0.0
    return out


def _lerp_b(arr, origin, T, pos):
    """linearInterpB / linearInterpB4 (ppafm/ocl/cl/FF.cl:34-113) at the float32 points
    pos = [x, y, z] of a periodic grid arr [n0, n1, n2(, 4)] (C order) with lattice origin
    origin and transform rows T (lattice coordinate = (pos - origin) . T rows)."""
    f32 = np.float32
    n = np.array(arr.shape[:3])
    T = np.asarray(T, np.float32)
    oi = np.asarray(origin, np.float32)
    cc = [pos[c] - oi[c] for c in range(3)]
    g = [cc[0] * T[a, 0] + cc[1] * T[a, 1] + cc[2] * T[a, 2] for a in range(3)]
    fl = [np.floor(x) for x in g]
    t = [np.minimum(g[a] - fl[a], f32(0.99999994)) for a in range(3)]
    i0 = [np.mod(fl[a].astype(np.int64), n[a]) for a in range(3)]
    i1 = [(i0[a] + 1) % n[a] for a in range(3)]
    out = np.zeros(pos[0].shape + arr.shape[3:], np.float32)
    vec = arr.ndim == 4
    for bx in (0, 1):
        for by in (0, 1):
            for bz in (0, 1):
                w = (t[0] if bx else 1 - t[0]) * (t[1] if by else 1 - t[1]) * (t[2] if bz else 1 - t[2])
                v = arr[(i1 if bx else i0)[0], (i1 if by else i0)[1], (i1 if bz else i0)[2]]
                out += (w[..., None] if vec else w) * v
    return out


def hartree_ff_point_charges(nDim, lvec, pot_array, pot_lvec, xyzs, cLJs, Qs, QZs, h=0.05, nthreads=0):
    """The Hartree route with a point-charge tip (ppafm/ocl/field.py:1168-1315, used by makeFF
    at :1716-1720 when no tip density is set), float32 like the kernels: the electric field
    on the force-field grid -- the potential's periodic centred differences where both grids
    coincide (grad, FF.cl:920-961), else centred differences of the interpolated potential
    with step h (gradPotentialGrid, FF.cl:964-1008) -- then Lennard-Jones plus, per tip
    charge, Q times the field interpolated at the point shifted by QZ along z
    (evalLJC_Hartree, FF.cl:860-915).  FE [nz, ny, nx, 4] x-fastest like afm_ff_qzs."""
    nDim = np.asarray(nDim)
    lvec = np.asarray(lvec, np.float64)
    pot = np.asarray(pot_array, np.float32)
    pot_lvec = np.asarray(pot_lvec, np.float64)
    npot = np.array(pot.shape)
    pstep = pot_lvec[1:] / npot[:, None]
    step = lvec[1:4] / nDim[:, None]
    f32 = np.float32
    matching = (np.array_equal(npot, nDim) and (np.abs(pot_lvec[0] - lvec[0]) < 1e-3).all()
                and (np.abs(np.diag(pstep) * npot - np.diag(lvec[1:4])) < 1e-3).all() and (pstep == np.diag(np.diag(pstep))).all())
    i, j, k = np.meshgrid(*[np.arange(m, dtype=np.float32) for m in nDim], indexing="ij")
    so = step.astype(np.float32)
    o = lvec[0].astype(np.float32)
    pos = [o[c] + i * so[0, c] + j * so[1, c] + k * so[2, c] for c in range(3)]
    field = np.zeros(tuple(nDim) + (4,), np.float32)
    if matching:
        hs = np.diag(pstep).astype(np.float32)
        for a in range(3):
            field[..., a] = -(f32(0.5) * (np.roll(pot, -1, axis=a) - np.roll(pot, 1, axis=a)) / hs[a])
        field[..., 3] = pot
    else:
        Tp = np.linalg.inv(pstep).T.astype(np.float32)
        hh = f32(h)
        field[..., 3] = _lerp_b(pot, pot_lvec[0], Tp, pos)
        for a in range(3):
            pm = [pos[c] - hh if c == a else pos[c] for c in range(3)]
            pp = [pos[c] + hh if c == a else pos[c] for c in range(3)]
            field[..., a] = f32(0.5) * (_lerp_b(pot, pot_lvec[0], Tp, pm) - _lerp_b(pot, pot_lvec[0], Tp, pp)) / hh
    LJ = afm_ff_qzs(nDim, lvec, xyzs, np.zeros(len(xyzs)), cLJs, np.zeros(4), np.zeros(4), nthreads=nthreads)
    FE = LJ.transpose(2, 1, 0, 3).copy()
    T = np.linalg.inv(step).T.astype(np.float32)
    for Q, QZ in zip(np.asarray(Qs, np.float32), np.asarray(QZs, np.float32)):
        if Q != 0:
            FE += Q * _lerp_b(field, lvec[0], T, [pos[0], pos[1], pos[2] + QZ])
    return FE.transpose(2, 1, 0, 3).copy()


def hartree_ff(nDim, lvec, pot_array, pot_lvec, rho_multipole, sigma, xyzs, cLJs, rot_ff, rot_center, nthreads=0):
    """calc_force_hartree (ppafm/ocl/field.py:1446-1504) restated: the potential interpolated
    onto the force-field grid, cross-correlated with the tip density by FFT (float64 numpy),
    F = -grad E by periodic centred differences, plus Lennard-Jones (evalLJ form, R2SAFE
    1e-6).  rho_multipole: a multipole dict (the density made on the force-field grid), or
    (array, lvec) of a tip density on its own grid (resampled by interp_tip_at unless it is on
    the force-field grid).  FE [nz, ny, nx, 4] x-fastest like afm_ff_qzs."""
    nDim = np.asarray(nDim)
    lvec = np.asarray(lvec, np.float64)
    step = lvec[1:4] / nDim[:, None]
    pot_i = interp_at(pot_array, pot_lvec, nDim, lvec[0], step, rot_ff, rot_center).astype(np.float64)
    L = np.linalg.norm(lvec[1:4], axis=1)
    coords = []
    for a in range(3):
        c = np.linspace(0, L[a] * (1 - 1 / nDim[a]), nDim[a])
        c[c >= L[a] / 2] -= L[a]
        coords.append(c)
    X, Y, Z = np.meshgrid(*coords, indexing="ij")
    if isinstance(rho_multipole, dict):
        rho = getProbeDensity(np.vstack([np.zeros(3), lvec[1:4]]), X, Y, Z, L / nDim, sigma=sigma, multipole_dict=rho_multipole)
    else:
        arr, lv_t = np.asarray(rho_multipole[0], np.float32), np.asarray(rho_multipole[1], np.float64)
        same = tuple(arr.shape) == tuple(int(x) for x in nDim) and np.allclose(lv_t[1:], lvec[1:4])
        rho = arr if same else interp_tip_at(arr, lv_t, tuple(int(x) for x in nDim), lvec)
    rho = rho.astype(np.float32).astype(np.float64)
    E = np.real(np.fft.ifftn(np.conj(np.fft.fftn(rho)) * np.fft.fftn(pot_i))) * abs(np.linalg.det(step))
    hs = np.diag(step)
    F = [-0.5 * (np.roll(E, -1, axis=a) - np.roll(E, 1, axis=a)) / hs[a] for a in range(3)]
    FEc = np.stack(F + [E], axis=-1)
    LJ = afm_ff_qzs(nDim, lvec, xyzs, np.zeros(len(xyzs)), cLJs, np.zeros(4), np.zeros(4), nthreads=nthreads)
    return (FEc.transpose(2, 1, 0, 3) + LJ).astype(np.float32)


def afm_ff_qzs64(nDim, lvec, xyzs, qs, cLJs, Qs, QZs, points=None):
    """evalLJC_QZs_noPos's sum in float64 (numpy), at the listed grid points (ia,ib,ic) or
    all points; returns [npoints, 4] (Fx, Fy, Fz, E)."""
    nDim = np.asarray(nDim)
    lvec = np.asarray(lvec, dtype=np.float64)
    dl = lvec[1:4] / nDim[:, None]
    if points is None:
        ia, ib, ic = np.meshgrid(np.arange(nDim[0]), np.arange(nDim[1]), np.arange(nDim[2]), indexing="ij")
        points = np.column_stack([ia.ravel(), ib.ravel(), ic.ravel()])
    P = lvec[0] + points[:, 0:1] * dl[0] + points[:, 1:2] * dl[1] + points[:, 2:3] * dl[2]
    out = np.zeros((len(P), 4))
    x = np.asarray(xyzs, np.float64)
    c = np.asarray(cLJs, np.float64)
    q = np.asarray(qs, np.float64)
    for j in range(len(x)):
        dp = P - x[j]
        ir2 = 1.0 / ((dp * dp).sum(1) + 1e-6)
        ir6 = ir2**3
        out[:, 3] += (c[j, 1] * ir6 - c[j, 0]) * ir6
        out[:, :3] += dp * (((12.0 * c[j, 1] * ir6 - 6.0 * c[j, 0]) * ir6 * ir2))[:, None]
        for k in range(4):
            if Qs[k] == 0 or q[j] == 0:
                continue
            d2 = dp.copy()
            d2[:, 2] += QZs[k]
            jr2 = 1.0 / ((d2 * d2).sum(1) + 1e-6)
            E = q[j] * np.sqrt(jr2) * Qs[k] * 14.399644
            out[:, :3] += d2 * (E * jr2)[:, None]
            out[:, 3] += E
    return out


def rotTip(rot, zstep, tipR0):
    """relax.py:72-87."""
    tipRot = np.zeros((3, 4), np.float32)
    tipRot[:, :3] = rot
    tipRot[2, 3] = -zstep
    dpos0Tip = np.zeros(4, np.float32)
    dpos0Tip[0] = tipR0[0]
    dpos0Tip[1] = tipR0[1]
    dpos0Tip[2] = -np.sqrt(tipR0[2] ** 2 - tipR0[0] ** 2 - tipR0[1] ** 2)
    dpos0Tip[3] = tipR0[2]
    return tipRot, dpos0Tip


class AFMulator:
    """Point-charge AFMulator restated on the CPU (AFMulator.py:83-173, 211-241, 321-479).
    Relaxation uses exact FP32 trilinear weights where the reference samples an OpenCL
    image with hardware linear filtering."""

    relaxParams = [0.5, 0.1, 0.1 * 0.2, 0.1 * 5.0]

    def __init__(self, FFparams, pixPerAngstrome=10, lvec=None, scan_dim=(128, 128, 30), scan_window=((2.0, 2.0, 7.0), (18.0, 18.0, 10.0)),
                 iZPP=8, QZs=(0.1, 0, -0.1, 0), Qs=(-10, 20, -10, 0), df_steps=10, tipR0=(0.0, 0.0, 3.0),
                 tipStiffness=(0.25, 0.25, 0.0, 30.0), npbc=(1, 1, 0), f0Cantilever=30300, kCantilever=1800):
        self.FFparams = FFparams
        self.pixPerAngstrome = pixPerAngstrome
        self.scan_dim = tuple(scan_dim)
        self.scan_window = scan_window
        self.iZPP = iZPP
        self.QZs = np.array(QZs, np.float32)
        self.Qs = np.array(Qs, np.float32)
        self.df_steps = df_steps
        self.tipR0 = tipR0
        self.stiffness = np.array(tipStiffness, np.float32) / -np.float32(eVA_Nm)
        self.npbc = npbc
        self.f0 = f0Cantilever
        self.k = kCantilever
        self.lvec = get_lvec(scan_window, tipR0=tipR0, pixPerAngstrome=pixPerAngstrome) if lvec is None else np.asarray(lvec)
        self.nDim = genFFSampling(self.lvec, pixPerAngstrome)
        self.dz = (scan_window[1][2] - scan_window[0][2]) / scan_dim[2]
        self.dfWeight = get_simple_df_weight(df_steps, dz=self.dz).astype(np.float32)
        self.dfWeight *= eVA_Nm * f0Cantilever / kCantilever

    def eval(self, xyzs, Zs, qs, sample_lvec=None, nthreads=0, return_all=False, pot=None, rho=None, sigma=0.71, rot=np.eye(3), REAs=None):
        """pot = (array [n0,n1,n2], lvec [4,3]) selects the Hartree route with the multipole tip
        density rho (dict), or with the point-charge tip when rho is None; otherwise point
        charges qs.  REAs: per-atom (R, E, alpha) pair parameters (default: from FFparams)."""
        if pot is not None:
            sample_lvec = np.asarray(pot[1])[1:] if sample_lvec is None else sample_lvec
            qs = np.zeros(len(Zs))
        npbc = self.npbc if sample_lvec is not None else (0, 0, 0)
        REAs = getAtomsREA(self.iZPP, Zs, self.FFparams) if REAs is None else np.asarray(REAs, np.float64)
        cLJs = REA2LJ(REAs)
        xyzs = np.asarray(xyzs, np.float64)
        qs = np.asarray(qs, np.float64)
        rot_center = xyzs.mean(axis=0)
        if sum(npbc) > 0:
            Zs, xyzs, qs, cLJs = PBCAtoms3D_np(Zs, xyzs, qs, cLJs, sample_lvec, npbc=npbc)
        xyzs = np.dot(xyzs - rot_center, np.asarray(rot).T) + rot_center
        if pot is not None and rho is None:
            if not np.allclose(rot, np.eye(3)):
                raise NotImplementedError("the point-charge tip Hartree route has no rotation")
            FE = hartree_ff_point_charges(self.nDim, self.lvec, pot[0], pot[1], xyzs, cLJs, self.Qs, self.QZs, nthreads=nthreads)
        elif pot is not None:
            FE = hartree_ff(self.nDim, self.lvec, pot[0], pot[1], rho, sigma, xyzs, cLJs, np.linalg.inv(rot), rot_center, nthreads=nthreads)
        else:
            FE = afm_ff_qzs(self.nDim, self.lvec, xyzs, qs, cLJs, self.Qs, self.QZs, nthreads=nthreads)
        cell = self.lvec[1:4]
        invCell = np.transpose(np.linalg.inv(cell)).astype(np.float32)
        pos0 = np.array([0, 0, self.scan_window[1][2]]) - self.lvec[0]
        tipRot, dpos0Tip = rotTip(np.eye(3), self.dz, self.tipR0)
        xs = np.linspace(self.scan_window[0][0], self.scan_window[1][0], self.scan_dim[0])
        ys = np.linspace(self.scan_window[0][1], self.scan_window[1][1], self.scan_dim[1])
        As, Bs = np.meshgrid(xs, ys, indexing="ij")
        poss = np.zeros(As.shape + (4,), np.float32)
        poss[:, :, 0] = pos0[0] + As
        poss[:, :, 1] = pos0[1] + Bs
        poss[:, :, 2] = pos0[2]
        npix = self.scan_dim[0] * self.scan_dim[1]
        nz = self.scan_dim[2]
        FEs = np.zeros((npix, nz, 4), np.float32)
        paths = np.zeros((npix, nz, 4), np.float32)
        iters = np.zeros((npix, nz), np.int32)
        nD = _i32(self.nDim)
        relax = _c32(self.relaxParams)
        lib().oc_afm_relax_tilted(_p(_c32(FE), c_float), _p(nD, c_int), _p(_c32(invCell), c_float), npix, _p(_c32(poss), c_float), nz, _p(_c32(tipRot), c_float), _p(_c32(self.stiffness), c_float), _p(_c32(dpos0Tip), c_float), _p(relax, c_float), _p(np.zeros(4, np.float32), c_float), _p(FEs, c_float), _p(paths, c_float), _p(iters, c_int), nthreads)
        nzout = nz - len(self.dfWeight) + 1
        Fout = np.zeros((npix, nzout, 4), np.float32)
        lib().oc_afm_convolve_z(npix, nz, nzout, _p(FEs, c_float), _p(_c32(self.dfWeight), c_float), _p(Fout, c_float), nthreads)
        X = Fout[:, :, 2].reshape(self.scan_dim[0], self.scan_dim[1], nzout).copy()
        if return_all:
            return X, dict(FE=FE, FEs=FEs, paths=paths, iters=iters)
        return X


# ------------------------------------------------------------- the compiled reference


def reference_available():
    return os.path.exists(REF_PATH)


class Reference:
    """The reference C++ core compiled from its own sources (oracle/_ref), driven through
    the same C symbols ppafm/core.py binds (ProbeParticle.cpp:319-817)."""

    def __init__(self):
        L = ctypes.CDLL(REF_PATH)
        a1i = np.ctypeslib.ndpointer(dtype=np.int32, ndim=1, flags="CONTIGUOUS")
        a1d = np.ctypeslib.ndpointer(dtype=np.double, ndim=1, flags="CONTIGUOUS")
        a2d = np.ctypeslib.ndpointer(dtype=np.double, ndim=2, flags="CONTIGUOUS")
        a3d = np.ctypeslib.ndpointer(dtype=np.double, ndim=3, flags="CONTIGUOUS")
        a4d = np.ctypeslib.ndpointer(dtype=np.double, ndim=4, flags="CONTIGUOUS")
        L.setGridN.argtypes = [a1i]
        L.setGridCell.argtypes = [a2d]
        L.setFF_Fpointer.argtypes = [a4d]
        L.setFF_Epointer.argtypes = [a3d]
        L.setRelax.argtypes = [c_int, c_double, c_double, c_double]
        L.setFIRE.argtypes = [c_double, c_double, c_double]
        L.setTip.argtypes = [c_double, c_double, a1d, a1d]
        L.getLennardJonesFF.argtypes = [c_int, a2d, a2d]
        L.getCoulombFF.argtypes = [c_int, a2d, a1d, c_int]
        L.relaxTipStroke.argtypes = [c_int, c_int, c_int, a2d, a2d, a2d, ctypes.c_void_p]
        L.relaxTipStroke.restype = c_int
        L.relaxTipStrokes_omp.argtypes = [c_int, c_int, c_int, c_int, c_int, a4d, a4d, a4d, ctypes.c_void_p]
        L.relaxTipStrokes_omp.restype = c_int
        self.L = L

    def set_grid(self, n, cell):
        self.L.setGridN(np.array(n, dtype=np.int32))
        self.L.setGridCell(np.array(cell, dtype=np.float64).reshape(3, 3))
