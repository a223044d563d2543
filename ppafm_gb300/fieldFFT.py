"""The FFT density-overlap route, mirroring ppafm/fieldFFT.py on the GPU.

``potential2forces_mem`` keeps the reference's arguments and host float64 results; ``FFTGrid``
is the device-resident form (cuFFT plans and spectrum buffers kept per grid shape) used by
the density-overlap pipeline.  Arithmetic is float32 complex (cuFFT R2C/C2R) with fused
k-space kernels, agreeing with the reference's float64 numpy to ~1e-6 of the field's maximum,
or float64 complex (``f64=True``: D2Z/Z2D, ~1e-7 of each point's own value, the float32 grid
storage) where the small forces far from the atoms matter.
"""

import ctypes

import numpy as np
import torch

from ._lib import FF_ACCUMULATE, FF_WITH_E, FFT_F64, check, dptr, iptr, lib, stream_handle, tptr

MULTIPOLES = ("s", "px", "py", "pz", "dz2", "dx2", "dy2", "dxy", "dxz", "dyz")


def _lvec4(lvec):
    lvec = np.asarray(lvec, dtype=np.float64)
    if lvec.shape == (3, 3):
        lvec = np.vstack([np.zeros(3), lvec])
    return np.ascontiguousarray(lvec)


def multipole_vector(multipole):
    """Coefficients in the order of getSphericalHarmonic (fieldFFT.py:58-96); None = pure s."""
    v = np.zeros(10)
    if multipole is None:
        v[0] = 1.0
        return v
    for k, c in multipole.items():
        if k not in MULTIPOLES:
            raise ValueError(f"unknown multipole {k}")
        v[MULTIPOLES.index(k)] = c
    return v


class FFTGrid:
    """cuFFT plans + spectrum buffers for one grid shape (n0, n1, n2); f64 selects float64
    transforms (input and output grids stay float32)."""

    def __init__(self, n, device="cuda", f64=False):
        self.n = np.array(n, dtype=np.int32)
        self.N = int(np.prod(self.n.astype(np.int64)))
        self.device = device
        self.f64 = bool(f64)
        h = ctypes.c_void_p()
        check(lib().ppgpu_fft_create(iptr(self.n), FFT_F64 if f64 else 0, ctypes.byref(h)))
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                lib().ppgpu_fft_destroy(h)
            except Exception:
                pass
            self.handle = None

    def empty(self):
        return torch.empty(tuple(int(x) for x in self.n), dtype=torch.float32, device=self.device)

    def potential2forces(self, V, rho, lvec, FE=None, scale=1.0, with_E=True, accumulate=False, stream=None):
        """FE (float4 grid, flat) = (accumulate ? FE : 0) + scale * (Fx, Fy, Fz, E)."""
        if FE is None:
            FE = torch.empty(self.N * 4, dtype=torch.float32, device=self.device)
        flags = (FF_WITH_E if with_E else 0) | (FF_ACCUMULATE if accumulate else 0)
        lv = _lvec4(lvec)
        check(lib().ppgpu_fft_potential2forces(self.handle, tptr(V.contiguous()), tptr(rho.contiguous()), dptr(lv), float(scale), flags, tptr(FE), stream_handle(stream)))
        return FE

    def probe_density(self, lvec, sigma=0.7, multipole=None, out=None, stream=None):
        """getProbeDensity (fieldFFT.py:99-118), tilt 0."""
        out = self.empty() if out is None else out
        mp = multipole_vector(multipole)
        check(lib().ppgpu_fft_probe_density(self.handle, tptr(out), dptr(_lvec4(lvec)), float(sigma), dptr(mp), stream_handle(stream)))
        return out

    def density_power(self, rho, B=1.0, fix_negative=True, stream=None):
        """handle_negative_density then rho**B in place (cli/conv_rho.py:18-22, 57-64)."""
        check(lib().ppgpu_fft_density_power(self.handle, tptr(rho), float(B), 1 if fix_negative else 0, stream_handle(stream)))
        return rho

    def poisson(self, rho_charge, lvec, out=None, stream=None):
        """Hartree potential (V) of a periodic charge density (e/A^3), zero mean."""
        out = self.empty() if out is None else out
        check(lib().ppgpu_fft_poisson(self.handle, tptr(rho_charge.contiguous()), dptr(_lvec4(lvec)), tptr(out), stream_handle(stream)))
        return out

    def correlate(self, V, rho, scale=1.0, out=None, stream=None):
        """IFFT(conj(FFT(rho)) FFT(V)) * scale / N (the AFMulator's FFT cross-correlation);
        rho None reuses the spectrum of the last rho."""
        out = self.empty() if out is None else out
        check(lib().ppgpu_fft_correlate(self.handle, tptr(V.contiguous()), None if rho is None else tptr(rho.contiguous()), float(scale), tptr(out), stream_handle(stream)))
        return out

    def gaussians(self, lvec, atoms, out=None, accumulate=False, stream=None):
        """Sum of normalised Gaussians; atoms [n,5] = (x, y, z relative to the origin, sigma, weight)."""
        out = self.empty() if out is None else out
        a = torch.as_tensor(np.ascontiguousarray(atoms, dtype=np.float64)).to(self.device)
        check(lib().ppgpu_gaussian_density(tptr(out), iptr(self.n), dptr(_lvec4(lvec)), len(atoms), tptr(a), 1 if accumulate else 0, stream_handle(stream)))
        return out


def potential2forces_mem(V, lvec, nDim, sigma=0.7, rho=None, multipole=None, doForce=True, doPot=False, deleteV=True, tilt=0.0, f64=True):
    """fieldFFT.py:268-319 on the GPU: returns (Fx, Fy, Fz, E) float64 host arrays (None for
    the parts not requested).  rho=None builds the tip density from sigma/multipole.  The
    host-array drop-in defaults to float64 transforms (the reference is float64 numpy)."""
    if tilt != 0.0:
        raise NotImplementedError("tilted tip densities are not supported")
    dims = tuple(int(x) for x in nDim)
    V = np.asarray(V)
    if V.shape != dims:
        raise ValueError(f"V has shape {V.shape}, nDim is {dims}")
    g = FFTGrid(dims, f64=f64)
    Vd = torch.as_tensor(np.ascontiguousarray(V, dtype=np.float32)).to(g.device)
    rd = g.probe_density(lvec, sigma, multipole) if rho is None else torch.as_tensor(np.ascontiguousarray(rho, dtype=np.float32)).to(g.device)
    FE = g.potential2forces(Vd, rd, lvec, with_E=doPot)
    out = FE.view(dims + (4,)).cpu().numpy().astype(np.float64)
    Fx = Fy = Fz = E = None
    if doForce:
        Fx, Fy, Fz = out[..., 0].copy(), out[..., 1].copy(), out[..., 2].copy()
    if doPot:
        E = out[..., 3].copy()
    return Fx, Fy, Fz, E


def getSampleDimensions(lvec):
    """The cell rows of lvec (fieldFFT.py:17-19; a plain array where the reference returns the
    deprecated numpy matrix)."""
    return np.array(np.asarray(lvec, dtype=np.float64)[1:])


def getSize(inp_axis, dims, sampleSize):
    """(|cell vector|, its length per grid step) along 'x', 'y' or 'z' (fieldFFT.py:22-29)."""
    a = {"x": 0, "y": 1, "z": 2}[inp_axis]
    size = np.linalg.norm(np.asarray(sampleSize)[a])
    return size, size / dims[a]


def getMGrid(dims, dd):
    """Coordinate arrays X, Y, Z of the rolled grid the FFT route works on, the origin at index
    0 and negative coordinates past the middle (fieldFFT.py:32-48)."""
    out = []
    for a in range(3):
        n = int(dims[a])
        shift = n // 2
        shift_ = shift + (1.0 if n % 2 else 0.0)
        idx = np.arange(n, dtype=np.float64)
        line = dd[a] * np.roll(idx - shift_, shift)
        shape = [1, 1, 1]
        shape[a] = n
        out.append(np.broadcast_to(line.reshape(shape), tuple(int(x) for x in dims)).copy())
    return out[0], out[1], out[2]


def getProbeDensity(lvec, nDim=None, Z=None, dd=None, *args, sigma=0.7, multipole_dict=None, tilt=0.0, **kw):
    """The normalised Gaussian tip density with multipoles (fieldFFT.py:99-118) on the GPU, tilt
    0, on the rolled grid: ``getProbeDensity(lvec, nDim, sigma=..., multipole_dict=...)``, or
    the reference's form ``getProbeDensity(sampleSize, X, Y, Z, dd, sigma, multipole_dict,
    tilt)`` with X, Y, Z from getMGrid (the only coordinates the GPU makes)."""
    if isinstance(nDim, np.ndarray) and nDim.ndim == 3:  # the reference's (sampleSize, X, Y, Z, dd, ...)
        X, Y, Zc = nDim, Z, dd
        dd = args[0] if args else kw.pop("dd")
        rest = list(args[1:])
        if rest:
            sigma = rest.pop(0)
        if rest:
            multipole_dict = rest.pop(0)
        if rest:
            tilt = rest.pop(0)
        dims = X.shape
        Xg, Yg, Zg = getMGrid(dims, dd)
        if not (np.allclose(X, Xg) and np.allclose(Y, Yg) and np.allclose(Zc, Zg)):
            raise ValueError("the GPU makes the density on getMGrid's coordinates; X, Y, Z differ from them")
        cell = np.asarray(lvec, dtype=np.float64)
        lvec = np.vstack([np.zeros(3), cell[-3:]])
        nDim = dims
    elif Z is not None:
        sigma = Z
        if dd is not None:
            multipole_dict = dd
    if tilt != 0.0:
        raise NotImplementedError("tilted tip densities are not supported")
    g = FFTGrid(nDim)
    return g.probe_density(lvec, sigma, multipole_dict).cpu().numpy().astype(np.float64)
