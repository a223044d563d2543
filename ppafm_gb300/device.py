"""Device-resident building blocks of the hot path.

Force fields live in HBM as one float4 (Fx, Fy, Fz, E) per grid point, C order
[n0][n1][n2] -- the reference's i3D order (ppafm/cpp/Grid.h:16) with the three force
components and the energy interleaved so a trilinear corner is one 16-byte load.
torch only allocates the buffers and supplies the stream; all arithmetic is in
libppgpu.so.  Every function raises ``PPGPUError`` on failure -- there is no CPU fallback.
"""

import contextlib
import ctypes

import numpy as np
import torch

from ._lib import (
    ATOM_FLOATS,
    FF_ACCUMULATE,
    FF_COULOMB,
    FF_F64,
    FF_LJ,
    FF_LJC,
    FF_QZS,
    FF_WITH_E,
    RELAX_NPARAM,
    check,
    dptr,
    iptr,
    lib,
    stream_handle,
    tptr,
)

__all__ = ["pack_atoms", "DeviceFF", "relax_params", "relax_scan", "relax_strokes", "iter_counter", "tip_spline", "autotune_relax_tps"]


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("ppafm_gb300 device path needs a CUDA device (no CPU fallback)")


def pack_atoms(Rs, cLJs=None, kqq=None, device="cuda", stream=None):
    """Packs atoms into the 48-byte device records of include/ppgpu.h.
    Rs: [n,3] positions relative to the grid origin (float64); cLJs: [n,2] (c6, c12);
    kqq: [n] charge coefficients.  Returns (records tensor [n,12] float32, n, ncharged); the
    copy to the device is queued on stream (default: the current stream)."""
    _require_cuda()
    Rs = np.ascontiguousarray(Rs, dtype=np.float64).reshape(-1, 3)
    n = len(Rs)
    c = None if cLJs is None else np.ascontiguousarray(cLJs, dtype=np.float64).reshape(-1, 2)
    q = None if kqq is None else np.ascontiguousarray(kqq, dtype=np.float64).reshape(-1)
    dev = torch.device(device)
    # packed in pinned memory and copied without a synchronisation: the host can prepare the
    # next system while the GPU works (the caching host allocator keeps the buffer until the
    # copy has run)
    rec_t = torch.zeros((max(n, 1), ATOM_FLOATS), dtype=torch.float32, pin_memory=dev.type == "cuda")
    nch = np.zeros(1, dtype=np.int32)
    check(lib().ppgpu_pack_atoms(n, dptr(Rs), dptr(c), dptr(q), ctypes.cast(rec_t.data_ptr(), ctypes.POINTER(ctypes.c_float)), iptr(nch)))
    if dev.type != "cuda":
        return rec_t, n, int(nch[0])
    if stream is None:
        return rec_t.to(dev, non_blocking=True), n, int(nch[0])
    with torch.cuda.stream(stream):
        return rec_t.to(dev, non_blocking=True), n, int(nch[0])


def iter_counter(device="cuda"):
    return torch.zeros(1, dtype=torch.int64, device=device)


class DeviceFF:
    """A force-field grid in device memory.

    n: grid size (n0, n1, n2); lvec: 4x3 (origin, a, b, c) or 3x3 cell (origin 0)."""

    def __init__(self, n, lvec, device="cuda", FE=None):
        _require_cuda()
        self.n = np.array(n, dtype=np.int32)
        lvec = np.asarray(lvec, dtype=np.float64)
        if lvec.shape == (3, 3):
            lvec = np.vstack([np.zeros(3), lvec])
        self.lvec = lvec
        self.origin = lvec[0].copy()
        self.cell = np.ascontiguousarray(lvec[1:4])
        self.npts = int(np.prod(self.n.astype(np.int64)))
        self.FE = FE if FE is not None else torch.empty(self.npts * 4, dtype=torch.float32, device=device)

    @property
    def grid4(self):
        return self.FE.view(int(self.n[0]), int(self.n[1]), int(self.n[2]), 4)

    def compute(self, atoms, natoms, ncharged, mode, kind=0, Q=0.0, Fmax=0.0, Qs=None, QZs=None, with_E=False, accumulate=False, f64=False, stream=None):
        """Fills (or adds to) the grid; see ppgpu_ff_grid for the modes.  f64=True evaluates
        the sums in float64 (the GPU error oracle of the float32 kernels)."""
        flags = (FF_WITH_E if with_E else 0) | (FF_ACCUMULATE if accumulate else 0) | (FF_F64 if f64 else 0)
        qs = None if Qs is None else np.ascontiguousarray(Qs, dtype=np.float64)
        qz = None if QZs is None else np.ascontiguousarray(QZs, dtype=np.float64)
        check(lib().ppgpu_ff_grid(tptr(self.FE), iptr(self.n), dptr(self.cell), tptr(atoms), natoms, ncharged, mode, kind, float(Q), float(Fmax), dptr(qs), dptr(qz), flags, stream_handle(stream)))
        return self

    def compute_subgrid(self, i0, ns, atoms, natoms, ncharged, mode, kind=0, Q=0.0, Fmax=0.0, out=None, with_E=False, f64=False, stream=None):
        """Grid points [i0, i0+ns) into a new float4 tensor [ns0*ns1*ns2*4]."""
        ns = np.array(ns, dtype=np.int32)
        i0 = np.array(i0, dtype=np.int32)
        if out is None:
            out = torch.empty(int(np.prod(ns.astype(np.int64))) * 4, dtype=torch.float32, device=self.FE.device)
        flags = (FF_WITH_E if with_E else 0) | (FF_F64 if f64 else 0)
        check(lib().ppgpu_ff_subgrid(tptr(out), iptr(self.n), dptr(self.cell), iptr(i0), iptr(ns), tptr(atoms), natoms, ncharged, mode, kind, float(Q), float(Fmax), None, None, flags, stream_handle(stream)))
        return out

    def clamp(self, Fmax, stream=None):
        check(lib().ppgpu_clamp_grid(tptr(self.FE), self.npts, float(Fmax), stream_handle(stream)))
        return self

    def axpby(self, a, other, b, stream=None):
        """self = a*self + b*other."""
        check(lib().ppgpu_axpby_grid(tptr(self.FE), tptr(self.FE), float(a), tptr(other.FE), float(b), self.npts, stream_handle(stream)))
        return self

    def from_host_f64(self, F, E=None, stream=None):
        Fd = torch.as_tensor(np.ascontiguousarray(F, dtype=np.float64)).to(self.FE.device)
        Ed = None if E is None else torch.as_tensor(np.ascontiguousarray(E, dtype=np.float64)).to(self.FE.device)
        check(lib().ppgpu_grid_from_f64(tptr(self.FE), tptr(Fd), tptr(Ed), self.npts, stream_handle(stream)))
        return self

    def to_host(self):
        """(F [n0,n1,n2,3] float64, E [n0,n1,n2] float64)."""
        g = self.grid4.cpu().numpy().astype(np.float64)
        return g[..., :3].copy(), g[..., 3].copy()


def relax_params(maxIters=1000, convF2=1e-8, dt=0.1, damping=0.1, finc=1.1, fdec=0.5, falpha=0.99, lRadial=4.0, kRadial=0.0, rPP0=(0.0, 0.0, 4.0), kSpring=(0.0, 0.0, 0.0), make_consistent=True):
    """The 15-entry parameter vector of ppgpu_relax_* (setRelax/setFIRE/setTip state).
    rPP0 is put on the radial sphere like TIP::makeConsistent (ProbeParticle.cpp:64-69)."""
    rPP0 = np.array(rPP0, dtype=np.float64).copy()
    if make_consistent and abs(kRadial) > 1e-8:
        rPP0[2] = -np.sqrt(lRadial * lRadial - rPP0[0] ** 2 - rPP0[1] ** 2)
    p = np.zeros(RELAX_NPARAM)
    p[0:9] = [maxIters, convF2, dt, damping, finc, fdec, falpha, lRadial, kRadial]
    p[9:12] = rPP0
    p[12:15] = kSpring
    return p


@contextlib.contextmanager
def tip_spline(spline):
    """Radial tip spline for the relaxations run inside the block (ppgpu_set_tip_spline):
    None, a core.SplineParameters (or any object with np_rff_xs / np_rff_ydys), or a pair
    (xs [n], ydys [n, 2])."""
    if spline is None:
        yield
        return
    if hasattr(spline, "np_rff_xs"):
        xs, yd = spline.np_rff_xs, spline.np_rff_ydys
    else:
        xs, yd = spline
    xs = np.ascontiguousarray(xs, dtype=np.float64)
    yd = np.ascontiguousarray(yd, dtype=np.float64).reshape(-1)
    if yd.size != 2 * xs.size:
        raise ValueError("tip spline: ydys needs a (value, slope) pair per knot")
    check(lib().ppgpu_set_tip_spline(len(xs), dptr(xs), dptr(yd)))
    try:
        yield
    finally:
        check(lib().ppgpu_set_tip_spline(0, None, None))


def autotune_relax_tps(ff, prm, xs, ys, zs, candidates=(1, 2, 4, 8), reps=2, apply=True):
    """Times relax_scan with each number of lanes per stroke on this scan and (apply) keeps the
    fastest for the relaxations that follow.  Returns (best, {tps: ms})."""
    times = {}
    out = {}
    try:
        for t in candidates:
            check(lib().ppgpu_set_relax_tps(int(t)))
            relax_scan(ff, prm, xs, ys, zs, out=out)  # warm-up (and buffers)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(reps):
                relax_scan(ff, prm, xs, ys, zs, out=out)
            b.record()
            b.synchronize()
            times[int(t)] = a.elapsed_time(b) / reps
    finally:
        best = min(times, key=times.get) if times else 1
        check(lib().ppgpu_set_relax_tps(best if apply else 0))
    return best, times


def relax_strokes(ff, prm, rTips, probeStart=1, relaxAlg=1, iters=False, counter=None, stream=None):
    """relaxTipStrokes semantics on device tensors: rTips [..., nstep, 3] float64 (relative
    to the grid origin).  Returns (rs, fs, itrsum, iters-or-None)."""
    rT = rTips if isinstance(rTips, torch.Tensor) else torch.as_tensor(np.ascontiguousarray(rTips, dtype=np.float64))
    rT = rT.to(ff.FE.device).contiguous()
    shp = rT.shape
    nstep = shp[-2]
    nstroke = int(np.prod(shp[:-2]))
    rs = torch.empty_like(rT)
    fs = torch.empty_like(rT)
    itrsum = torch.empty(nstroke, dtype=torch.int32, device=rT.device)
    it = torch.empty(shp[:-1], dtype=torch.int32, device=rT.device) if iters else None
    prm = np.ascontiguousarray(prm, dtype=np.float64)
    check(lib().ppgpu_relax_strokes(tptr(ff.FE), iptr(ff.n), dptr(ff.cell), dptr(prm), probeStart, relaxAlg, nstroke, nstep, tptr(rT), tptr(rs), tptr(fs), tptr(it), tptr(itrsum), tptr(counter), stream_handle(stream)))
    return rs, fs, itrsum, it


def upload_f64(v, dev, stream=None):
    """A float64 device tensor of v: device tensors pass through; host arrays go through pinned
    memory without a synchronisation, on stream (default: the current stream)."""
    if isinstance(v, torch.Tensor) and v.is_cuda:
        return v.to(torch.float64).contiguous()
    t = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).pin_memory()
    if stream is None:
        return t.to(dev, non_blocking=True)
    with torch.cuda.stream(stream):
        return t.to(dev, non_blocking=True)


def relax_scan(ff, prm, xs, ys, zs, pos_offset=(0.0, 0.0, 0.0), df_weights=None, want_fzs=True, want_ppos=True, want_iters=False, counter=None, out=None, stream=None):
    """Regular scan with relaxedScan3D_omp semantics: tips at (xs[ix], ys[iy], zs[iz])
    relative to the grid origin, zs in approach order (descending); host arrays or float64
    device tensors.  Outputs ascending z.
    df_weights (already scaled, np.convolve orientation) adds the fused Δf epilogue."""
    dev = ff.FE.device
    xs_d, ys_d, zs_d = (upload_f64(v, dev, stream) for v in (xs, ys, zs))
    nx, ny, nz = len(xs), len(ys), len(zs)
    out = {} if out is None else out
    need_fzs = want_fzs or df_weights is not None
    if need_fzs and "fzs" not in out:
        out["fzs"] = torch.empty((nx, ny, nz), dtype=torch.float32, device=dev)
    if want_ppos and "ppos" not in out:
        out["ppos"] = torch.empty((nx, ny, nz, 3), dtype=torch.float32, device=dev)
    if want_iters and "iters" not in out:
        out["iters"] = torch.empty((nx, ny, nz), dtype=torch.int32, device=dev)
    nw = 0
    W = None
    if df_weights is not None:
        W = np.ascontiguousarray(df_weights, dtype=np.float64)
        nw = len(W)
        if "df" not in out:
            out["df"] = torch.empty((nx, ny, nz - nw + 1), dtype=torch.float32, device=dev)
    prm = np.ascontiguousarray(prm, dtype=np.float64)
    off = np.ascontiguousarray(pos_offset, dtype=np.float64)
    check(
        lib().ppgpu_relax_scan(
            tptr(ff.FE), iptr(ff.n), dptr(ff.cell), dptr(prm), nx, ny, nz, tptr(xs_d), tptr(ys_d), tptr(zs_d), dptr(off),
            tptr(out.get("fzs")), tptr(out.get("ppos")), tptr(out.get("iters")), nw, dptr(W), tptr(out.get("df")), tptr(counter), stream_handle(stream),
        )
    )
    return out


MODES = dict(LJ=FF_LJ, COULOMB=FF_COULOMB, LJC=FF_LJC, QZS=FF_QZS)
