"""AFMulator with the reference's constructor and ``eval`` signature
(ppafm/ocl/AFMulator.py:83-173), point-charge method, on libppgpu.

eval(xyzs, Zs, qs) builds the Lennard-Jones + tip-point-charge force field
(evalLJC_QZs_noPos, ppafm/ocl/cl/FF.cl:366-423) in HBM, relaxes every pixel column with
the tilted-stroke FIRE of relaxStrokesTilted (ppafm/ocl/cl/relax.cl:391-464) and applies
the z convolution (convolveZ, relax.cl:571-608) in the same kernel, returning the Δf
stack X [nx, ny, nz - df_steps + 1].  Interpolation uses exact float32 trilinear weights
where the reference samples an OpenCL image with hardware filtering.

Not provided: Hartree-potential and FDBM force fields (``qs`` as a potential,
``rho``/``rho_delta``/``rho_sample``), plotting.
"""

import time

import numpy as np
import torch

from . import common
from ._lib import AFM_NPARAM, FF_QZS, check, dptr, iptr, lib, stream_handle, tptr
from .device import DeviceFF, iter_counter, pack_atoms

VALID_SIZES = np.array([16, 32, 64, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048])


def get_lvec(scan_window, pad=(3.0, 3.0, 5.0), tipR0=(0.0, 0.0, 3.0), pixPerAngstrome=10):
    """Force-field box around the scan window (AFMulator.py:702-719)."""
    pad = np.array(pad)
    tipR0 = np.array(tipR0)
    center = (np.array(scan_window[0]) + np.array(scan_window[1])) / 2
    box = (np.array(scan_window[1]) - np.array(scan_window[0])) + 2 * pad
    nDim = (pixPerAngstrome * box).round().astype(np.int32)
    nDim = np.array([VALID_SIZES[VALID_SIZES >= d][0] for d in nDim])
    box = nDim / pixPerAngstrome
    origin = center - box / 2 - tipR0
    return np.array([origin, [box[0], 0, 0], [0, box[1], 0], [0, 0, box[2]]])


class AFMulator:
    bMergeConv = True  # relaxation and z convolution always run fused here
    relaxParams = [0.5, 0.1, 0.1 * 0.2, 0.1 * 5.0]

    def __init__(self, pixPerAngstrome=10, lvec=None, scan_dim=(128, 128, 30), scan_window=((2.0, 2.0, 7.0), (18.0, 18.0, 10.0)), iZPP=8, QZs=[0.1, 0, -0.1, 0], Qs=[-10, 20, -10, 0], rho=None, sigma=0.71, rho_delta=None, A_pauli=18.0, B_pauli=1.0,
                 fdbm_vdw_type="D3", d3_params="PBE", lj_vdw_damp=2, df_steps=10, tipR0=[0.0, 0.0, 3.0], tipStiffness=[0.25, 0.25, 0.0, 30.0], npbc=(1, 1, 0), f0Cantilever=30300, kCantilever=1800, colorscale="gray", minimize_memory=False):
        if rho is not None or rho_delta is not None:
            raise NotImplementedError("tip densities (Hartree / FDBM force fields) are not supported")
        self.iZPP = iZPP
        self.tipR0 = np.array(tipR0, dtype=np.float64)  # a copy: randomize_tip edits it in place
        self.f0Cantilever = f0Cantilever
        self.kCantilever = kCantilever
        self.npbc = npbc
        self.sigma = sigma
        self.A_pauli = A_pauli
        self.B_pauli = B_pauli
        self.colorscale = colorscale
        self.sample_lvec = None
        self.stiffness = np.array(tipStiffness, dtype=np.float32) / np.float32(-common.eVA_Nm)
        self.typeParams = common.loadSpecies()
        self.counter = None
        self._ff = None
        self.setScanWindow(scan_window, scan_dim, df_steps)
        self.setLvec(lvec, pixPerAngstrome)
        self.setQs(Qs, QZs)
        self.last_timing = {}

    # ------------------------------------------------------------------ set-up

    def setLvec(self, lvec=None, pixPerAngstrome=None):
        if pixPerAngstrome is not None:
            self.pixPerAngstrome = pixPerAngstrome
        self.lvec = np.asarray(lvec, dtype=np.float64) if lvec is not None else get_lvec(self.scan_window, tipR0=self.tipR0, pixPerAngstrome=self.pixPerAngstrome)
        self.nDim = common.genFFSampling(self.lvec, pixPerAngstrome=self.pixPerAngstrome)
        self._ff = None

    def setScanWindow(self, scan_window=None, scan_dim=None, df_steps=None):
        """Scan geometry and the Δf weights (AFMulator.py:211-241)."""
        if scan_window is not None:
            self.scan_window = scan_window
        if scan_dim is not None:
            self.scan_dim = tuple(int(x) for x in scan_dim)
        if df_steps is not None:
            if df_steps <= 0 or df_steps > self.scan_dim[2]:
                raise ValueError(f"df_steps should be between 1 and scan_dim[2]({self.scan_dim[2]}), but got {df_steps}.")
            self.df_steps = df_steps
        self.dz = (self.scan_window[1][2] - self.scan_window[0][2]) / self.scan_dim[2]
        self.dfWeight = common.get_simple_df_weight(self.df_steps, dz=self.dz).astype(np.float32)
        self.dfWeight *= common.eVA_Nm * self.f0Cantilever / self.kCantilever
        self.amplitude = self.dz * len(self.dfWeight)
        self._out = None

    def setQs(self, Qs, QZs):
        if len(Qs) != 4 or len(QZs) != 4:
            raise ValueError("Qs and Qzs must have length 4")
        self.Qs = np.array(Qs, dtype=np.float32)
        self.QZs = np.array(QZs, dtype=np.float32)

    def setStiffness(self, tipStiffness):
        self.stiffness = np.array(tipStiffness, dtype=np.float32) / np.float32(-common.eVA_Nm)

    def setRho(self, rho=None, sigma=0.71, B_pauli=1.0):
        if rho is not None:
            raise NotImplementedError("tip densities are not supported")

    # --------------------------------------------------------------- imaging

    def prepareFF(self, xyzs, Zs, qs, rho_sample=None, sample_lvec=None, rot=np.eye(3), rot_center=None, REAs=None, stream=None):
        """Point-charge force field on the device (AFMulator.py:321-429, field.py:1608-1713)."""
        if rho_sample is not None:
            raise NotImplementedError("FDBM (rho_sample) is not supported")
        if qs is not None and not isinstance(qs, np.ndarray):
            qs = np.asarray(qs)
        if qs is None:
            qs = np.zeros(len(Zs))
        if sample_lvec is not None:
            self.sample_lvec = np.asarray(sample_lvec)
        npbc = self.npbc if self.sample_lvec is not None else (0, 0, 0)
        xyzs = np.asarray(xyzs)
        if rot_center is None:
            rot_center = xyzs.mean(axis=0)
        if REAs is None:
            REAs = common.getAtomsREA(self.iZPP, Zs, self.typeParams, alphaFac=-1.0)
        cLJs = common.REA2LJ(np.asarray(REAs, dtype=np.float64))
        if sum(npbc) > 0:
            Zs, xyzs, qs, cLJs, REAs = common.PBCAtoms3D_np(Zs, xyzs, qs, cLJs, REAs, self.sample_lvec, npbc=npbc)
        x = np.array(xyzs, copy=True)
        x -= rot_center
        x = np.dot(x, np.asarray(rot).T) + rot_center
        atoms32 = np.concatenate([x, np.asarray(qs)[:, None]], axis=1).astype(np.float32)
        c32 = np.asarray(cLJs).astype(np.float32)
        if self._ff is None:
            self._ff = DeviceFF(self.nDim, self.lvec)
        R = atoms32[:, :3].astype(np.float64) - self.lvec[0]
        rec, na, nch = pack_atoms(R, c32.astype(np.float64), atoms32[:, 3].astype(np.float64))
        self._atoms = rec
        self._ff.compute(rec, na, nch, FF_QZS, Qs=self.Qs.astype(np.float64), QZs=self.QZs.astype(np.float64), with_E=True, stream=stream)
        return self._ff

    def _scan_points(self):
        pos0 = np.array([0, 0, self.scan_window[1][2]]) - self.lvec[0]
        xs = np.linspace(self.scan_window[0][0], self.scan_window[1][0], self.scan_dim[0])
        ys = np.linspace(self.scan_window[0][1], self.scan_window[1][1], self.scan_dim[1])
        As, Bs = np.meshgrid(xs, ys, indexing="ij")
        poss = np.zeros(As.shape + (4,), dtype=np.float32)
        poss[:, :, 0] = pos0[0] + As * 1.0 + Bs * 0.0
        poss[:, :, 1] = pos0[1] + As * 0.0 + Bs * 1.0
        poss[:, :, 2] = pos0[2] + As * 0.0 + Bs * 0.0
        return poss

    def _afm_params(self):
        p = np.zeros(AFM_NPARAM)
        p[0:4] = np.array(self.relaxParams, dtype=np.float32)
        p[4:8] = self.stiffness
        r0 = self.tipR0
        p[8:12] = np.array([r0[0], r0[1], -np.sqrt(r0[2] ** 2 - r0[0] ** 2 - r0[1] ** 2), r0[2]], dtype=np.float32)
        p[12:24] = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, -self.dz], dtype=np.float32)
        p[24:28] = 0.0
        return p

    def evalAFM(self, X=None, stream=None, keep_device=False, want_paths=False, want_iters=False, out=None):
        """Relaxation + z convolution of the prepared force field (AFMulator.py:447-479).
        out: a contiguous float32 device tensor [nx, ny, nz - df_steps + 1] that receives the
        image (returned as is, nothing is copied to the host)."""
        ff = self._ff
        nx, ny, nz = self.scan_dim
        npix = nx * ny
        nw = len(self.dfWeight)
        nout = nz - nw + 1
        dev = ff.FE.device
        if self._out is None:
            self._points = torch.from_numpy(self._scan_points().reshape(-1, 4)).to(dev)
            self._out = dict(FEs=torch.empty((npix, nz, 4), dtype=torch.float32, device=dev), X=torch.empty((npix, nout), dtype=torch.float32, device=dev))
        if want_paths and "paths" not in self._out:
            self._out["paths"] = torch.empty((npix, nz, 4), dtype=torch.float32, device=dev)
        if want_iters and "iters" not in self._out:
            self._out["iters"] = torch.empty((npix, nz), dtype=torch.int32, device=dev)
        if self.counter is None:
            self.counter = iter_counter(dev)
        invCell = np.ascontiguousarray(np.transpose(np.linalg.inv(self.lvec[1:4])), dtype=np.float64)
        prm = self._afm_params()
        W = np.ascontiguousarray(self.dfWeight, dtype=np.float64)
        o = self._out
        if out is not None:
            if tuple(out.shape) != (nx, ny, nout) or out.dtype != torch.float32 or not out.is_contiguous() or out.device != dev:
                raise ValueError(f"out must be a contiguous float32 tensor of shape {(nx, ny, nout)} on {dev}")
        Xt = o["X"] if out is None else out
        check(lib().ppgpu_relax_afm(tptr(ff.FE), iptr(ff.n), dptr(invCell), dptr(prm), npix, tptr(self._points), nz, tptr(o["FEs"]), tptr(o.get("paths")), tptr(o.get("iters")), nw, dptr(W), tptr(Xt), tptr(self.counter), stream_handle(stream)))
        if out is not None:
            return out
        Xd = o["X"].view(nx, ny, nout)
        if keep_device:
            return Xd
        Xh = Xd.cpu().numpy()
        if X is None:
            return Xh.copy()
        if X.shape != (nx, ny, nout):
            raise ValueError(f"Expected an array of shape {(nx, ny, nout)} for storing AFM image, but got an array of shape {X.shape} instead.")
        X[:, :, :] = Xh
        return X

    def eval(self, xyzs, Zs, qs, rho_sample=None, sample_lvec=None, rot=np.eye(3), rot_center=None, REAs=None, X=None, plot_to_dir=None):
        """Prepare and evaluate the AFM image stack (AFMulator.py:142-173)."""
        if plot_to_dir:
            raise NotImplementedError("plotting is not part of this library")
        t0 = time.perf_counter()
        self.prepareFF(xyzs, Zs, qs, rho_sample, sample_lvec, rot, rot_center, REAs)
        X = self.evalAFM(X)
        self.last_timing["eval"] = time.perf_counter() - t0
        return X

    def __call__(self, *args, **kwargs):
        return self.eval(*args, **kwargs)

    def downloadFF(self):
        """The force field as [nx, ny, nz, 4] float32 (Fx, Fy, Fz, E)."""
        return self._ff.grid4.cpu().numpy()
