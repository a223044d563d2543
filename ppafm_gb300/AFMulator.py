"""AFMulator with the reference's constructor and ``eval`` signature
(ppafm/ocl/AFMulator.py:83-173) on libppgpu: point-charge and Hartree force fields.

eval(xyzs, Zs, qs) builds the force field in HBM, relaxes every pixel column with the
tilted-stroke FIRE of relaxStrokesTilted (ppafm/ocl/cl/relax.cl:391-464) and applies the z
convolution (convolveZ, relax.cl:571-608) in the same kernel, returning the Δf stack
X [nx, ny, nz - df_steps + 1].  Interpolation uses exact float32 trilinear weights where the
reference samples an OpenCL image with hardware filtering.

Force fields:
  * point charges (qs an array): Lennard-Jones + tip point charges (evalLJC_QZs_noPos,
    ppafm/ocl/cl/FF.cl:366-423);
  * Hartree (qs a HartreePotential, a tip density set with ``rho``): the potential
    interpolated onto the force-field grid (interp_at), cross-correlated with the tip density
    (resampled onto the force-field grid when given on another) by FFT, differentiated by
    centred differences, plus Lennard-Jones (calc_force_hartree,
    ppafm/ocl/field.py:1446-1504);
  * Hartree without a tip density: the potential's electric field sampled at the tip point
    charges, plus Lennard-Jones (run_gradPotentialGrid + run_evalLJC_Hartree,
    field.py:1168-1317).

Not provided: FDBM (``rho_delta``, ``rho_sample``), plotting.
"""

import time

import numpy as np
import torch

from . import common
from ._lib import AFM_NPARAM, FF_QZS, check, dptr, iptr, lib, stream_handle, tptr
from .device import DeviceFF, iter_counter, pack_atoms
from .field import DataGrid, ElectronDensity, HartreePotential, MultipoleTipDensity, TipDensity  # noqa: F401  (the reference exports them here too)
from .fieldFFT import FFTGrid

FD_STEP = 0.05  # finite-difference step of the interpolated potential, A (field.py:27)
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
        if rho_delta is not None:
            raise NotImplementedError("tip delta densities (FDBM) are not supported")
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
        self.rho = None
        self._rho_dev = None
        self._rho_cache = {}
        self._rho_spectrum_of = None
        self._efield = None
        self._fft = None
        self._streams = None  # overlap mode (set_overlap): force-field and relaxation streams
        self.setScanWindow(scan_window, scan_dim, df_steps)
        self.setLvec(lvec, pixPerAngstrome)
        self.setQs(Qs, QZs)
        self.setRho(rho, sigma, B_pauli)
        self.last_timing = {}

    # ------------------------------------------------------------------ set-up

    def setLvec(self, lvec=None, pixPerAngstrome=None):
        if pixPerAngstrome is not None:
            self.pixPerAngstrome = pixPerAngstrome
        self.lvec = np.asarray(lvec, dtype=np.float64) if lvec is not None else get_lvec(self.scan_window, tipR0=self.tipR0, pixPerAngstrome=self.pixPerAngstrome)
        nDim = common.genFFSampling(self.lvec, pixPerAngstrome=self.pixPerAngstrome)
        if getattr(self, "nDim", None) is None or not np.array_equal(nDim, self.nDim) or not np.array_equal(self.lvec[1:], self._cell):
            self._ff = None
            self._rho_dev = None  # the tip density follows the force-field grid's shape
        elif self._ff is not None:  # same grid moved: keep its buffers
            self._ff.lvec = self.lvec.copy()
            self._ff.origin = self.lvec[0].copy()
        self.nDim = nDim
        self._cell = self.lvec[1:].copy()

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
        """Tip charge density for the Hartree route (AFMulator.py:243-288): a multipole dict
        (e.g. {"dz2": -0.1}) made on the force-field grid like MultipoleTipDensity, or a
        TipDensity (resampled about the origin onto the force-field grid when it is on
        another); None removes it."""
        if rho is not None and not isinstance(rho, (dict, TipDensity)):
            raise ValueError(f"rho should be a dict or a TipDensity, but got `{type(rho)}`")
        if not np.allclose(B_pauli, 1.0):
            raise NotImplementedError("density exponents other than 1 belong to FDBM, which is not supported")
        self.rho = rho
        self.sigma = sigma
        self.B_pauli = B_pauli
        self._rho_dev = None

    def setBPauli(self, B_pauli=1.0):
        """Pauli density exponent (AFMulator.py:286-288): only 1 here (other exponents belong
        to FDBM)."""
        self.setRho(self.rho, sigma=self.sigma, B_pauli=B_pauli)

    def setRhoDelta(self, rho_delta=None):
        """FDBM tip delta density (AFMulator.py:290-307): not supported; None is accepted."""
        if rho_delta is not None:
            raise NotImplementedError("tip delta densities (FDBM) are not supported")

    def _tip_density(self):
        """The tip density on the force-field grid (device, cached)."""
        if self._rho_dev is not None:
            return self._rho_dev
        n = tuple(int(x) for x in self.nDim)
        if self._fft is None or tuple(self._fft.n) != n:
            self._fft = FFTGrid(n)
            self._rho_cache = {}
            self._rho_spectrum_of = None
        # one device density per tip and grid shape (a generator alternates between tips)
        tag = ("dict", tuple(sorted(self.rho.items()))) if isinstance(self.rho, dict) else ("grid", id(self.rho))
        key = (tag, float(self.sigma), self.lvec[1:4].tobytes())
        hit = self._rho_cache.get(key)
        if hit is not None and (tag[0] == "dict" or hit[0] is self.rho):
            self._rho_dev = hit[1]
            return self._rho_dev
        if isinstance(self.rho, dict):
            # MultipoleTipDensity (field.py:653-700): getProbeDensity on coordinates wrapped
            # around the grid origin
            self._rho_dev = self._fft.probe_density(np.vstack([np.zeros(3), self.lvec[1:4]]), self.sigma, self.rho)
        elif tuple(self.rho.shape) == n and np.allclose(self.rho.lvec[1:], self.lvec[1:]):
            self._rho_dev = self.rho.device()
        else:
            # another grid: resampled about the origin onto the force-field grid
            # (prepareBuffers, field.py:957-962 -> TipDensity.interp_at)
            self._rho_dev = self.rho.interp_at(self.lvec, n).device()
        if len(self._rho_cache) >= 8:
            self._rho_cache.pop(next(iter(self._rho_cache)))
        self._rho_cache[key] = (self.rho, self._rho_dev)
        return self._rho_dev

    def _hartree_ff(self, pot, atoms_rec, na, rot, rot_center, stream=None):
        """calc_force_hartree (field.py:1446-1504) on the force-field grid: the potential
        interpolated onto it (rotated by the inverse of the atoms' rotation), cross-correlated
        with the tip density, F = -grad E by centred differences, then + Lennard-Jones."""
        if self.rho is None:
            if not np.allclose(rot, np.eye(3)):
                raise NotImplementedError("Force field calculation with rotation for Hartree potential with point charges tip density is not implemented.")
            return self._hartree_ff_point_charges(pot, atoms_rec, na, stream=stream)
        lv = self.lvec
        if (np.abs(lv[1:4] - np.diag(np.diag(lv[1:4]))) > 0).any():
            raise NotImplementedError("Forcefield calculation via FFT for non-rectangular grids is not implemented.")
        rho = self._tip_density()
        n = np.array(self.nDim, dtype=np.int32)
        step_out = np.ascontiguousarray(lv[1:4] / n[:, None], dtype=np.float64)
        pot_i = self._fft.empty()
        rot_ff = np.ascontiguousarray(np.linalg.inv(rot), dtype=np.float64)
        check(lib().ppgpu_interp_grid(tptr(pot.device()), iptr(np.array(pot.shape, dtype=np.int32)), dptr(np.ascontiguousarray(pot.origin, dtype=np.float64)),
                                      dptr(np.ascontiguousarray(pot.step, dtype=np.float64)), tptr(pot_i), iptr(n), dptr(np.ascontiguousarray(lv[0], dtype=np.float64)),
                                      dptr(step_out), dptr(rot_ff), dptr(np.ascontiguousarray(rot_center, dtype=np.float64)), stream_handle(stream)))
        vox = abs(np.linalg.det(step_out))
        fresh = self._rho_spectrum_of is not rho  # the tip's spectrum is transformed once
        E = self._fft.correlate(pot_i, rho if fresh else None, scale=vox, stream=stream)
        self._rho_spectrum_of = rho
        if self._ff is None:
            self._ff = DeviceFF(self.nDim, self.lvec)
        check(lib().ppgpu_grad_fd(tptr(E), iptr(n), dptr(np.ascontiguousarray(np.diag(step_out))), dptr(np.array([-1.0, -1.0, -1.0, 1.0])), tptr(self._ff.FE), 0, stream_handle(stream)))
        zero4 = np.zeros(4)
        self._ff.compute(atoms_rec, na, 0, FF_QZS, Qs=zero4, QZs=zero4, with_E=True, accumulate=True, stream=stream)
        return self._ff

    def _hartree_ff_point_charges(self, pot, atoms_rec, na, stream=None):
        """The Hartree route with the point-charge tip (field.py:1168-1317, makeFF :1716-1720):
        the electric field on the force-field grid -- periodic centred differences of the
        potential where the two grids coincide, else of the potential interpolated at +-h
        (h = 0.05 A) -- then Lennard-Jones plus the tip charges Qs at heights QZs in that field."""
        lv = self.lvec
        n = np.array(self.nDim, dtype=np.int32)
        step_out = np.ascontiguousarray(lv[1:4] / n[:, None], dtype=np.float64)
        pstep = np.ascontiguousarray(pot.step, dtype=np.float64)
        matching = (
            tuple(pot.shape) == tuple(n)
            and (np.abs(pot.origin - lv[0]) < 1e-3).all()
            and (np.abs(np.diag(pstep) * np.array(pot.shape) - np.diag(lv[1:4])) < 1e-3).all()
            and (pstep == np.diag(np.diag(pstep))).all()
        )
        if self._efield is None or tuple(self._efield.shape[:3]) != tuple(n):
            self._efield = torch.empty(tuple(int(x) for x in n) + (4,), dtype=torch.float32, device="cuda")
        if matching:
            check(lib().ppgpu_grad_fd(tptr(pot.device()), iptr(n), dptr(np.ascontiguousarray(np.diag(pstep))), dptr(np.array([-1.0, -1.0, -1.0, 1.0])), tptr(self._efield), 0, stream_handle(stream)))
        else:
            check(lib().ppgpu_grad_potential_grid(tptr(pot.device()), iptr(np.array(pot.shape, dtype=np.int32)), dptr(np.ascontiguousarray(pot.origin, dtype=np.float64)), dptr(pstep),
                                                  tptr(self._efield), iptr(n), dptr(np.ascontiguousarray(lv[0], dtype=np.float64)), dptr(step_out), dptr(np.full(3, FD_STEP)), stream_handle(stream)))
        if self._ff is None:
            self._ff = DeviceFF(self.nDim, self.lvec)
        zero4 = np.zeros(4)
        self._ff.compute(atoms_rec, na, 0, FF_QZS, Qs=zero4, QZs=zero4, with_E=True, stream=stream)
        check(lib().ppgpu_tip_charges_field(tptr(self._efield), iptr(n), dptr(np.ascontiguousarray(lv[0], dtype=np.float64)), dptr(step_out),
                                            dptr(self.Qs.astype(np.float64)), dptr(self.QZs.astype(np.float64)), tptr(self._ff.FE), 1, stream_handle(stream)))
        return self._ff

    # --------------------------------------------------------------- imaging

    # ------------------------------------------------------------------ overlap mode

    def set_overlap(self, on=True):
        """Overlap mode, for callers that queue many images (the ML generators): each image's
        force field goes to one of two device grids on a force-field stream, and its relaxation
        runs on a stream of higher priority after it, so that image k+1's force field runs
        beside image k's relaxation.  The results are those of the plain mode; what evalAFM
        writes into ``out`` is ready on the current stream after ``join()`` (evalAFM without
        ``out`` joins by itself).  Off: joins and returns to the current stream."""
        if not on:
            self.join()
            self._streams = None
            return
        if self._streams is None:
            _, high = torch.cuda.Stream.priority_range()
            self._streams = (torch.cuda.Stream(), torch.cuda.Stream(priority=high))
            self._slots = [None, None]  # the two force-field grids
            self._ff_done = [None, None]  # force field of slot k written
            self._rx_done = [None, None]  # relaxation that last read slot k finished
            self._slot = 1

    def join(self):
        """The current stream waits for the force fields and relaxations queued in overlap mode."""
        if self._streams is not None:
            cur = torch.cuda.current_stream()
            cur.wait_stream(self._streams[0])
            cur.wait_stream(self._streams[1])

    def prepareFF(self, xyzs, Zs, qs, rho_sample=None, sample_lvec=None, rot=np.eye(3), rot_center=None, REAs=None, stream=None):
        """Point-charge force field on the device (AFMulator.py:321-429, field.py:1608-1713)."""
        if self._streams is None or stream is not None:
            return self._prepare_ff(xyzs, Zs, qs, rho_sample, sample_lvec, rot, rot_center, REAs, stream)
        s_ff = self._streams[0]
        self._slot ^= 1
        k = self._slot
        s_ff.wait_stream(torch.cuda.current_stream())
        if self._rx_done[k] is not None:
            s_ff.wait_event(self._rx_done[k])  # the relaxation that read this grid has finished
        g = self._slots[k]
        with torch.cuda.stream(s_ff):
            if g is None or not np.array_equal(g.n, self.nDim) or not np.array_equal(g.cell, self.lvec[1:4]):
                g = DeviceFF(self.nDim, self.lvec)
                self._slots[k] = g
            else:
                g.lvec = self.lvec.copy()
                g.origin = self.lvec[0].copy()
            self._ff = g
            out = self._prepare_ff(xyzs, Zs, qs, rho_sample, sample_lvec, rot, rot_center, REAs, s_ff)
            self._ff_done[k] = torch.cuda.Event()
            self._ff_done[k].record(s_ff)
        return out

    def _prepare_ff(self, xyzs, Zs, qs, rho_sample, sample_lvec, rot, rot_center, REAs, stream):
        if rho_sample is not None:
            raise NotImplementedError("FDBM (rho_sample) is not supported")
        pot = None
        if isinstance(qs, HartreePotential):
            pot = qs
            qs = np.zeros(len(Zs))
            self.sample_lvec = np.asarray(sample_lvec) if sample_lvec is not None else pot.lvec[1:]
        elif qs is not None and not isinstance(qs, np.ndarray):
            qs = np.asarray(qs)
        if qs is None:
            qs = np.zeros(len(Zs))
        if sample_lvec is not None and pot is None:
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
        rec, na, nch = pack_atoms(R, c32.astype(np.float64), atoms32[:, 3].astype(np.float64), stream=stream)
        self._atoms = rec
        if pot is not None:
            return self._hartree_ff(pot, rec, na, np.asarray(rot, dtype=np.float64), np.asarray(rot_center, dtype=np.float64), stream=stream)
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
        image (returned as is, nothing is copied to the host; in overlap mode ready on the
        current stream after join())."""
        if self._streams is None or stream is not None:
            return self._eval_afm(X, stream, keep_device, want_paths, want_iters, out)
        s_rx = self._streams[1]
        k = self._slot
        s_rx.wait_stream(torch.cuda.current_stream())
        if self._ff_done[k] is not None:
            s_rx.wait_event(self._ff_done[k])
        with torch.cuda.stream(s_rx):
            res = self._eval_afm(X, s_rx, True if out is None else keep_device, want_paths, want_iters, out)
            self._rx_done[k] = torch.cuda.Event()
            self._rx_done[k].record(s_rx)
        if out is not None:
            return res
        self.join()
        return self._host_image(res, X, keep_device)

    def _host_image(self, Xd, X, keep_device):
        if keep_device:
            return Xd
        Xh = Xd.cpu().numpy()
        if X is None:
            return Xh.copy()
        if X.shape != Xd.shape:
            raise ValueError(f"Expected an array of shape {tuple(Xd.shape)} for storing AFM image, but got an array of shape {X.shape} instead.")
        X[:, :, :] = Xh
        return X

    def _eval_afm(self, X, stream, keep_device, want_paths, want_iters, out):
        ff = self._ff
        nx, ny, nz = self.scan_dim
        npix = nx * ny
        nw = len(self.dfWeight)
        nout = nz - nw + 1
        dev = ff.FE.device
        if self._out is None or self._out["X"].shape != (npix, nout) or self._out["FEs"].shape[1] != nz:
            self._out = dict(FEs=torch.empty((npix, nz, 4), dtype=torch.float32, device=dev), X=torch.empty((npix, nout), dtype=torch.float32, device=dev))
        key = (tuple(map(tuple, self.scan_window)), tuple(self.scan_dim), tuple(self.lvec[0]))
        if getattr(self, "_points_key", None) != key:
            # tip positions of this scan window: packed in pinned memory and copied without a
            # synchronisation, so a generator's next image is prepared while the GPU works
            pts = torch.from_numpy(self._scan_points().reshape(-1, 4)).pin_memory()
            if stream is None:
                self._points = pts.to(dev, non_blocking=True)
            else:
                with torch.cuda.stream(stream):
                    self._points = pts.to(dev, non_blocking=True)
            self._points_key = key
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
        return self._host_image(o["X"].view(nx, ny, nout), X, keep_device)

    def eval(self, xyzs, Zs, qs, rho_sample=None, sample_lvec=None, rot=np.eye(3), rot_center=None, REAs=None, X=None, plot_to_dir=None):
        """Prepare and evaluate the AFM image stack (AFMulator.py:142-173).  plot_to_dir: the
        reference plots the images there; this library has no plotting and saves the stack as
        ``df.npy`` in that directory instead (with a warning)."""
        t0 = time.perf_counter()
        self.prepareFF(xyzs, Zs, qs, rho_sample, sample_lvec, rot, rot_center, REAs)
        X = self.evalAFM(X)
        self.last_timing["eval"] = time.perf_counter() - t0
        if plot_to_dir:
            import os
            import warnings

            os.makedirs(plot_to_dir, exist_ok=True)
            np.save(os.path.join(plot_to_dir, "df.npy"), X)
            warnings.warn(f"plotting is not part of this library; the df stack is saved as {os.path.join(plot_to_dir, 'df.npy')}")
        return X

    def __call__(self, *args, **kwargs):
        return self.eval(*args, **kwargs)

    def eval_(self, mol):
        """eval of an object with xyzs, Zs and qs attributes (AFMulator.py:181-182)."""
        return self.eval(mol.xyzs, mol.Zs, mol.qs)

    def downloadFF(self):
        """The force field as [nx, ny, nz, 4] float32 (Fx, Fy, Fz, E)."""
        self.join()
        return self._ff.grid4.cpu().numpy()

    def plot_images(self, X, outdir="afm_images", prefix="df", **plot_kwargs):
        """The reference plots the Δf stack into outdir (AFMulator.py:609-640); this library has
        no plotting and saves it as <prefix>.npz there instead (X with heights top-down, the tip
        heights at mid-oscillation and the image extent, as the plots are labelled), with a
        warning."""
        import os
        import warnings

        os.makedirs(outdir, exist_ok=True)
        zTips = np.linspace(self.scan_window[0][2], self.scan_window[1][2] - self.df_steps * self.dz, self.scan_dim[2] - self.df_steps + 1) + self.amplitude / 2
        extent = [self.scan_window[0][0], self.scan_window[1][0], self.scan_window[0][1], self.scan_window[1][1]]
        path = os.path.join(outdir, f"{prefix}.npz")
        np.savez(path, X=np.asarray(X)[:, :, ::-1], zTips=zTips, extent=np.array(extent))
        warnings.warn(f"plotting is not part of this library; the images are saved as {path}")

    # ------------------------------------------------------------ parameter files

    @classmethod
    def from_params(cls, file_path="./params.ini"):
        """An AFMulator configured from a params.ini (or .toml) file (AFMulator.py:483-494)."""
        parameters, sample_lvec = _get_params(file_path)
        afm = cls(**parameters)
        afm.sample_lvec = sample_lvec
        return afm

    def load_params(self, file_path="./params.ini"):
        """Updates this AFMulator from a parameter file (AFMulator.py:496-520)."""
        parameters, sample_lvec = _get_params(file_path)
        if parameters["tipStiffness"] is not None:
            self.setStiffness(parameters["tipStiffness"])
        self.iZPP = parameters["iZPP"]
        self.tipR0 = np.array(parameters["tipR0"], dtype=np.float64)
        self.f0Cantilever = parameters["f0Cantilever"]
        self.kCantilever = parameters["kCantilever"]
        self.npbc = parameters["npbc"]
        self.A_pauli = parameters["A_pauli"]
        self.setScanWindow(parameters["scan_window"], parameters["scan_dim"], parameters["df_steps"])
        self.setLvec(parameters["lvec"], parameters["pixPerAngstrome"])
        if self.rho is None or isinstance(self.rho, dict):
            self.setRho(parameters["rho"], parameters["sigma"])
        else:
            import warnings

            warnings.warn(f'Using existing tip density with exponent {parameters["B_pauli"]}, instead of parameters from params.ini file.')
            self.setRho(self.rho, sigma=parameters["sigma"], B_pauli=parameters["B_pauli"])
        self.sample_lvec = sample_lvec
        self.colorscale = parameters["colorscale"]

    def save_params(self, file_path="./params.ini"):
        """Writes this AFMulator's parameters as a params.ini file (AFMulator.py:522-565)."""
        import warnings

        k = self.stiffness * -common.eVA_Nm
        scan_step = (
            (self.scan_window[1][0] - self.scan_window[0][0]) / (self.scan_dim[0] - 1),
            (self.scan_window[1][1] - self.scan_window[0][1]) / (self.scan_dim[1] - 1),
            (self.scan_window[1][2] - self.scan_window[0][2]) / self.scan_dim[2],
        )
        with open(file_path, "w") as f:
            f.write(f"probeType {self.iZPP}\n")
            if isinstance(self.rho, dict):
                if len(self.rho) > 1:
                    warnings.warn("More than one tip multipole type specified. Only writing the first one into params.ini.")
                tip = list(self.rho)[0]
                f.write(f"tip {tip}\n")
                f.write(f"charge {self.rho[tip]}\n")
                f.write(f"sigma {self.sigma}\n")
            f.write(f"stiffness {k[0]} {k[1]} {k[3]}\n")
            f.write(f"r0Probe {self.tipR0[0]} {self.tipR0[1]} {self.tipR0[2]}\n")
            f.write(f"PBC {(np.array(self.npbc) > 0).any()}\n")
            f.write(f"nPBC {self.npbc[0]} {self.npbc[1]} {self.npbc[2]}\n")
            if self.sample_lvec is not None:
                sl = np.asarray(self.sample_lvec)
                for name, row in zip(("gridA", "gridB", "gridC"), sl):
                    f.write(f"{name} {row[0]} {row[1]} {row[2]}\n")
            for name, row in zip(("FFgrid0", "FFgridA", "FFgridB", "FFgridC"), self.lvec):
                f.write(f"{name} {row[0]} {row[1]} {row[2]}\n")
            f.write(f"gridN {self.nDim[0]} {self.nDim[1]} {self.nDim[2]}\n")
            f.write(f"scanMin {self.scan_window[0][0]} {self.scan_window[0][1]} {self.scan_window[0][2]}\n")
            f.write(f"scanMax {self.scan_window[1][0]} {self.scan_window[1][1]} {self.scan_window[1][2]}\n")
            f.write(f"scanStep {scan_step[0]} {scan_step[1]} {scan_step[2]}\n")
            f.write(f"kCantilever {self.kCantilever}\n")
            f.write(f"f0Cantilever {self.f0Cantilever}\n")
            f.write(f"Amplitude {self.amplitude}\n")
            f.write(f"Apauli {self.A_pauli}\n")
            f.write(f"Bpauli {self.B_pauli}\n")

    # ------------------------------------------------------------ debugging aids

    def saveFF(self, prefix="./"):
        """The force field's components, |F| clamped to 10 eV/A, as XSF files FF_x/y/z.xsf
        (AFMulator.py:569-583)."""
        FF = self.downloadFF()
        F = FF[..., :3].astype(np.float64)
        Fr = np.sqrt((F**2).sum(axis=-1))
        k = np.where(Fr > 10.0, 10.0 / np.where(Fr > 0, Fr, 1.0), 1.0)
        for c, name in enumerate("xyz"):
            self.saveDebugXSF_FF(f"{prefix}FF_{name}.xsf", F[..., c] * k)

    def saveDebugXSF_FF(self, fname, F):
        from . import io

        io.saveXSFData(fname, F, self.lvec)

    def check_scan_window(self):
        """Warns when the scan window comes within 0.3 A of a non-periodic edge of the
        force-field grid (AFMulator.py:589-607)."""
        import warnings

        for i, dim in enumerate("xyz"):
            if self.npbc[i]:
                continue
            lo = self.lvec[0, i]
            hi = lo + self.lvec[i + 1, i]
            s0 = self.scan_window[0][i] - 0.3
            s1 = self.scan_window[1][i] + 0.3
            if i == 2:
                s0 -= self.tipR0[2]
                s1 -= self.tipR0[2]
            if s0 < lo or s1 > hi:
                warnings.warn(
                    f"The edge of the scan window in {dim} dimension is very close or extends over the boundary of the force-field grid "
                    f"which is not periodic in {dim} dimension. If you get artifacts in the images, please check the boundary conditions "
                    "and the size of the scan window and the force field grid."
                )


def _get_params(file_path):
    """AFMulator arguments from a parameter file (AFMulator.py:642-699).  A file with PBC False
    gives npbc (0, 0, 0)."""
    import warnings

    from .species import SYMBOL_TO_Z

    p = common.PpafmParameters.from_file(file_path)
    lvec = np.array([p.FFgrid0, p.FFgridA, p.FFgridB, p.FFgridC], dtype=np.float64)
    if (lvec < 0).any():
        lvec = None
    sample_lvec = np.array([p.gridA, p.gridB, p.gridC], dtype=np.float64)
    if (np.array(p.gridN) == 0).any() or lvec is None:
        pix = 10
    else:
        rx, ry, rz = (round(p.gridN[i] / np.linalg.norm(lvec[i + 1])) for i in range(3))
        if np.allclose([rx, ry], rz):
            pix = rx
        else:
            pix = int(np.max([rx, ry, rz]))
            warnings.warn(f"Unequal grid densities in x, y, z directions is not supported by the AFMulator. Using the maximum of x, y, z directions, {pix}, for grid point density.")
    scan_window = (tuple(p.scanMin), tuple(p.scanMax))
    scan_dim = (
        round((scan_window[1][0] - scan_window[0][0]) / p.scanStep[0]) + 1,
        round((scan_window[1][1] - scan_window[0][1]) / p.scanStep[1]) + 1,
        round((scan_window[1][2] - scan_window[0][2]) / p.scanStep[2]),
    )
    iZPP = SYMBOL_TO_Z[p.probeType] if p.probeType in SYMBOL_TO_Z else int(p.probeType)
    stiff = p.stiffness
    stiff = [0.25, 0.25, 0.0, 30.0] if (np.array(stiff) < 0).any() else list(np.insert(np.array(stiff, dtype=np.float64), 2, 0.0))
    params = dict(
        lvec=lvec, pixPerAngstrome=pix, scan_dim=scan_dim, scan_window=scan_window, iZPP=iZPP, rho={p.tip: p.charge}, sigma=p.sigma,
        A_pauli=p.Apauli, B_pauli=p.Bpauli, df_steps=round(p.Amplitude / p.scanStep[2]), tipR0=p.r0Probe, tipStiffness=stiff,
        npbc=tuple(p.nPBC) if p.PBC else (0, 0, 0), f0Cantilever=p.f0Cantilever, kCantilever=p.kCantilever, colorscale=p.colorscale,
    )
    return params, sample_lvec
