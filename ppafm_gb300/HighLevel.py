"""High-level hot-path drivers, mirroring ppafm/HighLevel.py on the GPU.

* ``setFF``, ``relaxedScan3D_omp``, ``perform_relaxation``: the reference's functions with
  the same arguments and return values (host numpy in/out), run through the device path.
* ``computeLJ_atoms`` / ``computeELFF_pointCharge_atoms``: ``computeLJ`` /
  ``computeELFF_pointCharge`` (HighLevel.py:260-387) from in-memory atoms instead of
  geometry files (file I/O is outside this library).
* ``relaxed_scan_pipeline``: the whole CPU pipeline of the reference -- LJ grid, point-charge
  grid, clamps, FF = FFLJ + Q*FFel, relaxed scan, Fz -> Δf -- as one device-resident pass
  with no host copy of the force field.
* ``DensityOverlapPipeline``: the full-density route -- Pauli force from the density
  overlap (cli/conv_rho.py:24-88), electrostatics from a Hartree potential correlated with
  the tip density (computeElFF, HighLevel.py:390-411), relaxed scan, Δf -- on the GPU.
"""

import contextlib

import numpy as np
import torch

from . import common as PPU
from . import core
from .device import DeviceFF, iter_counter, pack_atoms, relax_params, relax_scan, relax_strokes, upload_f64
from .device import tip_spline as tip_spline_ctx
from .fieldFFT import FFTGrid
from ._lib import FF_COULOMB, FF_LJ, FF_LJC

Fmax_DEFAULT = 10.0  # HighLevel.py:17
Vmax_DEFAULT = 10.0
TIP_KINDS = {"s": 0, "pz": 1, "dz2": 2}


def _get(p, name, default=None):
    if p is None:
        return default
    if isinstance(p, dict):
        return p.get(name, default)
    return getattr(p, name, default)


# ------------------------------------------------------------ reference mirrors


def setFF(FF=None, computeVpot=False, n=None, lvec=None, parameters=None):
    """HighLevel.py:190-257: registers (or allocates) the host force field with the core."""
    if FF is not None:
        gridN = np.array(np.shape(FF)[0:3], dtype=np.int32)
    else:
        if n is not None:
            gridN = np.array(n, dtype=np.int32)
        elif parameters is not None:
            gridN = np.array(_get(parameters, "gridN"), dtype=np.int32)
        else:
            raise ValueError("FF dimensions not set !!")
        FF = np.zeros((gridN[0], gridN[1], gridN[2], 3))
    core.setGridN(gridN)
    if FF.ndim == 4 and FF.shape[-1] == 3:
        core.setFF_Fpointer(FF)
    elif FF.ndim == 3 or FF.shape[-1] == 1:
        core.setFF_Epointer(FF)
        computeVpot = False
    else:
        raise ValueError("setFF: Array dimensions wrong for both vector and array field !!")
    V = None
    if computeVpot:
        V = np.zeros((gridN[0], gridN[1], gridN[2]))
        core.setFF_Epointer(V)
    if lvec is None and parameters is not None:
        lvec = np.array([_get(parameters, "gridA"), _get(parameters, "gridB"), _get(parameters, "gridC")], dtype=np.float64)
    lvec = np.array(lvec, dtype=np.float64)
    if lvec.shape == (4, 3):
        lvec = lvec[1:, :].copy()
    elif lvec.shape != (3, 3):
        raise ValueError("lvec matrix has a wrong format !!")
    core.setGridCell(lvec)
    return FF, V


def trjByDir(n, d, p0):
    """Tip trajectory of a tilted scan (HighLevel.py:36-41): n points from p0 along d, in
    approach order."""
    trj = np.zeros((n, 3))
    for k in range(3):
        trj[:, k] = p0[k] + (np.arange(n)[::-1]) * d[k]
    return trj


def relaxedScan3D(xTips, yTips, zTips, trj=None, bF3d=False, tip_spline=None):
    """HighLevel.py:63-101 (one relaxTipStroke per pixel) as one batched stroke relaxation:
    pixel (x, y) follows trj + (x, y, 0), trj defaulting to the straight approach over zTips."""
    nx, ny, nz = len(xTips), len(yTips), len(zTips)
    if trj is None:
        trj = np.zeros((nz, 3))
        trj[:, 2] = zTips[::-1]
    trj = np.asarray(trj, dtype=np.float64)
    rTips = np.zeros((nx, ny, len(trj), 3))
    rTips[:, :, :, 0] = trj[None, None, :, 0] + np.asarray(xTips)[:, None, None]
    rTips[:, :, :, 1] = trj[None, None, :, 1] + np.asarray(yTips)[None, :, None]
    rTips[:, :, :, 2] = trj[None, None, :, 2]
    rs = np.zeros_like(rTips)
    fs = np.zeros_like(rTips)
    core.relaxTipStrokes_omp(rTips, rs, fs, tip_spline=tip_spline)
    PPpos = rs[:, :, ::-1, :].copy()
    fzs = fs[:, :, ::-1, :].copy() if bF3d else fs[:, :, ::-1, 2].transpose(2, 1, 0).copy()
    return fzs, PPpos


def relaxedScan3D_omp(xTips, yTips, zTips, trj=None, bF3d=False, tip_spline=None):
    """HighLevel.py:104-124 through the drop-in core (FF registered with setFF).  Like the
    reference, the trajectory argument is accepted and not used: the tips approach straight
    down over zTips."""
    nx, ny, nz = len(xTips), len(yTips), len(zTips)
    rTips = np.zeros((nx, ny, nz, 3))
    rTips[:, :, :, 0] = xTips[:, None, None]
    rTips[:, :, :, 1] = yTips[None, :, None]
    rTips[:, :, :, 2] = zTips[::-1][None, None, :]
    rs = np.zeros((nx, ny, nz, 3))
    fs = np.zeros((nx, ny, nz, 3))
    core.relaxTipStrokes_omp(rTips, rs, fs, tip_spline=tip_spline)
    rs = rs[:, :, ::-1, :].copy()
    fzs = fs[:, :, ::-1, :].copy() if bF3d else fs[:, :, ::-1, 2].copy()
    return fzs, rs


def tip_vector(parameters, relax=None):
    """setTip/setRelax state of perform_relaxation (HighLevel.py:157-160) as the
    parameter vector of the device relax kernels."""
    stiff = np.array(_get(parameters, "stiffness", [-1.0, -1.0, -1.0]), dtype=np.float64)
    if (stiff < 0.0).any():
        stiff = np.array([_get(parameters, "klat"), _get(parameters, "klat"), _get(parameters, "krad")], dtype=np.float64)
    r0 = _get(parameters, "r0Probe")
    relax = relax or {}
    return relax_params(
        maxIters=relax.get("maxIters", _get(parameters, "maxIters", 1000)),
        convF2=relax.get("convF2", _get(parameters, "convF2", 1e-8)),
        dt=relax.get("dt", _get(parameters, "dt", 0.1)),
        damping=relax.get("damping", _get(parameters, "damping", 0.1)),
        lRadial=r0[2],
        kRadial=stiff[2] / -PPU.eVA_Nm,
        rPP0=(r0[0], r0[1], 0.0),
        kSpring=np.array((stiff[0], stiff[1], 0.0)) / -PPU.eVA_Nm,
    )


def perform_relaxation(lvec, FFLJ, FFel=None, FFpauli=None, FFboltz=None, FFkpfm_t0sV=None, FFkpfm_tVs0=None, tip_spline=None, bPPdisp=False, bFFtotDebug=False, parameters=None, relax=None):
    """HighLevel.py:127-184 on the GPU: FF = FFLJ + Q*FFel (+ Pauli, Boltzmann, KPFM
    terms) composed on the host like the reference, then one device relaxed scan.
    ``relax`` optionally overrides maxIters/convF2/dt/damping (the reference reads the
    core's global setRelax state)."""
    tilted = bool(_get(parameters, "tiltedScan", False))
    lvec = np.asarray(lvec, dtype=np.float64)
    xTips, yTips, zTips, lvecScan = PPU.prepareScanGrids(_get(parameters, "scanMin"), _get(parameters, "scanMax"), _get(parameters, "scanStep"), _get(parameters, "r0Probe"))
    FF = FFLJ.copy()
    if FFel is not None:
        FF += FFel * _get(parameters, "charge")
    if FFkpfm_t0sV is not None and FFkpfm_tVs0 is not None:
        FF += (_get(parameters, "charge") * FFkpfm_t0sV - FFkpfm_tVs0) * _get(parameters, "Vbias", 0.0)
    if FFpauli is not None:
        FF += FFpauli * _get(parameters, "Apauli")
    if FFboltz is not None:
        FF += FFboltz
    if bFFtotDebug:
        from . import io

        io.save_vec_field("FFtotDebug", FF, lvec)
    ff = DeviceFF(FF.shape[:3], lvec).from_host_f64(FF.reshape(-1, 3))
    prm = tip_vector(parameters, relax)
    with tip_spline_ctx(tip_spline):
        return _relax_and_collect(ff, prm, lvec, xTips, yTips, zTips, lvecScan, tilted, bPPdisp, parameters)


def _relax_and_collect(ff, prm, lvec, xTips, yTips, zTips, lvecScan, tilted, bPPdisp, parameters):
    if tilted:
        # the reference builds the tilted trajectory and passes it to relaxedScan3D_omp,
        # which does not use it (HighLevel.py:164-167, 104-124): the tips approach straight
        # down and the full force vector is kept for Fz2df_tilt
        rTips = np.zeros((len(xTips), len(yTips), len(zTips), 3))
        rTips[..., 0] = (xTips - lvec[0, 0])[:, None, None]
        rTips[..., 1] = (yTips - lvec[0, 1])[None, :, None]
        rTips[..., 2] = (zTips[::-1] - lvec[0, 2])[None, None, :]
        rs, fs, _, _ = relax_strokes(ff, prm, rTips)
        fzs = fs.flip(2).cpu().numpy()
        PPpos = rs.flip(2).cpu().numpy() + lvec[0]
    else:
        out = relax_scan(ff, prm, xTips - lvec[0, 0], yTips - lvec[0, 1], zTips[::-1] - lvec[0, 2], pos_offset=lvec[0])
        fzs = out["fzs"].cpu().numpy().astype(np.float64)
        PPpos = out["ppos"].cpu().numpy().astype(np.float64)
    PPdisp = None
    if bPPdisp:
        r0 = _get(parameters, "r0Probe")
        init_pos = np.array(np.meshgrid(xTips, yTips, zTips)).transpose(3, 1, 2, 0) + np.array([r0[0], r0[1], -r0[2]])
        PPdisp = PPpos - init_pos
    return fzs, PPpos, PPdisp, lvecScan


# ----------------------------------------------------------------- atom input


_SPECIES = None


def _default_species():
    """The built-in species table and its symbol index, made once (read only here)."""
    global _SPECIES
    if _SPECIES is None:
        table = PPU.loadSpecies()
        _SPECIES = (table, PPU.getFFdict(table))
    return _SPECIES


def prepare_atoms(Zs, Rs, Qs, lvec, parameters, FFparams=None):
    """parseAtoms + getAtomsLJ + origin shift (common.py:828-868, HighLevel.py:269-277):
    returns (Rs0 relative to the grid origin, cLJs, kQQs) after in-plane PBC replication."""
    lvec = np.asarray(lvec, dtype=np.float64)
    if FFparams is None:
        FFparams, elem_dict = _default_species()
    else:
        elem_dict = PPU.getFFdict(FFparams)
    iZs = np.asarray(Zs, dtype=np.int32)
    Rs = np.asarray(Rs, dtype=np.float64)
    Qs = np.asarray(Qs, dtype=np.float64)
    if _get(parameters, "PBC", True):
        nP = _get(parameters, "nPBC", (1, 1, 1))
        iZs, Rs, Qs = PPU.PBCAtoms(iZs, Rs, Qs, lvec[1], lvec[2], na=nP[0], nb=nP[1])
    iPP = PPU.atom2iZ(_get(parameters, "probeType", "O"), elem_dict)
    cLJs = PPU.getAtomsLJ(iPP, iZs, FFparams)
    return Rs - lvec[0], cLJs, Qs * PPU.CoulombConst


def computeLJ_atoms(Zs, Rs, lvec, gridN, parameters, Fmax=Fmax_DEFAULT, computeVpot=False, FFparams=None, device=False):
    """computeLJ (HighLevel.py:260-307) from in-memory atoms; returns (FF, V) float64 host
    arrays (or the DeviceFF when device=True)."""
    Rs0, cLJs, _ = prepare_atoms(Zs, Rs, np.zeros(len(Zs)), lvec, parameters, FFparams)
    atoms, na, _ = pack_atoms(Rs0, cLJs, None)
    ff = DeviceFF(gridN, lvec).compute(atoms, na, 0, FF_LJ, with_E=computeVpot)
    if Fmax is not None:
        ff.clamp(Fmax)
    if device:
        return ff
    F, E = ff.to_host()
    V = None
    if computeVpot:
        V = E
        if Vmax_DEFAULT is not None:
            V[V > Vmax_DEFAULT] = Vmax_DEFAULT
    return F, V


def computeELFF_pointCharge_atoms(Zs, Rs, Qs, lvec, gridN, parameters, tip="s", Fmax=Fmax_DEFAULT, computeVpot=False, device=False):
    """computeELFF_pointCharge (HighLevel.py:353-387) from in-memory atoms."""
    Rs0, _, kqq = prepare_atoms(Zs, Rs, Qs, lvec, parameters)
    atoms, na, nch = pack_atoms(Rs0, None, kqq)
    ff = DeviceFF(gridN, lvec).compute(atoms, na, nch, FF_COULOMB, kind=TIP_KINDS[tip], with_E=computeVpot)
    if Fmax is not None:
        ff.clamp(Fmax)
    if device:
        return ff
    F, E = ff.to_host()
    V = None
    if computeVpot:
        V = E
        if Vmax_DEFAULT is not None:
            V[V > Vmax_DEFAULT] = Vmax_DEFAULT
    return F, V


# ------------------------------------------------------ file-based stage functions


def _load_stage_geometry(geomFile, geometry_format, parameters, FFparams):
    from . import io

    elem_dict = PPU.getFFdict(FFparams)
    atoms, nDim, lvec = io.loadGeometry(geomFile, format=geometry_format, parameters=parameters)
    head = io.primcoords2Xsf(PPU.atoms2iZs(atoms[0], elem_dict), [atoms[1], atoms[2], atoms[3]], lvec)
    iZs, Rs, Qs = PPU.parseAtoms(atoms, elem_dict, autogeom=False, PBC=parameters.PBC, lvec=lvec, parameters=parameters)
    n = PPU.autoGridN(parameters) if parameters.gridN[0] <= 0 else parameters.gridN
    return atoms, nDim, lvec, head, elem_dict, iZs, Rs, Qs, np.array(n, dtype=np.int32)


def _finish_stage(ff, computeVpot, Fmax, Vmax, names, save_format, lvec, head, atoms):
    from . import io

    if Fmax is not None:
        ff.clamp(Fmax)
    F, E = ff.to_host()
    V = None
    if computeVpot:
        V = E
        if Vmax is not None:
            V[V > Vmax] = Vmax
    if save_format is not None:
        io.save_vec_field(names[0], F, lvec, data_format=save_format, head=head, atomic_info=(atoms[:4], lvec))
        if computeVpot:
            io.save_scal_field(names[1], V, lvec, data_format=save_format, head=head, atomic_info=(atoms[:4], lvec))
    return F, V


def computeLJ(geomFile, speciesFile, geometry_format=None, save_format=None, computeVpot=False, Fmax=Fmax_DEFAULT, Vmax=Vmax_DEFAULT, ffModel="LJ", parameters=None):
    """The Lennard-Jones stage of the command-line pipeline (HighLevel.py:260-307): geometry
    from a file (io.loadGeometry: xyz, xsf, POSCAR, FHI-aims .in), species from speciesFile
    (the built-in table when it does not exist), in-plane images when PBC, the grid on the GPU,
    |F| and V clamped, saved as FFLJ_x/y/z (and ELJ) when save_format is 'xsf' or 'npy'.
    Returns (FF [n0, n1, n2, 3], V or None, grid size, lvec), float64.  Only ffModel 'LJ' (the
    Morse and vdW models are not part of this library).  parameters: a PpafmParameters; its
    grid is set from the geometry like the reference's."""
    if ffModel != "LJ":
        raise NotImplementedError(f"force-field model {ffModel!r} is not part of this library")
    FFparams = PPU.loadSpecies(speciesFile)
    atoms, nDim, lvec, head, elem_dict, iZs, Rs, Qs, n = _load_stage_geometry(geomFile, geometry_format, parameters, FFparams)
    iPP = PPU.atom2iZ(parameters.probeType, elem_dict)
    cLJs = PPU.getAtomsLJ(iPP, iZs, FFparams)
    rec, na, _ = pack_atoms(Rs - lvec[0], cLJs, None)
    ff = DeviceFF(n, lvec).compute(rec, na, 0, FF_LJ, with_E=computeVpot)
    F, V = _finish_stage(ff, computeVpot, Fmax, Vmax, ("FF" + ffModel, "E" + ffModel), save_format, lvec, head, atoms)
    return F, V, nDim, lvec


def computeELFF_pointCharge(geomFile, geometry_format=None, tip="s", save_format=None, computeVpot=False, Fmax=Fmax_DEFAULT, Vmax=Vmax_DEFAULT, parameters=None):
    """The point-charge electrostatics stage (HighLevel.py:353-387): charges from the geometry
    file, Coulomb grid of the s / pz / dz2 tip on the GPU, clamped, saved as FFel_x/y/z (and
    Vel).  Returns (FF, V or None, grid size, lvec)."""
    tipKind = TIP_KINDS[tip]
    FFparams = PPU.loadSpecies()
    atoms, nDim, lvec, head, elem_dict, iZs, Rs, Qs, n = _load_stage_geometry(geomFile, geometry_format, parameters, FFparams)
    rec, na, nch = pack_atoms(Rs - lvec[0], None, Qs * PPU.CoulombConst)
    ff = DeviceFF(n, lvec).compute(rec, na, nch, FF_COULOMB, kind=tipKind, with_E=computeVpot)
    F, V = _finish_stage(ff, computeVpot, Fmax, Vmax, ("FFel", "Vel"), save_format, lvec, head, atoms)
    return F, V, nDim, lvec


def computeElFF(V, lvec, nDim, tip, computeVpot=False, tilt=0.0, sigma=None, deleteV=True, parameters=None):
    """Electrostatic force field of a Hartree potential V [n0, n1, n2] and the tip charge
    density (HighLevel.py:390-411) by FFT on the GPU: tip a multipole name ('s', 'pz', 'dz2',
    ...) or dict (Gaussian of width sigma, the parameters' sigma by default), a density array
    on V's grid, or an XSF file of the tip's electron density (negated into a charge density).
    Returns (FF [n0, n1, n2, 3], V_out or None), float64."""
    from . import fieldFFT as fFFT
    from . import io

    rho = None
    multipole = None
    if sigma is None:
        sigma = _get(parameters, "sigma", 0.7)
    if isinstance(tip, (list, np.ndarray)):
        rho = tip
    elif isinstance(tip, dict):
        multipole = tip
    elif tip in {"s", "px", "py", "pz", "dx2", "dy2", "dz2", "dxy", "dxz", "dyz"}:
        multipole = {tip: 1.0}
    elif str(tip).endswith(".xsf"):
        rho, _, nDim_tip, _ = io.loadXSFData(tip)
        if any(np.asarray(nDim_tip) != np.asarray(nDim)):
            raise ValueError("Input file for tip charge density has been specified, but the dimensions are incompatible with the Hartree potential file!")
        rho = -rho  # charge density from the electron density
    else:
        raise ValueError(f"unknown tip {tip!r}")
    Fx, Fy, Fz, Vout = fFFT.potential2forces_mem(V, lvec, nDim, rho=rho, sigma=sigma, multipole=multipole, doPot=computeVpot, tilt=tilt, deleteV=deleteV)
    return io.packVecGrid(Fx, Fy, Fz), Vout


# ------------------------------------------------------------------- pipeline


def _scan_coords(self, stream=None):
    """The pipeline's tip coordinates (xs, ys, zs) as device tensors, uploaded again only when
    the host arrays change."""
    host = (self.xs, self.ys, self.zs)
    cached = getattr(self, "_coords", None)
    if cached is None or not all(np.array_equal(a, b) for a, b in zip(cached[0], host)):
        dev = self.ff.FE.device
        self._coords = (tuple(np.array(v, dtype=np.float64) for v in host), tuple(upload_f64(v, dev, stream) for v in host))
    return self._coords[1]


def _relax(self, stream=None, ff=None, out=None):
    """The relaxed scan + Δf on ``ff`` (default: the pipeline's grid) into the output set
    ``out`` (a dict filled on first use; default: the pipeline's own, ``self.out``)."""
    ff = self.ff if ff is None else ff
    own = out is None
    res = relax_scan(ff, self.prm, *self._scan_coords(stream), pos_offset=self.lvec[0], df_weights=self.W, want_ppos=self.want_ppos, want_iters=self.want_iters, counter=self.counter, out=self.out if own else out, stream=stream)
    if own:
        self.out = res
    return res


class StepPipeline:
    """Back-to-back scans of one pipeline (``Pipeline`` or ``DensityOverlapPipeline``), each
    step a full force field + relaxed scan + Δf of the pipeline's current inputs, with step
    k+1's force field computed while step k's relaxation runs.

    The relaxation of a scan is latency-bound: its time is set by its longest strokes, and for
    most of it few SMs are busy.  So the steps alternate between ``nbuf`` force-field grids and
    output sets; the force fields run in order on one stream and the relaxations in order on
    another, of higher priority, so a relaxation's blocks are placed first and the force field
    of the next step fills the SMs around them.  Step k's force field waits for the relaxation
    that last read its grid (and for ``after``, e.g. the copy of the step's inputs); step k's
    relaxation waits for its force field and for ``release``d events on its output set (e.g.
    the copy of that set's previous outputs to the host).  Results are those of ``run()``."""

    def __init__(self, pl, nbuf=2):
        if nbuf < 1:
            raise ValueError("nbuf >= 1")
        self.pl = pl
        self.nbuf = nbuf
        self.ffs = [pl.ff] + [DeviceFF(pl.gridN, pl.lvec) for _ in range(nbuf - 1)]
        self.outs = [{} for _ in range(nbuf)]
        self.s_ff = torch.cuda.Stream()
        _, high = torch.cuda.Stream.priority_range()
        self.s_rx = torch.cuda.Stream(priority=high)
        self._grid_free = [None] * nbuf  # relaxation that last read grid j
        self._out_free = [None] * nbuf  # consumer of output set j (released)
        self.k = 0

    def step(self, after=None, timing=None, before_relax=None):
        """Queues one step into slot k % nbuf; returns (slot, outputs, force-field done event,
        relaxation done event).  timing: a list that gets (ff start, ff end, relax start,
        relax end) timing events of this step.  before_relax: a callable queued on the
        relaxation stream once the step's force field is done, before its relaxation."""
        j = self.k % self.nbuf
        sf, sr = self.s_ff, self.s_rx
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if timing is not None else None
        with torch.cuda.stream(sf):
            if self._grid_free[j] is not None:
                sf.wait_event(self._grid_free[j])
            if after is not None:
                sf.wait_event(after)
            if ev:
                ev[0].record(sf)
            self.pl.build_ff(stream=sf, ff=self.ffs[j])
            ff_done = torch.cuda.Event()
            ff_done.record(sf)
            if ev:
                ev[1].record(sf)
        with torch.cuda.stream(sr):
            sr.wait_event(ff_done)
            if self._out_free[j] is not None:
                sr.wait_event(self._out_free[j])
            if before_relax is not None:
                before_relax()
            if ev:
                ev[2].record(sr)
            out = self.pl.relax(stream=sr, ff=self.ffs[j], out=self.outs[j])
            rx_done = torch.cuda.Event()
            rx_done.record(sr)
            if ev:
                ev[3].record(sr)
        self._grid_free[j] = rx_done
        self._out_free[j] = None
        if ev:
            timing.append(ev)
        self.k += 1
        return j, out, ff_done, rx_done

    def release(self, j, event):
        """Output set j is written again only after ``event``."""
        self._out_free[j] = event

    def wait_idle(self, stream=None):
        """``stream`` (default: the current one) waits for every queued step."""
        s = stream if stream is not None else torch.cuda.current_stream()
        s.wait_stream(self.s_ff)
        s.wait_stream(self.s_rx)

    def start_after(self, event):
        """The next steps start only after ``event`` (e.g. the start of a timed interval)."""
        self.s_ff.wait_event(event)
        self.s_rx.wait_event(event)


class Pipeline:
    """The reference CPU pipeline (computeLJ + computeELFF_pointCharge with the default
    clamp, perform_relaxation, Fz2df) as device-resident stages.  Build once per system,
    then ``run()``; all buffers stay in HBM between runs."""

    def __init__(self, Zs, Rs, Qs, lvec, gridN, parameters, relax=None, with_df=True, want_ppos=True, want_iters=False, FFparams=None):
        self.p = parameters
        self.lvec = np.asarray(lvec, dtype=np.float64)
        self.gridN = tuple(int(x) for x in gridN)
        self.Rs0, self.cLJs, self.kqq = prepare_atoms(Zs, Rs, Qs, self.lvec, parameters, FFparams)
        self.natoms = len(self.Rs0)
        self.Q = float(_get(parameters, "charge", 0.0))
        self.tip = _get(parameters, "tip", "s")
        self.ff = DeviceFF(self.gridN, self.lvec)
        self.ff_el = None
        self.prm = tip_vector(parameters, relax)
        xT, yT, zT, self.lvecScan = PPU.prepareScanGrids(_get(parameters, "scanMin"), _get(parameters, "scanMax"), _get(parameters, "scanStep"), _get(parameters, "r0Probe"))
        self.xs = xT - self.lvec[0, 0]
        self.ys = yT - self.lvec[0, 1]
        self.zs = zT[::-1] - self.lvec[0, 2]
        self.scan_shape = (len(xT), len(yT), len(zT))
        self.W = None
        if with_df:
            units = 16.0217656
            W = PPU.get_df_weight(_get(parameters, "Amplitude", 1.0), dz=_get(parameters, "scanStep")[2])
            self.W = W * units * _get(parameters, "f0Cantilever") / _get(parameters, "kCantilever")
        self.want_ppos = want_ppos
        self.want_iters = want_iters
        self.counter = iter_counter()
        self.out = None
        self.upload_atoms()

    def upload_atoms(self, stream=None):
        """Host -> device copy of the atom records (the inputs of one run)."""
        self.atoms, _, self.ncharged = pack_atoms(self.Rs0, self.cLJs, self.kqq if self.Q != 0.0 else None, stream=stream)
        if self.tip != "s" and self.Q != 0.0:
            self.atoms_el, _, self.nch_el = pack_atoms(self.Rs0, None, self.kqq, stream=stream)

    def build_ff(self, stream=None, ff=None):
        """The force field into ``ff`` (default: the pipeline's own grid)."""
        ff = self.ff if ff is None else ff
        if self.Q == 0.0:
            ff.compute(self.atoms, self.natoms, 0, FF_LJ, stream=stream).clamp(Fmax_DEFAULT, stream=stream)
        elif self.tip == "s":
            ff.compute(self.atoms, self.natoms, self.ncharged, FF_LJC, Q=self.Q, Fmax=Fmax_DEFAULT, stream=stream)
        else:
            ff.compute(self.atoms, self.natoms, 0, FF_LJ, stream=stream).clamp(Fmax_DEFAULT, stream=stream)
            if self.ff_el is None:
                self.ff_el = DeviceFF(self.gridN, self.lvec)
            self.ff_el.compute(self.atoms_el, self.natoms, self.nch_el, FF_COULOMB, kind=TIP_KINDS[self.tip], stream=stream).clamp(Fmax_DEFAULT, stream=stream)
            ff.axpby(1.0, self.ff_el, self.Q, stream=stream)
        return ff

    _scan_coords = _scan_coords
    relax = _relax


    def run(self, stream=None):
        self.build_ff(stream)
        return self.relax(stream)

    def iterations(self):
        return int(self.counter.item())


def relaxed_scan_pipeline(Zs, Rs, Qs, lvec, gridN, parameters, relax=None, with_df=True):
    """One call: host atoms in, host (fzs, PPpos, df, lvecScan) out (float64)."""
    pl = Pipeline(Zs, Rs, Qs, lvec, gridN, parameters, relax=relax, with_df=with_df)
    out = pl.run()
    res = {k: v.cpu().numpy().astype(np.float64) for k, v in out.items()}
    return res.get("fzs"), res.get("ppos"), res.get("df"), pl.lvecScan


class DensityOverlapPipeline:
    """Pauli (density overlap) + Hartree electrostatics force field and the relaxed scan.

    Inputs (device, float32 grids of ``gridN``): the sample electron density ``rho_s``, the
    sample charge density ``rho_q`` (e/A^3, net zero for a neutral cell) and the tip electron
    density ``rho_t`` centred on the grid origin (rolled layout).  One ``build_ff``:

      rho_s^B, rho_t^B after the negative-density fix (conv_rho.py:57-64),
      FF  = A  * potential2forces(rho_s^B, rho_t^B)                 (conv_rho.py:75-83)
      V   = Poisson(rho_q)
      FF += Q/Ne * potential2forces(V, rho_t)                       (computeElFF with the tip
                                                                     density as one charge)
    then ``relax`` runs the relaxed scan + Δf on FF like ``Pipeline``.
    ``from_workload`` synthesises the three densities on the GPU from Gaussian atoms.
    f64 selects float64 transforms: float32 ones leave ~1e-6 of the field's maximum as noise
    everywhere, which moves ~0.2% of relaxed positions by more than 1e-3 A."""

    def __init__(self, lvec, gridN, parameters, A=12.0, B=1.0, tip_electrons=6.0, relax=None, with_df=True, want_ppos=True, want_iters=False, fix_negative=True, f64=False):
        self.p = parameters
        self.lvec = np.asarray(lvec, dtype=np.float64)
        self.gridN = tuple(int(x) for x in gridN)
        self.A, self.B, self.Ne = float(A), float(B), float(tip_electrons)
        self.Q = float(_get(parameters, "charge", 0.0))
        self.fix_negative = fix_negative
        self.fft = FFTGrid(self.gridN, f64=f64)
        self.rho_s = self.fft.empty()
        self.rho_q = self.fft.empty()
        self.rho_t = self.fft.empty()
        self._ws = self.fft.empty()  # rho_s^B
        self._wt = self.fft.empty()  # rho_t^B
        self.V = self.fft.empty()
        self.ff = DeviceFF(self.gridN, self.lvec)
        self.prm = tip_vector(parameters, relax)
        xT, yT, zT, self.lvecScan = PPU.prepareScanGrids(_get(parameters, "scanMin"), _get(parameters, "scanMax"), _get(parameters, "scanStep"), _get(parameters, "r0Probe"))
        self.xs = xT - self.lvec[0, 0]
        self.ys = yT - self.lvec[0, 1]
        self.zs = zT[::-1] - self.lvec[0, 2]
        self.scan_shape = (len(xT), len(yT), len(zT))
        self.W = None
        if with_df:
            units = 16.0217656
            W = PPU.get_df_weight(_get(parameters, "Amplitude", 1.0), dz=_get(parameters, "scanStep")[2])
            self.W = W * units * _get(parameters, "f0Cantilever") / _get(parameters, "kCantilever")
        self.want_ppos = want_ppos
        self.want_iters = want_iters
        self.counter = iter_counter()
        self.out = None

    @classmethod
    def from_workload(cls, w, relax=None, **kw):
        pl = cls(w["lvec"], w["gridN"], w, A=w["Apauli"], B=w["Bpauli"], tip_electrons=w["tip_electrons"], relax=relax, **kw)
        pl.synthesize(w["rho_e_atoms"], w["core_atoms"], w["tip_atoms"])
        return pl

    def synthesize(self, rho_e_atoms, core_atoms, tip_atoms, stream=None):
        """Gaussian densities: rho_s from rho_e_atoms, rho_q = cores - rho_s, rho_t."""
        g = self.fft
        g.gaussians(self.lvec, rho_e_atoms, out=self.rho_s, stream=stream)
        neg = np.array(rho_e_atoms, dtype=np.float64)
        neg[:, 4] *= -1.0
        g.gaussians(self.lvec, core_atoms, out=self.rho_q, stream=stream)
        g.gaussians(self.lvec, neg, out=self.rho_q, accumulate=True, stream=stream)
        g.gaussians(self.lvec, tip_atoms, out=self.rho_t, stream=stream)

    def set_densities(self, rho_s, rho_q, rho_t):
        """Host or device arrays of gridN (float32 on the device afterwards)."""
        for dst, src in ((self.rho_s, rho_s), (self.rho_q, rho_q), (self.rho_t, rho_t)):
            dst.copy_(torch.as_tensor(np.asarray(src, dtype=np.float32) if not torch.is_tensor(src) else src))

    def build_ff(self, stream=None, ff=None):
        """The force field into ``ff`` (default: the pipeline's own grid)."""
        ff = self.ff if ff is None else ff
        g = self.fft
        with torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext():
            self._ws.copy_(self.rho_s)
            self._wt.copy_(self.rho_t)
        g.density_power(self._ws, self.B, self.fix_negative, stream=stream)
        g.density_power(self._wt, self.B, self.fix_negative, stream=stream)
        g.potential2forces(self._ws, self._wt, self.lvec, FE=ff.FE, scale=self.A, with_E=True, stream=stream)
        if self.Q != 0.0:
            g.poisson(self.rho_q, self.lvec, out=self.V, stream=stream)
            g.potential2forces(self.V, self.rho_t, self.lvec, FE=ff.FE, scale=self.Q / self.Ne, with_E=True, accumulate=True, stream=stream)
        return ff

    _scan_coords = _scan_coords
    relax = _relax

    def run(self, stream=None):
        self.build_ff(stream)
        return self.relax(stream)

    def iterations(self):
        return int(self.counter.item())


# ------------------------------------------------------------ file hand-off between stages
# The relaxed-scan stage writes Fz to <dir>/OutFz (cli/relaxed_scan.py:184-188); the plotting
# stage reads it back, converts to Δf and writes <dir>/df with the lattice of the Δf stack
# (cli/plot_results.py:296-316).  Same files, Fz2df on the GPU.


def save_OutFz(dirname, fzs, lvec_scan, data_format="xsf", head=None):
    """Writes the relaxed scan's Fz [nx, ny, nz] as <dirname>/OutFz.xsf (or .npz)."""
    import os

    from . import io as pio

    os.makedirs(dirname, exist_ok=True)
    kw = {} if head is None else dict(head=head, atomic_info=head)
    pio.save_scal_field(os.path.join(dirname, "OutFz"), fzs, lvec_scan, data_format=data_format, **kw)


def OutFz_to_df(dirname, dz, amplitude, k0, f0, data_format="xsf", save_df=True):
    """Reads <dirname>/OutFz, converts it to Δf (common.Fz2df, on the GPU) and, with save_df,
    writes <dirname>/df.  The Δf stack's lattice starts amplitude/2 higher and is amplitude
    shorter along z.  Returns (dfs, lvec_df)."""
    import os

    from . import io as pio

    fzs, lvec, _, info = pio.load_scal_field(os.path.join(dirname, "OutFz"), data_format=data_format)
    dfs = PPU.Fz2df(fzs, dz=dz, k0=k0, f0=f0, amplitude=amplitude)
    lvec_df = np.array(lvec.copy())
    lvec_df[0][2] += amplitude / 2
    lvec_df[3][2] -= amplitude
    if save_df:
        kw = {} if data_format != "xsf" or not isinstance(info, list) else dict(head=info)
        pio.save_scal_field(os.path.join(dirname, "df"), dfs, lvec_df, data_format=data_format, **kw)
    return dfs, lvec_df
