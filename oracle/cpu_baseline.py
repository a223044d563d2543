"""Bounded CPU timing sample of the reference pipeline -- TEST/BENCH INFRASTRUCTURE ONLY.

Times the reference's CPU hot path for a workload on the host cores and extrapolates to
the full job.  The pipeline is the reference's own composition (HighLevel.computeLJ +
computeELFF_pointCharge with the Fmax clamp, perform_relaxation's FF = FFLJ + Q*FFel,
relaxTipStrokes_omp, common.Fz2df), run either by the reference core compiled from its
sources (oracle/_ref, kind "reference") or by the C restatement (libpporacle, kind "port"),
both built with the reference's compiler flags.  Built that way on an x86 host, the port
takes 1.02x (LJ grid) / 1.03x (Coulomb grid) / 1.19x (relaxation) the reference's time.

Sample, chosen so one call takes roughly ``budget_s`` seconds:
  * force field: a slab of whole z-planes of the full grid (cost is exactly linear in
    grid points x atoms), LJ and Coulomb passes over all atoms like the reference;
  * clamp and FF composition (numpy): timed on the same slab;
  * relaxation: blocks of adjacent pixel columns (one over the molecule, one at a seeded
    random place); the force field is filled on a box around each block (not timed) and
    the strokes are relaxed with the reference's FIRE;
  * Fz -> Δf: numpy convolution on the sampled columns.
Each stage's time per unit (grid point, pixel-height) is scaled to the full workload.

The density-overlap workload (FFT route) is timed by ``sample_overlap``: the whole force
field at full size with the reference's numpy algorithm (negative-density fix and power,
potential2forces_mem for Pauli and for the Hartree potential, the Poisson solve), then the
relaxation on pixel blocks of that force field as above.
"""

import ctypes
import os
import time

import numpy as np

from . import oracle as O


def _ref_lib():
    return O.Reference() if O.reference_available() else None


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform string)."""
    import platform
    import subprocess

    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def _prep(w):
    """Atoms after in-plane PBC, LJ coefficients, kqq, shifted to the grid origin."""
    from ppafm_gb300 import common as C

    FFp = C.loadSpecies()
    lv = np.asarray(w["lvec"], dtype=np.float64)
    iZ, R, Q = O.PBCAtoms(np.asarray(w["Zs"]), np.asarray(w["Rs"], np.float64), np.asarray(w["Qs"], np.float64), lv[1], lv[2], w["nPBC"][0], w["nPBC"][1])
    FFarr = np.array([(r[0], r[1], r[2]) for r in FFp])
    cLJ = O.getAtomsLJ(int(w["probeType"]), iZ, FFarr)
    return np.ascontiguousarray(R - lv[0]), np.ascontiguousarray(cLJ), np.ascontiguousarray(Q * O.CoulombConst)


def _ff_slab(ref, n, cell, R, coefs, kind, iz0, nzs, nthreads):
    """One force-field pass over the z-planes [iz0, iz0+nzs) of the full grid."""
    if ref is None:
        F, _ = O.ff_subgrid(n, cell, (0, 0, iz0), (n[0], n[1], nzs), R, coefs, kind, nthreads=nthreads)
        return F
    dC = np.asarray(cell[2]) / n[2]
    sub_cell = np.array(cell, dtype=np.float64).copy()
    sub_cell[2] = dC * nzs
    ref.set_grid(np.array([n[0], n[1], nzs], np.int32), sub_cell)
    F = np.zeros((n[0], n[1], nzs, 3))
    ref.L.setFF_Fpointer(F)
    Rs = np.ascontiguousarray(R - iz0 * dC)
    if kind < 0:
        ref.L.getLennardJonesFF(len(Rs), Rs, np.ascontiguousarray(coefs).reshape(-1, 2))
    else:
        ref.L.getCoulombFF(len(Rs), Rs, np.ascontiguousarray(coefs), kind)
    return F


def _relax_blocks(ref, w, n, cell, FF, xT, yT, zT, nthreads, seed, nb=8):
    """Relaxes two nb x nb pixel blocks on a full float64 force field; (seconds, relaxed
    pixel-heights, Fz columns).  8 x 8 blocks give every one of 16 threads four strokes."""
    lv = np.asarray(w["lvec"], np.float64)
    Z = len(zT)
    rng = np.random.default_rng(seed)
    blocks = [(len(xT) // 2 - nb // 2, len(yT) // 2 - nb // 2), (int(rng.integers(0, len(xT) - nb)), int(rng.integers(0, len(yT) - nb)))]
    r0 = w["r0Probe"]
    stiff = [w["klat"], w["klat"], w["krad"]]
    tip = O.tip_params(r0[2], stiff[2] / -O.eVA_Nm, [r0[0], r0[1], 0.0], np.array([stiff[0], stiff[1], 0.0]) / -O.eVA_Nm)
    prm = O.relax_param_vector(tip, maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    t_relax, nrel, cols = 0.0, 0, []
    for bx, by in blocks:
        rT = np.zeros((nb, nb, Z, 3))
        rT[..., 0] = (xT[bx : bx + nb] - lv[0, 0])[:, None, None]
        rT[..., 1] = (yT[by : by + nb] - lv[0, 1])[None, :, None]
        rT[..., 2] = (zT[::-1] - lv[0, 2])[None, None, :]
        t0 = time.perf_counter()
        if ref is not None:
            L = ref.L
            ref.set_grid(n, cell)
            L.setFF_Fpointer(FF)
            L.setRelax(int(w["maxIters"]), float(w["convF2"]), float(w["dt"]), float(w["damping"]))
            L.setFIRE(1.1, 0.5, 0.99)
            L.setTip(float(r0[2]), stiff[2] / -O.eVA_Nm, np.array([r0[0], r0[1], 0.0]), np.array([stiff[0], stiff[1], 0.0]) / -O.eVA_Nm)
            rs = np.zeros_like(rT)
            fs = np.zeros_like(rT)
            L.relaxTipStrokes_omp(nb, nb, 1, 1, Z, rT, rs, fs, None)
        else:
            rs, fs, _, _ = O.relax_strokes(n, cell, FF, prm, rT, nthreads=nthreads)
        t_relax += time.perf_counter() - t0
        nrel += nb * nb * Z
        cols.append(fs[:, :, ::-1, 2].reshape(-1, Z))
    return t_relax, nrel, np.concatenate(cols), len(blocks)


def sample_overlap(w, budget_s=20.0, nthreads=0, use_reference=True, seed=0):
    """Density-overlap (FFT) route: full-size force field with the reference's numpy
    algorithm, relaxation sampled on pixel blocks.  Same return keys as sample_pipeline."""
    ref = _ref_lib() if use_reference else None
    if nthreads <= 0:
        nthreads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(nthreads)
    n = np.array(w["gridN"], np.int32)
    lv = np.asarray(w["lvec"], np.float64)
    cell = lv[1:4]
    dims = tuple(int(x) for x in n)
    # inputs (not timed): float32 densities like the device path
    rho_s = O.gaussian_density(dims, lv, w["rho_e_atoms"]).astype(np.float32).astype(np.float64)
    neg = np.array(w["rho_e_atoms"])
    neg[:, 4] *= -1
    rho_q = (O.gaussian_density(dims, lv, w["core_atoms"]) + O.gaussian_density(dims, lv, neg)).astype(np.float32).astype(np.float64)
    rho_t = O.gaussian_density(dims, lv, w["tip_atoms"]).astype(np.float32).astype(np.float64)
    t0 = time.perf_counter()
    ws = O.handle_negative_density(rho_s.copy()) ** w["Bpauli"]
    wt = O.handle_negative_density(rho_t.copy()) ** w["Bpauli"]
    t_pow = time.perf_counter() - t0
    t0 = time.perf_counter()
    fx, fy, fz, _ = O.potential2forces_mem(ws, lv, dims, rho=wt, doPot=True)
    FF = w["Apauli"] * np.stack([fx, fy, fz], axis=-1)
    t_pauli = time.perf_counter() - t0
    t0 = time.perf_counter()
    V = O.poisson_hartree(rho_q, lv)
    t_poisson = time.perf_counter() - t0
    t0 = time.perf_counter()
    fx, fy, fz, _ = O.potential2forces_mem(V, lv, dims, rho=rho_t, doPot=True)
    FF += (w["charge"] / w["tip_electrons"]) * np.stack([fx, fy, fz], axis=-1)
    t_el = time.perf_counter() - t0
    del fx, fy, fz, V, ws, wt
    FF = np.ascontiguousarray(FF)
    from ppafm_gb300 import common as C

    xT, yT, zT, _ = C.prepareScanGrids(w["scanMin"], w["scanMax"], w["scanStep"], w["r0Probe"])
    P = len(xT) * len(yT)
    Z = len(zT)
    t_relax, nrel, fz_cols, nblocks = _relax_blocks(ref, w, n, cell, FF, xT, yT, zT, nthreads, seed)
    t0 = time.perf_counter()
    O.Fz2df_numpy(fz_cols[:, None, :], w["scanStep"][2], w["kCantilever"], w["f0Cantilever"], w["Amplitude"])
    t_df = time.perf_counter() - t0
    full = dict(density_power=t_pow, ff_pauli_fft=t_pauli, poisson_fft=t_poisson, ff_hartree_fft=t_el, relax=t_relax * (P * Z) / nrel, df=t_df * P / len(fz_cols))
    total = sum(full.values())
    return dict(
        kind="port",
        cores=nthreads,
        cpu_model=cpu_model(),
        seconds_full_job=full,
        total_s=total,
        pixel_z_per_s=P * Z / total,
        sample=f"force field: full {dims[0]}x{dims[1]}x{dims[2]} grid with numpy float64 FFTs (single-threaded like the reference's numpy); relax: {nblocks} blocks of 8x8 pixels x {Z} heights with the {'reference' if ref is not None else 'restated'} FIRE on {nthreads} threads; extrapolated per pixel-height",
    )


def sample_pipeline(w, budget_s=20.0, nthreads=0, use_reference=True, seed=0):
    """Returns a dict with per-stage seconds for the full job, pixel-z/s, pair rate,
    cores, kind and a description of the sample."""
    if w.get("name") == "density_overlap":
        return sample_overlap(w, budget_s, nthreads, use_reference, seed)
    ref = _ref_lib() if use_reference else None
    kind = "reference" if ref is not None else "port"
    if nthreads <= 0:
        nthreads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(nthreads)
    n = np.array(w["gridN"], np.int32)
    lv = np.asarray(w["lvec"], np.float64)
    cell = lv[1:4]
    R, cLJ, kqq = _prep(w)
    na = len(R)
    npts = int(np.prod(n.astype(np.int64)))
    from ppafm_gb300 import common as C

    xT, yT, zT, _ = C.prepareScanGrids(w["scanMin"], w["scanMax"], w["scanStep"], w["r0Probe"])
    P = len(xT) * len(yT)
    Z = len(zT)

    # ---- force field: calibrate on a few rows, then one timed slab
    t0 = time.perf_counter()
    _ = O.ff_subgrid(n, cell, (0, 0, 0), (1, min(16, n[1]), min(8, n[2])), R, cLJ, -1, nthreads=nthreads)
    t_cal = max(time.perf_counter() - t0, 1e-4)
    rate = (min(16, n[1]) * min(8, n[2])) / t_cal  # points/s of one pass, roughly
    plane = int(n[0]) * int(n[1])
    nzs = int(max(1, min(n[2], (0.3 * budget_s * rate) / plane)))
    iz0 = int(n[2] // 2)
    if iz0 + nzs > n[2]:
        iz0 = int(n[2]) - nzs
    t0 = time.perf_counter()
    Fl = _ff_slab(ref, n, cell, R, cLJ, -1, iz0, nzs, nthreads)
    t_lj = time.perf_counter() - t0
    t0 = time.perf_counter()
    Fe = _ff_slab(ref, n, cell, R, kqq, 0, iz0, nzs, nthreads)
    t_el = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.limit_vec_field(Fl, 10.0)
    O.limit_vec_field(Fe, 10.0)
    FFs = Fl.copy()
    FFs += Fe * w["charge"]
    t_np = time.perf_counter() - t0
    scale_ff = npts / float(plane * nzs)

    # ---- relaxation on pixel blocks
    rng = np.random.default_rng(seed)
    nb = 8  # 64 strokes per block: four for each of 16 threads
    blocks = [(len(xT) // 2 - nb // 2, len(yT) // 2 - nb // 2), (int(rng.integers(0, len(xT) - nb)), int(rng.integers(0, len(yT) - nb)))]
    ds = np.linalg.norm(cell, axis=1) / n
    r0 = w["r0Probe"]
    stiff = [w["klat"], w["klat"], w["krad"]]
    tip = O.tip_params(r0[2], stiff[2] / -O.eVA_Nm, [r0[0], r0[1], 0.0], np.array([stiff[0], stiff[1], 0.0]) / -O.eVA_Nm)
    prm = O.relax_param_vector(tip, maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    t_relax = 0.0
    nrel = 0
    fz_cols = []
    patch_ok = True
    FFbox = np.zeros(tuple(n) + (3,))  # lazily committed: only the boxes are touched
    for bx, by in blocks:
        xs = xT[bx : bx + nb] - lv[0, 0]
        ys = yT[by : by + nb] - lv[0, 1]
        lo = np.array([xs.min() - 1.5, ys.min() - 1.5, zT.min() - lv[0, 2] - r0[2] - 1.5])
        hi = np.array([xs.max() + 1.5, ys.max() + 1.5, zT.max() - lv[0, 2] - r0[2] + 1.5])
        i_lo = np.floor(lo / ds).astype(int)
        i_hi = np.ceil(hi / ds).astype(int) + 1
        ns = i_hi - i_lo
        for k in range(3):
            if i_lo[k] < 0 or i_hi[k] > n[k]:
                ns[k] = min(ns[k], n[k])
                i_lo[k] = max(0, min(i_lo[k], n[k] - ns[k]))
        # the box's force field (not timed); uncharged atoms add exactly +0.0 to the Coulomb sums
        Fb, _ = O.ff_subgrid(n, cell, i_lo, ns, R, cLJ, -1, nthreads=nthreads)
        q = kqq != 0.0
        Fq, _ = O.ff_subgrid(n, cell, i_lo, ns, R[q], kqq[q], 0, nthreads=nthreads) if q.any() else (np.zeros(tuple(ns) + (3,)), None)
        O.limit_vec_field(Fb, 10.0)
        O.limit_vec_field(Fq, 10.0)
        FFbox[i_lo[0] : i_lo[0] + ns[0], i_lo[1] : i_lo[1] + ns[1], i_lo[2] : i_lo[2] + ns[2]] = Fb + Fq * w["charge"]
        rT = np.zeros((nb, nb, Z, 3))
        rT[..., 0] = xs[:, None, None]
        rT[..., 1] = ys[None, :, None]
        rT[..., 2] = (zT[::-1] - lv[0, 2])[None, None, :]
        t0 = time.perf_counter()
        if ref is not None:
            L = ref.L
            ref.set_grid(n, cell)
            L.setFF_Fpointer(FFbox)
            L.setRelax(int(w["maxIters"]), float(w["convF2"]), float(w["dt"]), float(w["damping"]))
            L.setFIRE(1.1, 0.5, 0.99)
            L.setTip(float(r0[2]), stiff[2] / -O.eVA_Nm, np.array([r0[0], r0[1], 0.0]), np.array([stiff[0], stiff[1], 0.0]) / -O.eVA_Nm)
            rs = np.zeros_like(rT)
            fs = np.zeros_like(rT)
            L.relaxTipStrokes_omp(nb, nb, 1, 1, Z, rT, rs, fs, None)
        else:
            rs, fs, _, _ = O.relax_strokes(n, cell, FFbox, prm, rT, nthreads=nthreads)
        t_relax += time.perf_counter() - t0
        nrel += nb * nb * Z
        gpos = rs / ds
        if (gpos < i_lo + 1).any() or (gpos > i_lo + ns - 2).any():
            patch_ok = False
        fz_cols.append(fs[:, :, ::-1, 2].reshape(-1, Z))
    del FFbox
    fz = np.concatenate(fz_cols)
    t0 = time.perf_counter()
    O.Fz2df_numpy(fz[:, None, :], w["scanStep"][2], w["kCantilever"], w["f0Cantilever"], w["Amplitude"])
    t_df = time.perf_counter() - t0
    full = dict(
        ff_lj=t_lj * scale_ff,
        ff_el=t_el * scale_ff,
        clamp_and_sum=t_np * scale_ff,
        relax=t_relax * (P * Z) / nrel,
        df=t_df * P / len(fz),
    )
    total = sum(full.values())
    return dict(
        kind=kind,
        cores=nthreads,
        cpu_model=cpu_model(),
        seconds_full_job=full,
        total_s=total,
        pixel_z_per_s=P * Z / total,
        ff_pairs_per_s=npts * na / (full["ff_lj"] + full["ff_el"]),
        sample=f"FF: {nzs} of {n[2]} z-planes ({plane * nzs} points x {na} atoms, LJ + Coulomb passes); relax: {len(blocks)} blocks of {nb}x{nb} pixels x {Z} heights; patch_ok={patch_ok}; extrapolated linearly per grid point / pixel-height",
    )
