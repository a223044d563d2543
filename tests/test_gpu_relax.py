"""GPU relaxation and Δf against the reference-generated fixtures and the oracle.

Bars (the double-float relaxation path), written in ``_check_positions``:
  * every Δf value within 0.1 Hz (checked by each test);
  * no basin flips, and every relaxed probe position within the FIRE convergence ball of the
    reference's: |F| < 1e-4 eV/A leaves the stopping point undetermined by up to
    |F|/k_lat = 6.4e-3 A along the soft lateral spring (k_lat = 0.25 N/m);
  * positions within 1e-3 A of the reference's for all but at most 1 in 10^4 pixel heights
    (rounded up).
The double-float interpolation, springs and force sum keep the GPU's trajectories on the
reference's (measured max 1.6e-4 A on the relaxed-scan fixture).  What is left is the float32
storage of the force grid (interleaved float4, ~6e-8 relative): near the end of a stroke the
residual |F| ~ 1e-4 eV/A is a difference of forces ~1 eV/A, so that rounding can move the
iteration at which |F| first drops below the criterion, and the stopping point moves inside
the ball (measured: 7 of 192 000 pixel heights past 1e-3 A, at most 5.2e-3 A, on the FFT route
with float64 transforms).  Two paths do not follow the reference's trajectories and are held
to a stated looser bound in their own tests: the FFT route with float32 transforms (transform
noise of ~1e-6 of the field's maximum) and the learned warm start (a different starting
point inside the same ball); they use ``_split_flips``."""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POS_TOL = 1e-3
DF_TOL = 0.1
# |F_conv| / k_lat: sqrt(convF2) = 1e-4 eV/A over 0.25 N/m = 0.25/16.0217662 eV/A^2
BALL = 1e-4 / (0.25 / 16.0217662)
OUTLIER_FRAC = 1e-4


def _relax_fixture(oracle, golden):
    from tests.test_oracle import _relax_golden_setup

    g = golden("relax")
    FF, prm, xT, yT, zT = _relax_golden_setup(oracle, g)
    return g, FF, prm, xT, yT, zT


def _split_flips(dpos):
    """Per pixel height: position error; flips = error above 0.05 A (a different minimum).
    For the paths with a stated looser bound only."""
    flips = dpos > 0.05
    return flips, dpos[~flips]


def _check_positions(dpos):
    """The bar of the double-float path (module docstring).  Returns the mask of the pixel
    heights past 1e-3 A (at most 1 in 10^4), which the callers' force comparisons skip;
    Δf is compared everywhere."""
    dpos = np.asarray(dpos)
    n_out = int((dpos > POS_TOL).sum())
    worst = float(dpos.max()) if dpos.size else 0.0
    allowed = math.ceil(OUTLIER_FRAC * dpos.size)
    assert worst < BALL, f"a pixel height {worst:.3g} A from the reference's: outside the convergence ball ({BALL:.3g} A)"
    assert n_out <= allowed, f"{n_out} of {dpos.size} pixel heights beyond {POS_TOL} A (max {worst:.3g} A; at most {allowed} allowed)"
    return dpos > POS_TOL


END_TO_END_OUT_FRAC = 1e-2


def _check_end_to_end(dpos, ddf):
    """End to end: the GPU's float32 force field and its relaxation against the oracle's float64
    force field and relaxation on the same atoms (dpos [..., heights], ddf [..., df values]).
    The float32 grid's own error (stated per grid by the force-field tests) moves stopping points
    inside the convergence ball more often than the grid's storage rounding alone, and at a
    pixel whose two minima are a hair apart it can send the probe into the other one (a basin
    flip; Δf of that pixel then differs).  Bar: basin flips (beyond the ball) at most 1 in 10^4
    pixel heights (rounded up); every other height within the ball, at most 1 in 100 past
    1e-3 A; Δf within 0.1 Hz at every pixel without a flip.  Returns (flipped heights, pixels
    with a flip)."""
    dpos = np.asarray(dpos)
    flips = dpos > BALL
    n_flip = int(flips.sum())
    assert n_flip <= math.ceil(OUTLIER_FRAC * dpos.size), f"{n_flip} of {dpos.size} pixel heights in another basin"
    rest = dpos[~flips]
    assert np.mean(rest > POS_TOL) <= END_TO_END_OUT_FRAC, f"{int((rest > POS_TOL).sum())} of {rest.size} pixel heights beyond {POS_TOL} A"
    pix_flip = flips.any(axis=-1)
    assert np.abs(ddf)[~pix_flip].max() < DF_TOL
    return flips, pix_flip


def test_relax_scan_golden(gpulib, oracle, golden):
    from ppafm_gb300 import common, device

    g, FF, prm, xT, yT, zT = _relax_fixture(oracle, golden)
    lv = g["lvec"]
    ff = device.DeviceFF(g["n"], lv).from_host_f64(FF.reshape(-1, 3))
    W = common.get_df_weight(1.0, dz=0.1) * 16.0217656 * 30000.0 / 1800.0
    cnt = device.iter_counter()
    out = device.relax_scan(ff, prm, xT - lv[0, 0], yT - lv[0, 1], zT[::-1] - lv[0, 2], pos_offset=lv[0], df_weights=W, want_iters=True, counter=cnt)
    fzs = out["fzs"].cpu().numpy()
    pp = out["ppos"].cpu().numpy()
    it = out["iters"].cpu().numpy()
    df = out["df"].cpu().numpy()
    dpos = np.linalg.norm(pp - g["PPpos"], axis=-1)
    outl = _check_positions(dpos)
    assert np.abs(fzs - g["fzs"])[~outl].max() < 1e-4
    assert np.abs(df - g["df"]).max() < DF_TOL
    # iteration counts of the sampled strokes: same FIRE, float32 vs float64 rounding
    for (ix, iy), s in zip(g["picks"], g["itsum"]):
        assert abs(int(it[ix, iy].sum()) - int(s)) <= 0.05 * s + 3
    assert int(cnt.item()) >= int(it.sum())


@pytest.mark.parametrize("probeStart,relaxAlg", [(1, 1), (0, 1), (-1, 1), (1, 0)])
def test_dropin_relax_strokes_vs_oracle(gpulib, oracle, golden, probeStart, relaxAlg):
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import core

    g, FF, prm, xT, yT, zT = _relax_fixture(oracle, golden)
    lv = g["lvec"]
    FFc = np.ascontiguousarray(FF)
    HL.setFF(FFc, lvec=lv)
    core.setRelax(300, 1e-8, 0.5 if relaxAlg == 1 else 0.1, 0.1)
    core.setFIRE(1.1, 0.5, 0.99)
    core.setTip(lRadial=4.0, kRadial=20.0 / -16.0217662, rPP0=np.array([0.0, 0.0, 0.0]), kSpring=np.array([0.25, 0.25, 0.0]) / -16.0217662)
    rT = oracle.scan_tips(xT[::3], yT[::3], zT, lv[0])
    rs = np.zeros_like(rT)
    fs = np.zeros_like(rT)
    core.relaxTipStrokes_omp(rT, rs, fs, probeStart=probeStart, relaxAlg=relaxAlg)
    p2 = prm.copy()
    if relaxAlg == 0:
        p2[2] = 0.1
    rs2, fs2, sums, _ = oracle.relax_strokes(g["n"], lv[1:], FFc, p2, rT, probeStart=probeStart, relaxAlg=relaxAlg)
    dpos = np.linalg.norm(rs - rs2, axis=-1)
    outl = _check_positions(dpos)
    assert np.abs(fs - fs2)[~outl].max() < 1e-4
    assert core.last_iterations() > 0
    # one stroke: the iteration sum is returned
    s1 = core.relaxTipStroke(np.ascontiguousarray(rT[1, 1]), np.zeros_like(rT[1, 1]), np.zeros_like(rT[1, 1]), probeStart=probeStart, relaxAlg=relaxAlg)
    assert abs(s1 - sums.reshape(rT.shape[0], rT.shape[1])[1, 1]) <= 0.05 * max(1, s1) + 3
    core.deleteFF_Fpointer()


def test_relax_edge_cases(gpulib, oracle, golden):
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import core
    from ppafm_gb300._lib import PPGPUError

    g, FF, prm, xT, yT, zT = _relax_fixture(oracle, golden)
    lv = g["lvec"]
    FFc = np.ascontiguousarray(FF)
    HL.setFF(FFc, lvec=lv)
    core.setTip(lRadial=4.0, kRadial=20.0 / -16.0217662, rPP0=np.array([0.0, 0.0, 0.0]), kSpring=np.array([0.25, 0.25, 0.0]) / -16.0217662)
    rT = oracle.scan_tips(xT[:2], yT[:3], zT[:5], lv[0])
    # maxIters = 0: no move; rs = start, fs = grid force there (reference loop body never runs)
    core.setRelax(0, 1e-8, 0.5, 0.1)
    rs = np.zeros_like(rT)
    fs = np.zeros_like(rT)
    core.relaxTipStrokes_omp(rT, rs, fs)
    p0 = prm.copy()
    p0[0] = 0
    rs2, fs2, _, _ = oracle.relax_strokes(g["n"], lv[1:], FFc, p0, rT)
    assert np.abs(rs - rs2).max() < 1e-5 and np.abs(fs - fs2).max() < 1e-4
    # empty stroke set
    e = np.zeros((0, 3, 5, 3))
    assert core.relaxTipStrokes_omp(e, e.copy(), e.copy()) == 0
    # a tip spline must be a SplineParameters structure with at least two knots
    with pytest.raises(TypeError):
        core.relaxTipStrokes_omp(rT, rs, fs, tip_spline=object())
    with pytest.raises(PPGPUError, match="knots"):
        core.relaxTipStrokes_omp(rT, rs, fs, tip_spline=core.SplineParameters([4.0], [[0.0, 1.0]]))
    core.deleteFF_Fpointer()
    with pytest.raises(PPGPUError):
        core.relaxTipStrokes_omp(rT, rs, fs)


def test_fz2df_gpu_golden(gpulib, golden):
    from ppafm_gb300 import common

    g = golden("df")
    d1 = common.Fz2df(g["Fz"], dz=0.1, k0=1800.0, f0=30000.0, amplitude=1.0)
    d2 = common.Fz2df(g["Fz"], dz=0.1, k0=1800.0, f0=30300.0, amplitude=0.5)
    assert d1.shape == g["df1"].shape and np.abs(d1 - g["df1"]).max() < 1e-3
    assert np.abs(d2 - g["df2"]).max() < 1e-3
    with pytest.raises(ValueError):
        common.Fz2df(g["Fz"][..., :5], dz=0.1, k0=1800.0, f0=30000.0, amplitude=1.0)


@pytest.mark.parametrize("shape", [(512, 512, 40), (1000, 31), (37, 30), (300, 100)])
def test_fz2df_device_sizes(gpulib, oracle, shape):
    """ppgpu_fz2df on device arrays: the shared-memory kernel (columns of at most 64 samples, whole
    and ragged 32-column tiles, nz not a multiple of 4) is bit for bit the column-per-thread
    kernel (which a misaligned input takes), and both agree with the float64 oracle; columns of
    more than 64 samples take the column-per-thread kernel."""
    import torch

    from ppafm_gb300 import common

    rng = np.random.default_rng(7)
    Fh = rng.standard_normal(shape).astype(np.float32)
    F = torch.from_numpy(Fh).cuda()
    kw = dict(dz=0.1, k0=1800.0, f0=30300.0, amplitude=1.0)
    got = common.Fz2df(F, **kw)
    n = Fh.size
    buf = torch.empty(n + 1, dtype=torch.float32, device="cuda")
    mis = buf[1:].view(shape)  # 4 bytes past a 16-byte boundary
    mis.copy_(F)
    assert mis.data_ptr() % 16 != 0
    ref_kernel = common.Fz2df(mis, **kw)
    assert torch.equal(got, ref_kernel)
    want = oracle.Fz2df(Fh.astype(np.float64), **kw)
    W = common.get_df_weight(1.0, dz=0.1) * 16.0217656 * 30300.0 / 1800.0
    bound = 1e-6 * np.abs(W).sum() * np.abs(Fh).max()  # float32 rounding of an nw-term sum
    assert np.abs(got.cpu().numpy() - want).max() <= bound


@pytest.mark.parametrize("tps", [2, 4, 8])
def test_lanes_per_stroke_bit_identical(gpulib, oracle, golden, tps):
    """Splitting each stroke's gathers over 2, 4 or 8 lanes gives the one-lane results bit for
    bit (scan and stroke entry points), including iteration counts."""
    import ctypes

    import torch

    from ppafm_gb300 import _lib, device

    g, FF, prm, xT, yT, zT = _relax_fixture(oracle, golden)
    lv = g["lvec"]
    ff = device.DeviceFF(g["n"], lv).from_host_f64(FF.reshape(-1, 3))

    def run():
        out = device.relax_scan(ff, prm, xT - lv[0, 0], yT - lv[0, 1], zT[::-1] - lv[0, 2], pos_offset=lv[0], want_iters=True)
        torch.cuda.synchronize()
        return {k: v.clone() for k, v in out.items()}

    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import core

    FFc = np.ascontiguousarray(FF)
    HL.setFF(FFc, lvec=lv)
    core.setRelax(300, 1e-8, 0.5, 0.1)
    core.setFIRE(1.1, 0.5, 0.99)
    core.setTip(lRadial=4.0, kRadial=20.0 / -16.0217662, rPP0=np.array([0.0, 0.0, 0.0]), kSpring=np.array([0.25, 0.25, 0.0]) / -16.0217662)
    rT = oracle.scan_tips(xT[::3], yT[::3], zT, lv[0])

    def strokes():
        rs, fs = np.zeros_like(rT), np.zeros_like(rT)
        core.relaxTipStrokes_omp(rT, rs, fs, probeStart=1, relaxAlg=1)
        return rs, fs

    L = _lib.lib()
    try:
        _lib.check(L.ppgpu_set_relax_tps(1))
        ref, ref_s = run(), strokes()
        _lib.check(L.ppgpu_set_relax_tps(tps))
        got, got_s = run(), strokes()
    finally:
        _lib.check(L.ppgpu_set_relax_tps(0))
        core.deleteFF_Fpointer()
    for k in ref:
        assert ref[k].equal(got[k]), k
    assert np.array_equal(ref_s[0], got_s[0]) and np.array_equal(ref_s[1], got_s[1])
    t = ctypes.c_int()
    _lib.check(L.ppgpu_get_relax_tps(16384, ctypes.byref(t)))
    assert t.value in (1, 2, 4, 8)
    with pytest.raises(_lib.PPGPUError):
        _lib.check(L.ppgpu_set_relax_tps(3))


@pytest.mark.parametrize("cell", ["orthogonal", "skewed"])
@pytest.mark.parametrize("tip", ["straight", "offset"])
def test_lanes_per_stroke_bit_identical_cells_and_tips(gpulib, oracle, golden, cell, tip):
    """One lane per stroke against two lanes per stroke on an axis-aligned and a skewed cell
    (general grid coordinates), with a straight tip (rPP0 = 0, no z lateral spring) and an
    offset tip (rPP0 and a z lateral spring nonzero): identical bits for the scan and the stroke
    entry points."""
    import torch

    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import _lib, core, device

    g, FF, prm, xT, yT, zT = _relax_fixture(oracle, golden)
    lv = np.array(g["lvec"], dtype=np.float64)
    if cell == "skewed":
        lv[2] = [1.5, 9.8, 0.0]
        lv[3] = [0.7, -0.4, 10.0]
    prm = np.array(prm, dtype=np.float64)
    rPP0, kS = np.zeros(3), np.array([0.25, 0.25, 0.0]) / -16.0217662
    if tip == "offset":
        rPP0 = np.array([0.12, -0.07, 0.05])
        kS = np.array([0.25, 0.2, 0.3]) / -16.0217662
        prm[9:12] = rPP0
        prm[12:15] = kS
    ff = device.DeviceFF(g["n"], lv).from_host_f64(FF.reshape(-1, 3))

    def run():
        out = device.relax_scan(ff, prm, xT - lv[0, 0], yT - lv[0, 1], zT[::-1] - lv[0, 2], pos_offset=lv[0], want_iters=True)
        torch.cuda.synchronize()
        return {k: v.clone() for k, v in out.items()}

    HL.setFF(np.ascontiguousarray(FF), lvec=lv)
    core.setRelax(300, 1e-8, 0.5, 0.1)
    core.setFIRE(1.1, 0.5, 0.99)
    core.setTip(lRadial=4.0, kRadial=20.0 / -16.0217662, rPP0=rPP0, kSpring=kS)
    rT = oracle.scan_tips(xT[::3], yT[::3], zT, lv[0])

    def strokes():
        rs, fs = np.zeros_like(rT), np.zeros_like(rT)
        core.relaxTipStrokes_omp(rT, rs, fs, probeStart=1, relaxAlg=1)
        return rs, fs

    L = _lib.lib()
    try:
        _lib.check(L.ppgpu_set_relax_tps(1))
        ref, ref_s = run(), strokes()
        _lib.check(L.ppgpu_set_relax_tps(2))
        got, got_s = run(), strokes()
    finally:
        _lib.check(L.ppgpu_set_relax_tps(0))
        core.deleteFF_Fpointer()
    assert ref["iters"].float().mean() > 1.0
    for k in ref:
        assert ref[k].equal(got[k]), k
    assert np.array_equal(ref_s[0], got_s[0]) and np.array_equal(ref_s[1], got_s[1])


@pytest.mark.parametrize("fmt", ["xsf", "npy"])
def test_outfz_file_handoff(gpulib, golden, tmp_path, fmt):
    """Relaxed-scan Fz through the OutFz file and back to Δf (the CLI stages' hand-off):
    Δf equals the reference's within 0.1 Hz after the 6-digit XSF round trip."""
    from ppafm_gb300 import HighLevel as HL

    g = golden("relax")
    lv = np.array(g["lvecScan"])
    HL.save_OutFz(str(tmp_path), g["fzs"], lv, data_format=fmt)
    dfs, lvec_df = HL.OutFz_to_df(str(tmp_path), dz=0.1, amplitude=1.0, k0=1800.0, f0=30000.0, data_format=fmt)
    assert np.abs(dfs - g["df"]).max() < DF_TOL
    assert np.isclose(lvec_df[0][2], lv[0][2] + 0.5) and np.isclose(lvec_df[3][2], lv[3][2] - 1.0)
    ext = ".xsf" if fmt == "xsf" else ".npz"
    assert (tmp_path / ("df" + ext)).exists()


def test_fz2df_tilt_golden(gpulib, golden):
    """Fz2df_tilt (common.py:433-445) against the reference's values."""
    from ppafm_gb300 import common

    g = golden("tilt")
    for i in range(3):
        got = common.Fz2df_tilt(g["F"], g[f"d_{i}"], k0=1800.0, f0=30300.0, amplitude=float(g[f"amp_{i}"]))
        want = g[f"df_{i}"]
        assert got.shape == want.shape
        assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max() + 1e-6, i


def test_tilted_scan_relaxation(gpulib, oracle, golden):
    """perform_relaxation with tiltedScan keeps the full force vector (the reference's
    relaxedScan3D_omp ignores the trajectory): positions as the plain scan's, Fz equal to the
    plain scan's, and Fz2df_tilt along z equal to |d| Fz2df."""
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import common

    g, FF, prm, xT, yT, zT = _relax_fixture(oracle, golden)
    p = dict(charge=0.0, klat=float(g["klat"]), krad=float(g["krad"]), r0Probe=list(g["r0Probe"]), scanMin=list(g["scanMin"]), scanMax=list(g["scanMax"]), scanStep=list(g["scanStep"]), tiltedScan=False, scanTilt=[0.0, 0.0, 0.1])
    relax = dict(maxIters=300, convF2=1e-8, dt=0.5, damping=0.1)
    f_plain, pp_plain, _, _ = HL.perform_relaxation(g["lvec"], FF, parameters=p, relax=relax)
    p["tiltedScan"] = True
    f_tilt, pp_tilt, _, lvs = HL.perform_relaxation(g["lvec"], FF, parameters=p, relax=relax)
    assert f_tilt.shape == f_plain.shape + (3,)
    dpos = np.linalg.norm(pp_tilt - g["PPpos"], axis=-1)
    outl = _check_positions(dpos)
    assert np.abs(f_tilt[..., 2] - f_plain)[~outl].max() < 1e-4
    # along z the tilted conversion is the plain one times the step length (the projection
    # on d is not normalised, common.py:443-445)
    df_t = common.Fz2df_tilt(f_tilt, [0.0, 0.0, 0.1], k0=1800.0, f0=30000.0, amplitude=1.0)
    df_p = common.Fz2df(f_tilt[..., 2], dz=0.1, k0=1800.0, f0=30000.0, amplitude=1.0)
    assert np.abs(df_t - 0.1 * df_p).max() < 1e-6 * max(1.0, np.abs(df_p).max())


def _spline(krad):
    """A radial tip spline: 9 knots (not a power of two, so the reference's halving interval
    search is exercised as it is), 1.3 times stiffer than the harmonic spring plus a cubic."""
    k = 1.3 * krad / -16.0217662
    xs = np.linspace(3.0, 5.0, 9)
    ydys = np.column_stack([k * (xs - 4.0) + 0.5 * (xs - 4.0) ** 3, k + 1.5 * (xs - 4.0) ** 2])
    return xs, ydys


def test_tip_spline_strokes_and_scan_vs_oracle(gpulib, oracle, golden):
    """Radial tip spline (forceRSpline) through the drop-in strokes call and through
    perform_relaxation's scan, against the oracle (itself bit-identical to the reference)."""
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import core

    g, FF, prm, xT, yT, zT = _relax_fixture(oracle, golden)
    lv = g["lvec"]
    xs, ydys = _spline(float(g["krad"]))
    FFc = np.ascontiguousarray(FF)
    HL.setFF(FFc, lvec=lv)
    core.setRelax(300, 1e-8, 0.5, 0.1)
    core.setFIRE(1.1, 0.5, 0.99)
    core.setTip(lRadial=4.0, kRadial=float(g["krad"]) / -16.0217662, rPP0=np.array([0.0, 0.0, 0.0]), kSpring=np.array([g["klat"], g["klat"], 0.0]) / -16.0217662)
    rT = oracle.scan_tips(xT[::3], yT[::3], zT, lv[0])
    rs = np.zeros_like(rT)
    fs = np.zeros_like(rT)
    try:
        core.relaxTipStrokes_omp(rT, rs, fs, tip_spline=core.SplineParameters(xs, ydys))
    finally:
        core.deleteFF_Fpointer()
    rs2, fs2, _, _ = oracle.relax_strokes(g["n"], lv[1:], FFc, prm, rT, spline=(xs, ydys))
    outl = _check_positions(np.linalg.norm(rs - rs2, axis=-1))
    assert np.abs(fs - fs2)[~outl].max() < 1e-4
    rs3, _, _, _ = oracle.relax_strokes(g["n"], lv[1:], FFc, prm, rT)
    assert np.abs(rs3 - rs2).max() > 1e-3  # the spline changes the relaxed positions
    # the scan path (relax_scan inside perform_relaxation)
    p = dict(charge=0.0, klat=float(g["klat"]), krad=float(g["krad"]), r0Probe=list(g["r0Probe"]), scanMin=list(g["scanMin"]), scanMax=list(g["scanMax"]), scanStep=list(g["scanStep"]))
    fzs, PPpos, _, _ = HL.perform_relaxation(lv, FF, parameters=p, relax=dict(maxIters=300, convF2=1e-8, dt=0.5, damping=0.1), tip_spline=core.SplineParameters(xs, ydys))
    fz_o, pp_o, _ = oracle.relaxed_scan(g["n"], lv[1:], FF, prm, xT, yT, zT, lv[0], spline=(xs, ydys))
    outl = _check_positions(np.linalg.norm(PPpos - pp_o, axis=-1))
    assert np.abs(fzs - fz_o)[~outl].max() < 1e-4


def test_batch_refuses_tip_spline(gpulib):
    from ppafm_gb300 import device, workloads
    from ppafm_gb300._lib import PPGPUError
    from ppafm_gb300.batch import BatchPipeline

    systems = workloads.molecule_batch(seed=1, nmol=1, scale=0.2)
    w = systems[0]
    relax = dict(maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    with device.tip_spline(_spline(20.0)):
        with pytest.raises(PPGPUError, match="spline"):
            BatchPipeline(systems, w, relax=relax)
    BatchPipeline(systems, w, relax=relax).close()  # cleared again


def test_autotune_lanes_per_stroke(gpulib, oracle, golden):
    """The lanes-per-stroke autotuner times every candidate, keeps the fastest, and the scan
    it leaves selected gives the same result as one lane."""
    import ctypes

    from ppafm_gb300 import _lib, device

    g, FF, prm, xT, yT, zT = _relax_fixture(oracle, golden)
    lv = g["lvec"]
    ff = device.DeviceFF(g["n"], lv).from_host_f64(FF.reshape(-1, 3))
    L = _lib.lib()
    try:
        best, times = device.autotune_relax_tps(ff, prm, xT - lv[0, 0], yT - lv[0, 1], zT[::-1] - lv[0, 2], candidates=(1, 2, 4), reps=1)
        assert best in (1, 2, 4) and set(times) == {1, 2, 4} and all(t > 0 for t in times.values())
        t = ctypes.c_int()
        _lib.check(L.ppgpu_get_relax_tps(1000, ctypes.byref(t)))
        assert t.value == best
        got = device.relax_scan(ff, prm, xT - lv[0, 0], yT - lv[0, 1], zT[::-1] - lv[0, 2])
        _lib.check(L.ppgpu_set_relax_tps(1))
        ref = device.relax_scan(ff, prm, xT - lv[0, 0], yT - lv[0, 1], zT[::-1] - lv[0, 2])
        assert got["ppos"].equal(ref["ppos"]) and got["fzs"].equal(ref["fzs"])
    finally:
        _lib.check(L.ppgpu_set_relax_tps(0))
