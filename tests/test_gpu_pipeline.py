"""End-to-end pipelines on the GPU against the oracle: the CPU-core pipeline (LJ + Coulomb
grids, clamps, FF composition, relaxed scan, Δf) on a scaled-down small_molecule workload,
and the AFMulator point-charge pipeline against its float32 restatement."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_pipeline(oracle, w, relax):
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import common

    Rs0, cLJs, kqq = HL.prepare_atoms(w["Zs"], w["Rs"], w["Qs"], w["lvec"], w)
    n = np.array(w["gridN"], np.int32)
    lv = w["lvec"]
    Fl, _ = oracle.lj_grid(n, lv[1:], Rs0, cLJs)
    oracle.limit_vec_field(Fl, 10.0)
    Fe, _ = oracle.coulomb_grid(n, lv[1:], Rs0, kqq, 0)
    oracle.limit_vec_field(Fe, 10.0)
    FF = Fl + w["charge"] * Fe
    prm = HL.tip_vector(w, relax)
    xT, yT, zT, _ = common.prepareScanGrids(w["scanMin"], w["scanMax"], w["scanStep"], w["r0Probe"])
    fzs, pp, it = oracle.relaxed_scan(n, lv[1:], FF, prm, xT, yT, zT, lv[0])
    df = oracle.Fz2df(fzs, w["scanStep"][2], w["kCantilever"], w["f0Cantilever"], w["Amplitude"])
    return FF, fzs, pp, df, it


def test_small_molecule_pipeline_vs_oracle(gpulib, oracle):
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import workloads

    w = workloads.small_molecule(seed=1, scale=0.3)
    relax = dict(maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    FF, fzs, pp, df, it = _oracle_pipeline(oracle, w, relax)
    pl = HL.Pipeline(w["Zs"], w["Rs"], w["Qs"], w["lvec"], w["gridN"], w, relax=relax, want_iters=True)
    out = pl.run()
    Fg, _ = pl.ff.to_host()
    from tests.conftest import check_ff, grid_coords

    check_ff("small molecule (scaled) LJ+Coulomb force field", Fg, FF, grid_coords(w["gridN"], w["lvec"]), pl.Rs0, pl.cLJs, pl.kqq, pl.Q)
    ppg = out["ppos"].cpu().numpy()
    dpos = np.linalg.norm(ppg - pp, axis=-1)
    from tests.test_gpu_relax import _check_positions

    _check_positions(dpos)
    dfg = out["df"].cpu().numpy()
    assert np.abs(dfg - df).max() < 0.1
    itg = out["iters"].cpu().numpy()
    assert abs(itg.mean() - it.mean()) < 0.05 * it.mean() + 0.5
    assert pl.iterations() == int(itg.sum()) or pl.iterations() >= int(itg.sum())


def test_afmulator_vs_oracle(gpulib, oracle):
    from ppafm_gb300 import species
    from ppafm_gb300.AFMulator import AFMulator

    rng = np.random.default_rng(4)
    na = 20
    xyzs = np.column_stack([rng.uniform(4, 12, na), rng.uniform(4, 12, na), rng.uniform(-0.3, 0.3, na)])
    Zs = rng.choice([1, 6, 7, 8], size=na)
    qs = rng.uniform(-0.3, 0.3, na)
    qs -= qs.mean()
    kw = dict(pixPerAngstrome=10, scan_dim=(32, 28, 24), scan_window=((4.0, 4.0, 7.0), (12.0, 11.0, 9.4)), df_steps=8, npbc=(1, 1, 0))
    lvec_sample = np.array([[16.0, 0, 0], [0, 16.0, 0], [0, 0, 20.0]])
    afm = AFMulator(**kw)
    X = afm.eval(xyzs, Zs, qs, sample_lvec=lvec_sample)
    T = species.loadSpecies()
    FFp = np.array([(r[0], r[1], r[2]) for r in T])
    ora = oracle.AFMulator(FFp, **kw)
    Xo, aux = ora.eval(xyzs, Zs, qs, sample_lvec=lvec_sample, return_all=True)
    assert X.shape == Xo.shape == (32, 28, 24 - 8 + 1)
    # float32 on both sides; relaxation trajectories agree to float rounding except at
    # bistable pixels
    d = np.abs(X - Xo)
    bad = d > 0.1
    assert bad.mean() < 0.01, bad.mean()
    assert np.median(d) < 1e-2
    # repeated eval reuses buffers and gives the same image
    X2 = afm(xyzs, Zs, qs, sample_lvec=lvec_sample)
    assert np.array_equal(X, X2)
    with pytest.raises(NotImplementedError):
        AFMulator(rho_delta={"s": 1.0})  # FDBM


def _hartree_case(oracle, grid=None):
    """Atoms and the Hartree potential of their Gaussian charges, on a 16 x 16 x 20 A cell of
    48 x 48 x 60 points or on grid = (shape, lvec)."""
    rng = np.random.default_rng(9)
    na = 16
    xyzs = np.column_stack([rng.uniform(5, 11, na), rng.uniform(5, 11, na), rng.uniform(-0.3, 0.3, na)])
    Zs = rng.choice([1, 6, 7, 8], size=na)
    q = rng.uniform(-0.4, 0.4, na)
    q -= q.mean()
    lvp = np.array([[0.0, 0, -10.0], [16.0, 0, 0], [0, 16.0, 0], [0, 0, 20.0]])
    n = (48, 48, 60)
    if grid is not None:
        n, lvp = tuple(int(x) for x in grid[0]), np.array(grid[1], dtype=np.float64)
    atoms = np.column_stack([xyzs - lvp[0], np.full(na, 0.7), q])
    rho = oracle.gaussian_density(n, lvp, atoms)
    pot = oracle.poisson_hartree(rho, lvp).astype(np.float32)
    return xyzs, Zs, pot, lvp


@pytest.mark.parametrize("rotate", [False, True])
def test_afmulator_hartree_vs_oracle(gpulib, oracle, rotate):
    """The Hartree route (potential interpolated onto the force-field grid, FFT
    cross-correlation with the dz2 tip density, centred-difference gradient, + Lennard-Jones)
    against its float64-FFT restatement: force field and Δf images."""
    from ppafm_gb300 import species
    from ppafm_gb300.AFMulator import AFMulator, HartreePotential

    xyzs, Zs, pot, lvp = _hartree_case(oracle)
    kw = dict(pixPerAngstrome=10, scan_dim=(32, 28, 24), scan_window=((4.0, 4.0, 7.0), (12.0, 11.0, 9.4)), df_steps=8, npbc=(1, 1, 0))
    rot = np.eye(3)
    if rotate:
        c, s_ = np.cos(0.3), np.sin(0.3)
        rot = np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1.0]])
    afm = AFMulator(rho={"dz2": -0.1}, sigma=0.71, **kw)
    X = afm.eval(xyzs, Zs, HartreePotential(pot, lvp), rot=rot)
    FE = afm.downloadFF()
    T = species.loadSpecies()
    FFp = np.array([(r[0], r[1], r[2]) for r in T])
    ora = oracle.AFMulator(FFp, **kw)
    Xo, aux = ora.eval(xyzs, Zs, None, pot=(pot, lvp), rho={"dz2": -0.1}, sigma=0.71, rot=rot, return_all=True)
    FEo = aux["FE"].transpose(2, 1, 0, 3)
    assert FE.shape == FEo.shape
    scale = np.abs(FEo[..., :3].astype(np.float64)).max()
    # the clamp-free LJ core makes the largest forces; compare where |F| is in the imaging range
    m = np.linalg.norm(FEo[..., :3].astype(np.float64), axis=-1) < 10.0
    assert np.abs(FE[..., :3] - FEo[..., :3])[m].max() <= 1e-4 * min(scale, 10.0) + 1e-5
    d = np.abs(X - Xo)
    assert (d > 0.1).mean() < 0.01 and np.median(d) < 1e-2
    # the tip's spectrum is transformed once and reused: the same image again
    assert np.array_equal(afm.eval(xyzs, Zs, HartreePotential(pot, lvp), rot=rot), X)
    if rotate:
        with pytest.raises(NotImplementedError):
            AFMulator(**kw).eval(xyzs, Zs, HartreePotential(pot, lvp), rot=rot)  # point-charge tip: no rotation


@pytest.mark.parametrize("matching", [False, True])
def test_afmulator_hartree_point_charge_tip_vs_oracle(gpulib, oracle, matching):
    """The Hartree route with the point-charge tip (no tip density): the electric field from
    the potential -- centred differences on the potential's own grid when it is the force
    field's grid, else of the interpolated potential -- sampled at the tip charges' heights,
    plus Lennard-Jones; force field and Δf images against the float32 restatement."""
    from ppafm_gb300 import species
    from ppafm_gb300.AFMulator import AFMulator, HartreePotential

    kw = dict(pixPerAngstrome=10, scan_dim=(32, 28, 24), scan_window=((4.0, 4.0, 7.0), (12.0, 11.0, 9.4)), df_steps=8, npbc=(1, 1, 0))
    afm = AFMulator(**kw)
    # matching: the potential made on the force-field grid itself
    xyzs, Zs, pot, lvp = _hartree_case(oracle, (afm.nDim, afm.lvec) if matching else None)
    X = afm.eval(xyzs, Zs, HartreePotential(pot, lvp))
    FE = afm.downloadFF()
    T = species.loadSpecies()
    FFp = np.array([(r[0], r[1], r[2]) for r in T])
    Xo, aux = oracle.AFMulator(FFp, **kw).eval(xyzs, Zs, None, pot=(pot, lvp), rho=None, return_all=True)
    FEo = aux["FE"].transpose(2, 1, 0, 3)
    assert FE.shape == FEo.shape
    scale = np.abs(FEo[..., :3].astype(np.float64)).max()
    m = np.linalg.norm(FEo[..., :3].astype(np.float64), axis=-1) < 10.0
    assert np.abs(FE[..., :3] - FEo[..., :3])[m].max() <= 1e-4 * min(scale, 10.0) + 1e-5
    assert np.abs(FE[..., 3] - FEo[..., 3])[m].max() <= 1e-4 * np.abs(FEo[..., 3][m]).max() + 1e-5
    d = np.abs(X - Xo)
    assert (d > 0.1).mean() < 0.01 and np.median(d) < 1e-2
    # the tip charges matter: without them the image differs
    afm0 = AFMulator(**kw, Qs=[0, 0, 0, 0])
    assert np.abs(afm0.eval(xyzs, Zs, HartreePotential(pot, lvp)) - X).max() > 0.1


def test_step_pipeline_matches_run(gpulib):
    """HighLevel.StepPipeline (step k+1's force field on its own stream while step k relaxes,
    two grids and output sets) gives run()'s results bit for bit, with the inputs alternating
    between two molecules: each step's atoms go in on a third stream after the previous
    force field has read the atom buffer, and the outputs of each step are checked."""
    import torch

    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import workloads

    w = workloads.small_molecule(seed=2, scale=0.3)
    relax = dict(maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    w2 = dict(w, Rs=w["Rs"] + np.array([0.37, -0.21, 0.05]))
    ref, recs = [], []
    for ww in (w, w2):
        pl = HL.Pipeline(ww["Zs"], ww["Rs"], ww["Qs"], ww["lvec"], ww["gridN"], ww, relax=relax, want_iters=True)
        ref.append({k: v.clone() for k, v in pl.run().items()})
        recs.append(pl.atoms.clone())
    assert not torch.equal(ref[0]["ppos"], ref[1]["ppos"])
    sp = HL.StepPipeline(pl)  # pl holds w2's atoms; every step below loads its own
    cs = torch.cuda.Stream()
    last_ff, steps = None, []
    for k in range(6):
        with torch.cuda.stream(cs):
            if last_ff is not None:
                cs.wait_event(last_ff)
            pl.atoms.copy_(recs[k % 2], non_blocking=True)
            loaded = torch.cuda.Event()
            loaded.record(cs)
        j, out, last_ff, rx = sp.step(after=loaded)
        snap = torch.cuda.Stream()
        with torch.cuda.stream(snap):  # keep a copy of this step's outputs before set j is reused
            snap.wait_event(rx)
            steps.append({key: v.clone() for key, v in out.items()})
            copied = torch.cuda.Event()
            copied.record(snap)
        sp.release(j, copied)
    sp.wait_idle()
    torch.cuda.synchronize()
    for k, got in enumerate(steps):
        for key, v in ref[k % 2].items():
            assert torch.equal(got[key], v), (k, key)
