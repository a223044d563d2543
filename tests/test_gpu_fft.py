"""The FFT density-overlap route on the GPU against the oracle.

cuFFT works in float32 complex, so every FFT-route comparison is normalised by the field's
maximum: an FFT spreads each output's rounding error over the whole grid, so pointwise
relative error is meaningless where the field crosses zero.  Tolerance: max |GPU - oracle|
<= 1e-5 * max |oracle| per component for float32 transforms (these sizes reach ~1e-6), and
1e-6 * max for float64 transforms (what remains is the float32 storage of the grids).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL64 = 1e-6


def _close(a, b, tol=TOL):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) <= tol, float(np.abs(a - b).max() / scale)


def _to_dev(x):
    import torch

    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32)).cuda()


def _fe(FE, dims):
    g = FE.view(tuple(dims) + (4,)).cpu().numpy().astype(np.float64)
    return g[..., 0], g[..., 1], g[..., 2], g[..., 3]


@pytest.mark.parametrize("f64", [False, True])
@pytest.mark.parametrize("tag", ["ortho", "skew_odd"])
def test_potential2forces_golden(gpulib, golden, tag, f64):
    """fieldFFT.potential2forces_mem outputs stored from the reference (float64 numpy)."""
    from ppafm_gb300.fieldFFT import FFTGrid

    tol = TOL64 if f64 else TOL
    g = golden("fft")
    V, rho, lv = g[f"{tag}_V"], g[f"{tag}_rho"], g[f"{tag}_lvec"]
    # float32 grids in: compare against the reference on the same float32-rounded inputs
    G = FFTGrid(V.shape, f64=f64)
    FE = G.potential2forces(_to_dev(V), _to_dev(rho), lv)
    for got, name in zip(_fe(FE, V.shape), ("Fx", "Fy", "Fz", "E")):
        ok, err = _close(got, g[f"{tag}_{name}"], tol if not f64 else 2e-6)
        assert ok, (tag, name, err)
    # the tip density built on the GPU (s + dz2 multipole, sigma 0.7)
    rt = G.probe_density(lv, 0.7, {"s": 1.0, "dz2": -0.3})
    FE = G.potential2forces(_to_dev(V), rt, lv)
    for got, name in zip(_fe(FE, V.shape), ("mFx", "mFy", "mFz", "mE")):
        ok, err = _close(got, g[f"{tag}_{name}"], tol if not f64 else 2e-6)
        assert ok, (tag, name, err)


@pytest.mark.parametrize("tag", ["ortho", "skew_odd"])
def test_potential2forces_f64_vs_oracle_same_inputs(gpulib, oracle, golden, tag):
    """float64 transforms on float32-rounded inputs against the oracle on the same inputs."""
    from ppafm_gb300.fieldFFT import FFTGrid

    g = golden("fft")
    V, rho, lv = (g[f"{tag}_V"].astype(np.float32).astype(np.float64), g[f"{tag}_rho"].astype(np.float32).astype(np.float64), g[f"{tag}_lvec"])
    ref = oracle.potential2forces_mem(V, lv, V.shape, rho=rho, doPot=True)
    FE = FFTGrid(V.shape, f64=True).potential2forces(_to_dev(V), _to_dev(rho), lv)
    got = _fe(FE, V.shape)
    for k, r in zip((0, 1, 2, 3), ref):
        ok, err = _close(got[k], r, TOL64)
        assert ok, (tag, k, err)


def test_potential2forces_mem_dropin(gpulib, golden):
    """The reference-signature host function (float64 numpy in and out)."""
    from ppafm_gb300 import fieldFFT

    g = golden("fft")
    V, rho, lv = g["skew_odd_V"], g["skew_odd_rho"], g["skew_odd_lvec"]
    fx, fy, fz, e = fieldFFT.potential2forces_mem(V, lv, np.array(V.shape), rho=rho, doForce=True, doPot=True)
    for got, name in ((fx, "Fx"), (fy, "Fy"), (fz, "Fz"), (e, "E")):
        assert got.dtype == np.float64 and got.shape == V.shape
        assert _close(got, g[f"skew_odd_{name}"])[0], name
    fx, fy, fz, e = fieldFFT.potential2forces_mem(V, lv, np.array(V.shape), sigma=0.7, multipole={"s": 1.0, "dz2": -0.3}, doPot=False)
    assert e is None and _close(fz, g["skew_odd_mFz"])[0]
    with pytest.raises(ValueError):
        fieldFFT.potential2forces_mem(V[:-1], lv, np.array(V.shape), rho=rho)
    # HighLevel.computeElFF (HighLevel.py:390-411): the same with a density array, a multipole
    # dict and an XSF tip-density file (its electron density negated)
    import os
    import tempfile

    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import io

    FF, E = HL.computeElFF(V, lv, np.array(V.shape), rho, computeVpot=True)
    assert _close(FF[..., 2], g["skew_odd_Fz"])[0] and _close(E, g["skew_odd_E"])[0]
    FF, E = HL.computeElFF(V, lv, np.array(V.shape), {"s": 1.0, "dz2": -0.3}, sigma=0.7)
    assert E is None and _close(FF[..., 2], g["skew_odd_mFz"])[0]
    d = tempfile.mkdtemp()
    io.saveXSFData(os.path.join(d, "tip.xsf"), -rho, lv)
    FF, _ = HL.computeElFF(V, lv, np.array(V.shape), os.path.join(d, "tip.xsf"))
    assert np.abs(FF[..., 2] - g["skew_odd_Fz"]).max() <= 1e-4 * np.abs(g["skew_odd_Fz"]).max()  # the file keeps 6 digits


@pytest.mark.parametrize("mp", [None, {"s": 1.0}, {"px": 1.0}, {"py": 0.7}, {"pz": -1.0}, {"dz2": 1.0}, {"dx2": 0.5}, {"dy2": 0.5}, {"dxy": 1.0}, {"dxz": 1.0}, {"dyz": 1.0}, {"s": 1.0, "dz2": -0.3}])
def test_probe_density_vs_oracle(gpulib, oracle, mp):
    from ppafm_gb300.fieldFFT import FFTGrid

    for dims, lv in (((24, 20, 16), np.array([[0.0, 0, 0], [6.0, 0, 0], [0, 5.0, 0], [0, 0, 4.0]])), ((15, 16, 17), np.array([[0.0, 0, 0], [6.0, 0, 0], [1.2, 5.5, 0], [0, 0.4, 4.3]]))):
        dd = oracle.grid_dd(lv, dims)
        X, Y, Z = oracle.getMGrid(dims, dd)
        ref = oracle.getProbeDensity(lv, X, Y, Z, dd, sigma=0.7, multipole_dict=mp)
        got = FFTGrid(dims).probe_density(lv, 0.7, mp).cpu().numpy()
        ok, err = _close(got, ref, 1e-6)
        assert ok, (dims, mp, err)


@pytest.mark.parametrize("B", [1.0, 1.3, 0.5])
def test_density_power_vs_oracle(gpulib, oracle, B):
    from ppafm_gb300.fieldFFT import FFTGrid

    rng = np.random.default_rng(3)
    dims = (20, 18, 22)
    rho = rng.normal(0.3, 0.5, size=dims)  # a fifth of the voxels negative
    G = FFTGrid(dims)
    d = _to_dev(rho)
    G.density_power(d, B, True)
    ref = oracle.handle_negative_density(rho.astype(np.float32).astype(np.float64).copy()) ** B
    assert _close(d.cpu().numpy(), ref, 1e-6)[0]
    # no fix: plain power of a positive density
    pos = np.abs(rho) + 0.01
    d = _to_dev(pos)
    G.density_power(d, B, False)
    assert _close(d.cpu().numpy(), pos.astype(np.float32).astype(np.float64) ** B, 1e-6)[0]


@pytest.mark.parametrize("f64", [False, True])
@pytest.mark.parametrize("cell", ["ortho", "skew"])
def test_poisson_vs_oracle(gpulib, oracle, cell, f64):
    from ppafm_gb300.fieldFFT import FFTGrid

    rng = np.random.default_rng(5)
    dims = (32, 30, 28)
    lv = np.array([[0.0, 0, 0], [9.0, 0, 0], [0, 8.5, 0], [0, 0, 8.0]]) if cell == "ortho" else np.array([[0.0, 0, 0], [9.0, 0, 0], [2.0, 8.0, 0], [0.5, -0.7, 8.0]])
    atoms = np.column_stack([rng.uniform(0, 8, (6, 3)), rng.uniform(0.6, 1.0, 6), rng.uniform(-1, 1, 6)])
    rho = oracle.gaussian_density(dims, lv, atoms)
    rho = rho.astype(np.float32).astype(np.float64)
    ref = oracle.poisson_hartree(rho, lv)
    got = FFTGrid(dims, f64=f64).poisson(_to_dev(rho), lv).cpu().numpy()
    ok, err = _close(got, ref, TOL64 if f64 else TOL)
    assert ok, err


def test_poisson_plane_wave_kat(gpulib):
    """rho = cos(G.r) with G a reciprocal-lattice vector of a skewed cell solves exactly to
    V = 4 pi k_e cos(G.r) / |G|^2."""
    from ppafm_gb300.fieldFFT import FFTGrid

    dims = (24, 20, 18)
    lv = np.array([[0.0, 0, 0], [7.0, 0, 0], [1.5, 6.0, 0], [0.3, 0.4, 5.5]])
    cell = lv[1:]
    Bm = 2 * np.pi * np.linalg.inv(cell).T
    Gv = 2 * Bm[0] - 1 * Bm[1] + 3 * Bm[2]
    f = np.stack(np.meshgrid(*[np.arange(dims[k]) / dims[k] for k in range(3)], indexing="ij"), axis=-1)
    r = f @ cell
    rho = np.cos(r @ Gv)
    exact = 4 * np.pi * 14.399645 * rho / (Gv @ Gv)
    got = FFTGrid(dims).poisson(_to_dev(rho), lv).cpu().numpy()
    assert _close(got, exact)[0]


def test_gaussian_density_vs_oracle(gpulib, oracle):
    from ppafm_gb300.fieldFFT import FFTGrid

    rng = np.random.default_rng(8)
    dims = (26, 22, 30)
    lv = np.array([[1.0, -2.0, 3.0], [8.0, 0, 0], [1.0, 7.0, 0], [0, 0.5, 9.0]])
    atoms = np.column_stack([rng.uniform(-2, 10, (9, 3)), rng.uniform(0.5, 0.9, 9), rng.uniform(0.5, 7, 9)])
    ref = oracle.gaussian_density(dims, lv, atoms)
    G = FFTGrid(dims)
    got = G.gaussians(lv, atoms)
    assert _close(got.cpu().numpy(), ref, 1e-6)[0]
    G.gaussians(lv, atoms[:3], out=got, accumulate=True)
    assert _close(got.cpu().numpy(), ref + oracle.gaussian_density(dims, lv, atoms[:3]), 1e-6)[0]


def test_scale_and_accumulate(gpulib, golden):
    from ppafm_gb300.fieldFFT import FFTGrid

    g = golden("fft")
    V, rho, lv = g["ortho_V"], g["ortho_rho"], g["ortho_lvec"]
    G = FFTGrid(V.shape)
    FE = G.potential2forces(_to_dev(V), _to_dev(rho), lv, with_E=False)
    base = FE.clone()
    G.potential2forces(_to_dev(V), _to_dev(rho), lv, FE=FE, scale=-2.5, with_E=True, accumulate=True)
    got = _fe(FE, V.shape)
    b = _fe(base, V.shape)
    assert np.all(b[3] == 0.0)  # E not requested: zero
    for k, name in enumerate(("Fx", "Fy", "Fz", "E")):
        ref = (g[f"ortho_{name}"] if k < 3 else 0.0) - 2.5 * g[f"ortho_{name}"]
        assert _close(got[k], ref)[0], name


def test_translation_equivariance_full_size(gpulib):
    """At the full 256^3 density-overlap grid: shifting the sample density by whole grid
    steps shifts the force field by the same steps (exact in exact arithmetic)."""
    import torch

    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import workloads

    w = workloads.density_overlap(seed=2)
    pl = HL.DensityOverlapPipeline.from_workload(w, want_ppos=False)
    FE0 = pl.build_ff().grid4.clone()
    sh = (3, -5, 7)
    pl.rho_s.copy_(torch.roll(pl.rho_s, sh, dims=(0, 1, 2)))
    pl.rho_q.copy_(torch.roll(pl.rho_q, sh, dims=(0, 1, 2)))
    FE1 = pl.build_ff().grid4
    ref = torch.roll(FE0, sh, dims=(0, 1, 2))
    for c in range(4):
        d = (FE1[..., c] - ref[..., c]).abs().max().item()
        m = ref[..., c].abs().max().item()
        assert d <= TOL * m, (c, d, m)


def _oracle_density_overlap(oracle, w, relax):
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import common

    n = tuple(w["gridN"])
    lv = w["lvec"]
    rho_s = oracle.gaussian_density(n, lv, w["rho_e_atoms"])
    neg = np.array(w["rho_e_atoms"])
    neg[:, 4] *= -1
    rho_q = oracle.gaussian_density(n, lv, w["core_atoms"]) + oracle.gaussian_density(n, lv, neg)
    rho_t = oracle.gaussian_density(n, lv, w["tip_atoms"])
    # float32 inputs on both sides (the GPU densities are float32)
    rho_s, rho_q, rho_t = (x.astype(np.float32).astype(np.float64) for x in (rho_s, rho_q, rho_t))
    ws = oracle.handle_negative_density(rho_s.copy()) ** w["Bpauli"]
    wt = oracle.handle_negative_density(rho_t.copy()) ** w["Bpauli"]
    fx, fy, fz, e = oracle.potential2forces_mem(ws, lv, n, rho=wt, doPot=True)
    FF = w["Apauli"] * np.stack([fx, fy, fz], axis=-1)
    E = w["Apauli"] * e
    V = oracle.poisson_hartree(rho_q, lv)
    fx, fy, fz, e = oracle.potential2forces_mem(V.astype(np.float32).astype(np.float64), lv, n, rho=rho_t, doPot=True)
    s = w["charge"] / w["tip_electrons"]
    FF += s * np.stack([fx, fy, fz], axis=-1)
    E += s * e
    prm = HL.tip_vector(w, relax)
    xT, yT, zT, _ = common.prepareScanGrids(w["scanMin"], w["scanMax"], w["scanStep"], w["r0Probe"])
    fzs, pp, it = oracle.relaxed_scan(np.array(n, np.int32), lv[1:], FF, prm, xT, yT, zT, lv[0])
    df = oracle.Fz2df(fzs, w["scanStep"][2], w["kCantilever"], w["f0Cantilever"], w["Amplitude"])
    return (rho_s, rho_q, rho_t), FF, E, fzs, pp, df, it


@pytest.fixture(scope="module")
def overlap_case(oracle):
    from ppafm_gb300 import workloads

    w = workloads.density_overlap(seed=1, scale=0.5)
    relax = dict(maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    return w, relax, _oracle_density_overlap(oracle, w, relax)


@pytest.mark.parametrize("f64", [True, False])
def test_density_overlap_pipeline_vs_oracle(gpulib, overlap_case, f64):
    """Pauli + Hartree force field, relaxed scan and Δf at half size (128^3 grid, 80x80x30
    scan).
    float64 transforms: the bar of the double-float relaxation path (every position within the
    convergence ball, at most 1 in 10^4 past 1e-3 A, every Δf within 0.1 Hz).  float32
    transforms (the default of the density-overlap workload): force field within
    1e-5 of its maximum; the ~1e-6 * max transform noise (~3e-5 eV/A against a 0.016 eV/A^2
    lateral spring) moves 0.2% of the positions past 1e-3 A, at most 0.028 A (stated bound:
    <= 0.5% past 1e-3 A, all within 0.04 A)."""
    from ppafm_gb300 import HighLevel as HL
    from tests.test_gpu_relax import POS_TOL, _check_positions, _split_flips

    w, relax, (dens, FF, E, fzs, pp, df, it) = overlap_case
    pl = HL.DensityOverlapPipeline.from_workload(w, relax=relax, want_iters=True, f64=f64)
    # the GPU-synthesised densities against the oracle's
    for got, ref in zip((pl.rho_s, pl.rho_q, pl.rho_t), dens):
        assert _close(got.cpu().numpy(), ref, 1e-6)[0]
    out = pl.run()
    Fg, Eg = pl.ff.to_host()
    tol = TOL64 if f64 else TOL
    for c in range(3):
        ok, err = _close(Fg[..., c], FF[..., c], tol)
        assert ok, (c, err)
    assert _close(Eg, E, tol)[0]
    ppg = out["ppos"].cpu().numpy()
    dpos = np.linalg.norm(ppg - pp, axis=-1)
    if f64:
        flips = _check_positions(dpos)
        assert np.abs(out["df"].cpu().numpy() - df).max() < 0.1
    else:
        flips, good = _split_flips(dpos)
        assert flips.mean() <= 0.005 and np.mean(good > POS_TOL) <= 0.005 and good.max() < 0.04, (flips.mean(), np.mean(good > POS_TOL), good.max())
        ok = ~flips.any(axis=-1)
        assert np.abs(out["df"].cpu().numpy() - df)[ok].max() < 0.1
    itg = out["iters"].cpu().numpy()
    assert abs(itg.mean() - it.mean()) < 0.05 * it.mean() + 0.5
    dfz = np.abs(out["fzs"].cpu().numpy() - fzs)[~flips].max()
    assert dfz < (1e-4 if f64 else 2e-3), dfz


def test_get_probe_density_reference_signature(gpulib, oracle):
    """fieldFFT.getProbeDensity called like the reference (sampleSize, X, Y, Z, dd, sigma,
    multipole_dict) with getMGrid coordinates equals the (lvec, nDim) form and the oracle."""
    from ppafm_gb300 import fieldFFT as F

    lv = np.array([[0.0, 0, 0], [6.0, 0, 0], [1.2, 5.5, 0], [0, 0.4, 4.3]])
    dims = (15, 16, 17)
    dd = [F.getSize(a, dims, F.getSampleDimensions(lv))[1] for a in "xyz"]
    X, Y, Z = F.getMGrid(dims, dd)
    mp = {"s": 1.0, "dz2": -0.3}
    a = F.getProbeDensity(F.getSampleDimensions(lv), X, Y, Z, dd, 0.7, mp)
    b = F.getProbeDensity(lv, dims, sigma=0.7, multipole_dict=mp)
    assert np.array_equal(a, b)
    Xo, Yo, Zo = oracle.getMGrid(dims, dd)
    ref = oracle.getProbeDensity(lv, Xo, Yo, Zo, dd, sigma=0.7, multipole_dict=mp)
    assert np.abs(a - ref).max() <= 1e-5 * np.abs(ref).max()
    with pytest.raises(ValueError):
        F.getProbeDensity(F.getSampleDimensions(lv), X + 0.1, Y, Z, dd, 0.7, mp)
