"""GPU force-field kernels against the oracle and the reference-generated fixtures.

Tolerance (float32 kernels vs float64 reference): per grid point,
|F_gpu - F_ref| <= 1e-5 * max(|F_ref|, 1e-2 eV/A) -- relative 1e-5 wherever the force is
above 1e-2 eV/A (100 times the FIRE convergence force), absolute 1e-7 eV/A below it.  The
float32 error is set by the rounding of each pair term (r^2 to one ulp, amplified seven
times by r^-14) times the cancellation between terms; where |F| is small the absolute
bound is what is meaningful.  Energies use the same rule with a 1e-2 eV floor.  The finite-difference tips (pz, dz2)
amplify float32 rounding by ~r/(2*0.1 A); they are held to 1e-4."""

import numpy as np
import pytest

from tests.conftest import check_ff, grid_coords, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL_E = 1e-4  # energies: the Coulomb energy of a neutral molecule cancels more than its force
FLOOR = 1e-2  # eV/A: relative 1e-5 above it, absolute 1e-7 eV/A below


def _dev():
    from ppafm_gb300 import device

    return device


def test_lj_and_coulomb_grids_golden(gpulib, golden):
    D = _dev()
    g = golden("ff")
    n, lvec = g["n"], g["lvec"]
    ff = D.DeviceFF(n, lvec)
    atoms, na, _ = D.pack_atoms(g["Rs0"], g["cLJs"], None)
    F, E = ff.compute(atoms, na, 0, D.FF_LJ, with_E=True).to_host()
    ok = np.linalg.norm(g["F_lj"], axis=-1) < 1e30
    assert rel_err(F[ok], g["F_lj"][ok], FLOOR) < TOL
    assert rel_err(E[ok], g["E_lj"][ok], FLOOR) < TOL_E
    atoms, na, nch = D.pack_atoms(g["Rs0"], None, g["kqq"])
    for kind in (0, 1, 2):  # pz and dz2 run the float64 kernel
        F, E = ff.compute(atoms, na, nch, D.FF_COULOMB, kind=kind, with_E=True).to_host()
        assert rel_err(F, g[f"F_el{kind}"], FLOOR) < TOL, kind
        assert rel_err(E, g[f"E_el{kind}"], FLOOR) < TOL_E, kind


def test_float64_twin_matches_reference(gpulib, golden):
    """The float64 kernel (the GPU error oracle) reproduces the reference sums closely."""
    D = _dev()
    g = golden("ff")
    n, lvec = g["n"], g["lvec"]
    ff = D.DeviceFF(n, lvec)
    atoms, na, _ = D.pack_atoms(g["Rs0"], g["cLJs"], None)
    F, E = ff.compute(atoms, na, 0, D.FF_LJ, with_E=True, f64=True).to_host()
    ok = np.linalg.norm(g["F_lj"], axis=-1) < 1e30
    assert rel_err(F[ok], g["F_lj"][ok], FLOOR) < 1e-6  # float32 coefficients and output rounding
    atoms, na, nch = D.pack_atoms(g["Rs0"], None, g["kqq"])
    F, E = ff.compute(atoms, na, nch, D.FF_COULOMB, kind=0, with_E=True, f64=True).to_host()
    assert rel_err(F, g["F_el0"], FLOOR) < 1e-6


@pytest.mark.parametrize("ortho", [True, False])
def test_ljc_pipeline_mode_vs_oracle(gpulib, oracle, ortho):
    """FF = clamp(F_LJ) + Q*clamp(F_el) in one pass (HighLevel.py:143-145, 294-296, 374-376)."""
    D = _dev()
    rng = np.random.default_rng(11)
    n = np.array([24, 20, 30], np.int32)
    cell = np.array([[7.0, 0, 0], [0.4, 6.0, 0], [0, 0, 9.0]]) if ortho else np.array([[7.0, 0, 0], [0.4, 6.0, 0], [0.2, -0.3, 9.0]])
    na = 40
    R = np.column_stack([rng.uniform(-3, 10, na), rng.uniform(-3, 9, na), rng.uniform(-0.5, 0.5, na)])
    cLJ = np.column_stack([rng.uniform(10, 60, na), rng.uniform(1e4, 8e4, na)])
    q = rng.uniform(-0.3, 0.3, na) * 14.399645
    q[::3] = 0.0
    Q = -0.05
    Fl, _ = oracle.lj_grid(n, cell, R, cLJ)
    oracle.limit_vec_field(Fl, 10.0)
    Fe, _ = oracle.coulomb_grid(n, cell, R, q, 0)
    oracle.limit_vec_field(Fe, 10.0)
    ref = Fl + Q * Fe
    ff = D.DeviceFF(n, cell)
    atoms, na_, nch = D.pack_atoms(R, cLJ, q)
    assert nch == np.count_nonzero(q)
    F, _ = ff.compute(atoms, na_, nch, D.FF_LJC, Q=Q, Fmax=10.0).to_host()
    coords = grid_coords(n, np.vstack([np.zeros(3), cell]))
    check_ff("LJC with clamps", F, ref, coords, R, cLJ, q, Q)
    # without clamps (points where the float64 sums overflow float32 left out)
    Fl, _ = oracle.lj_grid(n, cell, R, cLJ)
    Fe, _ = oracle.coulomb_grid(n, cell, R, q, 0)
    F, _ = ff.compute(atoms, na_, nch, D.FF_LJC, Q=Q, Fmax=0.0).to_host()
    ok = (np.linalg.norm(Fl, axis=-1) < 1e30)[..., None]
    check_ff("LJC without clamps", np.where(ok, F, 0.0), np.where(ok, Fl + Q * Fe, 0.0), coords, R, cLJ, q, Q)


def test_subgrid_and_accumulate(gpulib, golden):
    D = _dev()
    g = golden("ff")
    n, lvec = g["n"], g["lvec"]
    ff = D.DeviceFF(n, lvec)
    atoms, na, _ = D.pack_atoms(g["Rs0"], g["cLJs"], None)
    sub = ff.compute_subgrid((3, 2, 5), (7, 9, 4), atoms, na, 0, D.FF_LJ).view(7, 9, 4, 4).cpu().numpy()
    ref = g["F_lj"][3:10, 2:11, 5:9]
    ok = np.linalg.norm(ref, axis=-1) < 1e30
    assert rel_err(sub[..., :3][ok], ref[ok], FLOOR) < TOL
    ff.compute(atoms, na, 0, D.FF_LJ)
    ff.compute(atoms, na, 0, D.FF_LJ, accumulate=True)
    F, _ = ff.to_host()
    ok = np.linalg.norm(g["F_lj"], axis=-1) < 1e30
    assert rel_err(F[ok], 2 * g["F_lj"][ok], FLOOR) < TOL


def test_core_singularity_stays_finite_and_clamps_like_reference(gpulib, oracle):
    """An atom exactly on a grid node: float32 overflows there; the slow path keeps the
    value finite and the clamped field matches the reference's clamped field."""
    D = _dev()
    n = np.array([16, 16, 16], np.int32)
    cell = np.eye(3) * 4.0
    R = np.array([[1.0, 1.0, 1.0], [2.6, 2.2, 1.9]])  # first atom on node (4,4,4)
    cLJ = np.array([[30.0, 5e4], [25.0, 4e4]])
    ff = D.DeviceFF(n, cell)
    atoms, na, _ = D.pack_atoms(R, cLJ, None)
    F, _ = ff.compute(atoms, na, 0, D.FF_LJ).clamp(10.0).to_host()
    assert np.isfinite(F).all()
    ref, _ = oracle.lj_grid(n, cell, R, cLJ)
    oracle.limit_vec_field(ref, 10.0)
    # at the node on the atom, dR = 0 removes that atom's term in both; the rest matches
    assert rel_err(F, ref, FLOOR) < TOL


def test_qzs_grid_vs_oracle(gpulib, oracle):
    """AFMulator point-charge grid (evalLJC_QZs_noPos): LJ + 3 tip charges."""
    D = _dev()
    rng = np.random.default_rng(5)
    lvec = np.array([[-1.0, -2.0, -3.0], [6.4, 0, 0], [0, 6.4, 0], [0, 0, 9.6]])
    nD = np.array([32, 32, 48], np.int32)
    na = 25
    xyz = np.column_stack([rng.uniform(0, 6, na), rng.uniform(0, 6, na), rng.uniform(-0.3, 0.3, na)])
    q = rng.uniform(-0.3, 0.3, na)
    cLJ = np.column_stack([rng.uniform(10, 60, na), rng.uniform(1e4, 8e4, na)])
    Qs, QZs = [-10.0, 20.0, -10.0, 0.0], [0.1, 0.0, -0.1, 0.0]
    ff = D.DeviceFF(nD, lvec)
    atoms, n_, nch = D.pack_atoms(xyz - lvec[0], cLJ, q)
    g32 = ff.compute(atoms, n_, nch, D.FF_QZS, Qs=Qs, QZs=QZs, with_E=True).grid4.cpu().numpy().astype(np.float64)
    g64 = ff.compute(atoms, n_, nch, D.FF_QZS, Qs=Qs, QZs=QZs, with_E=True, f64=True).grid4.cpu().numpy().astype(np.float64)
    # float64 kernel vs a numpy float64 evaluation of the same sum at sampled points
    rng2 = np.random.default_rng(0)
    pts = np.column_stack([rng2.integers(0, nD[k], 300) for k in range(3)])
    ref64 = oracle.afm_ff_qzs64(nD, lvec, xyz, q, cLJ, np.array(Qs, np.float32).astype(np.float64), QZs, points=pts)
    ok = np.linalg.norm(ref64[:, :3], axis=-1) < 1e30
    assert rel_err(g64[pts[:, 0], pts[:, 1], pts[:, 2], :3][ok], ref64[ok, :3], FLOOR) < 1e-6
    # float32 kernel vs the float64 twin.  The tip (-10, +20, -10 e at +-0.1 A) is a second
    # difference of Coulomb terms; the kernel removes the (r/QZ)^2 cancellation, the first
    # order (r/QZ ~ 30) remains: held to 5e-5, against ~3e-3 for the reference's own float32
    # form (checked next).
    ok = np.linalg.norm(g64[..., :3], axis=-1) < 1e30
    assert rel_err(g32[..., :3][ok], g64[..., :3][ok], FLOOR) < 5e-5
    # the float32 restatement of the reference (absolute coordinates, like the OpenCL
    # kernel) is itself only good to ~1e-3 near the cores
    ref = np.transpose(oracle.afm_ff_qzs(nD, lvec, xyz, q, cLJ, Qs, QZs), (2, 1, 0, 3)).astype(np.float64)
    ok = np.linalg.norm(ref[..., :3], axis=-1) < 1e6
    assert rel_err(ref[..., :3][ok], g64[..., :3][ok], FLOOR) < 3e-3


def test_dropin_core_symbols(gpulib, golden):
    """ppafm.core call sequence through ppafm_gb300.core: accumulate into the borrowed grid."""
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import core

    g = golden("ff")
    n, lvec = g["n"], g["lvec"]
    keep = []
    FF, V = HL.setFF(None, True, n=n, lvec=lvec)
    keep += [FF, V]
    core.getLennardJonesFF(np.ascontiguousarray(g["Rs0"]), np.ascontiguousarray(g["cLJs"]))
    ok = np.linalg.norm(g["F_lj"], axis=-1) < 1e30
    assert rel_err(FF[ok], g["F_lj"][ok], FLOOR) < TOL
    assert rel_err(V[ok], g["E_lj"][ok], FLOOR) < TOL
    core.getCoulombFF(np.ascontiguousarray(g["Rs0"]), np.ascontiguousarray(g["kqq"]), kind=0)  # accumulates
    ref = g["F_lj"] + g["F_el0"]
    assert rel_err(FF[ok], ref[ok], FLOOR) < TOL
    with pytest.raises(TypeError):
        core.getLennardJonesFF(g["Rs0"].astype(np.float32), g["cLJs"])
    core.deleteFF_Fpointer()
    core.deleteFF_Epointer()


def test_empty_atom_list(gpulib):
    D = _dev()
    ff = D.DeviceFF((8, 8, 8), np.eye(3) * 3)
    atoms, na, nch = D.pack_atoms(np.zeros((0, 3)), np.zeros((0, 2)), np.zeros(0))
    F, E = ff.compute(atoms, 0, 0, D.FF_LJ, with_E=True).to_host()
    assert (F == 0).all() and (E == 0).all()
    F, _ = ff.compute(atoms, 0, 0, D.FF_COULOMB).to_host()
    assert (F == 0).all()


def test_bad_arguments_raise(gpulib):
    D = _dev()
    from ppafm_gb300._lib import PPGPUError

    ff = D.DeviceFF((8, 8, 8), np.eye(3) * 3)
    atoms, na, nch = D.pack_atoms(np.zeros((2, 3)), np.ones((2, 2)), None)
    with pytest.raises(PPGPUError):
        ff.compute(atoms, na, 0, 99)
    with pytest.raises(PPGPUError):
        ff.compute(atoms, na, 0, D.FF_COULOMB, kind=7)
    with pytest.raises(PPGPUError):
        D.DeviceFF((8, 8, 8), np.zeros((3, 3))).compute(atoms, na, 0, D.FF_LJ)


def test_file_stages_vs_reference(gpulib, tmp_path, monkeypatch):
    """HighLevel.computeLJ / computeELFF_pointCharge from a geometry file (HighLevel.py:260-307,
    353-387) against the reference's own stages on the same xyz and parameters
    (tests/golden/stages), and the files they save."""
    import os

    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import common, io

    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stages")
    g = np.load(os.path.join(gold, "grids.npz"))
    monkeypatch.chdir(tmp_path)  # the stages save into the working directory, like the reference
    p = common.PpafmParameters.from_file(os.path.join(gold, "params.ini"))
    F, V, nDim, lvec = HL.computeLJ(os.path.join(gold, "mol.xyz"), None, save_format="xsf", computeVpot=True, parameters=p)
    assert tuple(nDim) == tuple(g["nDim"]) and np.allclose(lvec, g["lvec"])
    ok = np.linalg.norm(g["F_lj"], axis=-1) < 1e30
    assert rel_err(F[ok], g["F_lj"][ok].astype(np.float64), FLOOR) < TOL
    assert np.abs(V - g["E_lj"]).max() <= 1e-4 * max(1.0, np.abs(g["E_lj"]).max())
    p = common.PpafmParameters.from_file(os.path.join(gold, "params.ini"))
    F, V, _, _ = HL.computeELFF_pointCharge(os.path.join(gold, "mol.xyz"), tip="dz2", save_format="npy", computeVpot=True, parameters=p)
    assert rel_err(F, g["F_el"].astype(np.float64), FLOOR) < TOL
    assert np.abs(V - g["E_el"]).max() <= 1e-4 * max(1.0, np.abs(g["E_el"]).max())
    Fx, lv, _, _ = io.loadXSFData("FFLJ_x.xsf")
    assert Fx.shape == tuple(g["nDim"]) and np.allclose(lv, g["lvec"], atol=1e-6)
    atoms, _, _ = io.loadXSFGeom("ELJ.xsf")  # the header: the file's atoms (without images)
    assert len(atoms[0]) == 14
    d = np.load("FFel.npz")
    assert np.allclose(d["FF"], F)
