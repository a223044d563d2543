"""Pins the CPU oracle: against the reference's own golden vectors (tests/test_common.py of
ppafm), against fixtures produced by running the reference package (tests/golden), and
bit for bit against the reference C++ core compiled from its sources (oracle/_ref)."""

import numpy as np
import pytest


def test_df_weights_reference_test_vectors(oracle):
    # ppafm tests/test_common.py:10-24
    assert np.allclose(oracle.get_df_weight(0.1), np.array([-5.0, 5.0]))
    assert np.allclose(oracle.get_df_weight(1.0, dz=0.2), np.array([-0.35594622, -0.22193265, -0.05447093, 0.05447093, 0.22193265, 0.35594622]))
    assert np.allclose(oracle.get_simple_df_weight(n=5, dz=0.2), np.array([-0.31362841, -0.37274317, 0, 0.37274317, 0.31362841]))


def test_df_weights_golden(oracle, golden):
    g = golden("df")
    for i, (a, d) in enumerate(g["cases"]):
        assert np.array_equal(oracle.get_df_weight(a, dz=d), g[f"w_{i}"])
    for i, (n, d) in enumerate(g["scases"]):
        assert np.array_equal(oracle.get_simple_df_weight(n=int(n), dz=d), g[f"s_{i}"])


def test_fz2df_golden(oracle, golden):
    g = golden("df")
    assert np.allclose(oracle.Fz2df(g["Fz"], 0.1, 1800.0, 30000.0, 1.0), g["df1"], rtol=1e-12, atol=1e-12)
    assert np.allclose(oracle.Fz2df(g["Fz"], 0.1, 1800.0, 30300.0, 0.5), g["df2"], rtol=1e-12, atol=1e-12)
    assert np.allclose(oracle.Fz2df_numpy(g["Fz"], 0.1, 1800.0, 30000.0, 1.0), g["df1"], rtol=1e-13, atol=0)


def test_atoms_golden(oracle, golden):
    g = golden("atoms")
    FFp = g["species"][:, :3]
    iZ, R, Q = oracle.PBCAtoms(g["Zs"], g["Rs"], g["Qs"], g["lvec"][1], g["lvec"][2])
    assert np.array_equal(iZ, g["iZ9"]) and np.array_equal(R, g["R9"]) and np.array_equal(Q, g["Q9"])
    assert np.array_equal(oracle.getAtomsLJ(8, iZ, FFp), g["cLJ9"])
    REAs = oracle.getAtomsREA(8, g["Zs"], FFp)
    assert np.array_equal(REAs, g["REAs"])
    assert np.array_equal(oracle.REA2LJ(REAs), g["cLJ_rea"])
    Z3, xyz3, q3, c3 = oracle.PBCAtoms3D_np(g["Zs"], g["Rs"], g["Qs"], g["cLJ_rea"], g["lvec"][1:], npbc=(1, 1, 0))
    assert np.array_equal(Z3, g["Z3"]) and np.array_equal(xyz3, g["xyz3"]) and np.array_equal(q3, g["q3"]) and np.array_equal(c3, g["c3"])
    xT, yT, zT, lv = oracle.prepareScanGrids([0.0, 0.0, 5.0], [7.5, 6.0, 7.9], [0.25, 0.5, 0.1], [0.0, 0.0, 4.0])
    for a, b in ((xT, "xT"), (yT, "yT"), (zT, "zT"), (lv, "lvecScan")):
        assert np.array_equal(a, g[b])


def test_ff_grids_golden_bitexact(oracle, golden):
    g = golden("ff")
    n, lvec = g["n"], g["lvec"]
    F, E = oracle.lj_grid(n, lvec[1:], g["Rs0"], g["cLJs"], gridE=np.zeros(tuple(n)))
    assert np.array_equal(F, g["F_lj"]) and np.array_equal(E, g["E_lj"])
    for kind in (0, 1, 2):
        F, E = oracle.coulomb_grid(n, lvec[1:], g["Rs0"], g["kqq"], kind, gridE=np.zeros(tuple(n)))
        assert np.array_equal(F, g[f"F_el{kind}"]), kind
        assert np.array_equal(E, g[f"E_el{kind}"]), kind


def test_ff_subgrid_matches_full(oracle, golden):
    g = golden("ff")
    n, lvec = g["n"], g["lvec"]
    F, _ = oracle.ff_subgrid(n, lvec[1:], (3, 2, 5), (7, 9, 4), g["Rs0"], g["cLJs"], -1)
    assert np.array_equal(F, g["F_lj"][3:10, 2:11, 5:9])


def test_clamp_golden(oracle, golden):
    g = golden("clamp")
    G = g["G"].copy()
    oracle.limit_vec_field(G, 10.0)
    assert np.array_equal(G, g["Gc"])


def _relax_golden_setup(oracle, g):
    FFp = golden_species(oracle)
    lv = g["lvec"]
    iZ, R, Q = oracle.PBCAtoms(g["Zm"], g["Rm"], g["Qm"], lv[1], lv[2])
    cLJ = oracle.getAtomsLJ(8, iZ, FFp)
    n = g["n"]
    FFLJ, _ = oracle.lj_grid(n, lv[1:], R, cLJ)
    oracle.limit_vec_field(FFLJ, 10.0)
    FFel, _ = oracle.coulomb_grid(n, lv[1:], R, Q * oracle.CoulombConst, 0)
    oracle.limit_vec_field(FFel, 10.0)
    FF = FFLJ + FFel * float(g["charge"])
    tip = oracle.tip_params(4.0, float(g["krad"]) / -oracle.eVA_Nm, [0, 0, 0], np.array([g["klat"], g["klat"], 0.0]) / -oracle.eVA_Nm)
    prm = oracle.relax_param_vector(tip, maxIters=300, convF2=1e-8, dt=0.5, damping=0.1)
    xT, yT, zT, _ = oracle.prepareScanGrids(g["scanMin"], g["scanMax"], g["scanStep"], g["r0Probe"])
    return FF, prm, xT, yT, zT


def golden_species(oracle):
    from ppafm_gb300 import species

    t = species.loadSpecies()
    return np.array([(r[0], r[1], r[2]) for r in t])


def test_relax_golden_bitexact(oracle, golden):
    g = golden("relax")
    FF, prm, xT, yT, zT = _relax_golden_setup(oracle, g)
    fzs, PPpos, iters = oracle.relaxed_scan(g["n"], g["lvec"][1:], FF, prm, xT, yT, zT, g["lvec"][0])
    assert np.array_equal(fzs, g["fzs"])
    assert np.array_equal(PPpos, g["PPpos"])
    for (ix, iy), s in zip(g["picks"], g["itsum"]):
        assert iters[ix, iy].sum() == s
    assert np.allclose(oracle.Fz2df(fzs, 0.1, 1800.0, 30000.0, 1.0), g["df"], rtol=1e-12, atol=1e-12)


def test_fft_route_golden(oracle, golden):
    g = golden("fft")
    for tag in ("ortho", "skew_odd"):
        V, rho, lv = g[f"{tag}_V"], g[f"{tag}_rho"], g[f"{tag}_lvec"]
        fx, fy, fz, e = oracle.potential2forces_mem(V, lv, V.shape, rho=rho, doPot=True)
        for a, b in ((fx, "Fx"), (fy, "Fy"), (fz, "Fz"), (e, "E")):
            assert np.allclose(a, g[f"{tag}_{b}"], rtol=1e-10, atol=1e-10 * np.abs(g[f"{tag}_{b}"]).max()), (tag, b)
        fx, fy, fz, e = oracle.potential2forces_mem(V, lv, V.shape, sigma=0.7, multipole={"s": 1.0, "dz2": -0.3}, doPot=True)
        for a, b in ((fx, "mFx"), (fy, "mFy"), (fz, "mFz"), (e, "mE")):
            assert np.allclose(a, g[f"{tag}_{b}"], rtol=1e-10, atol=1e-10 * np.abs(g[f"{tag}_{b}"]).max()), (tag, b)


def test_poisson_gaussian_kat(oracle):
    """Known answer: the potential of a normalised Gaussian charge is q*k*erf(r/(sqrt2 s))/r
    away from the periodic images (no reference counterpart for the Poisson step)."""
    from math import erf

    L, n, s = 24.0, 96, 0.8
    x = (np.arange(n) * L / n) - L / 2
    X, Y, Zg = np.meshgrid(x, x, x, indexing="ij")
    r2 = X**2 + Y**2 + Zg**2
    rho = np.exp(-r2 / (2 * s * s)) / ((2 * np.pi) ** 1.5 * s**3)
    lv = np.array([[0, 0, 0], [L, 0, 0], [0, L, 0], [0, 0, L]], float)
    V = oracle.poisson_hartree(rho, lv)
    # compare potential differences (the periodic solution has an arbitrary offset and
    # a small image/background correction that is quadratic in r)
    i0 = n // 2
    for k in (3, 6, 10):
        r = x[i0 + k]
        exact = oracle.CoulombConst * (erf(r / (np.sqrt(2) * s)) / r)
        r1 = x[i0 + 3]
        exact1 = oracle.CoulombConst * (erf(r1 / (np.sqrt(2) * s)) / r1)
        num = V[i0 + k, i0, i0] - V[i0 + 3, i0, i0]
        ana = exact - exact1
        corr = oracle.CoulombConst * (2 * np.pi / 3) / L**3 * (r * r - r1 * r1)  # uniform neutralising background
        assert abs(num - (ana + corr)) < 2e-3 * abs(ana) + 1e-3, (k, num, ana + corr)


@pytest.mark.skipif(not __import__("oracle.oracle", fromlist=["x"]).reference_available(), reason="reference library not built here")
def test_oracle_vs_compiled_reference(oracle):
    rng = np.random.default_rng(7)
    ref = oracle.Reference()
    L = ref.L
    n = np.array([11, 13, 9], np.int32)
    cell = np.array([[6.0, 0.3, 0.0], [0.0, 6.5, 0.2], [0.1, 0.0, 7.0]])
    na = 17
    Rs = rng.uniform(-1, 7, size=(na, 3))
    cLJ = np.column_stack([rng.uniform(1, 10, na), rng.uniform(100, 3000, na)])
    kqq = rng.uniform(-3, 3, na)
    ref.set_grid(n, cell)
    for kind in (-1, 0, 1, 2):
        Fr = np.zeros(tuple(n) + (3,))
        Er = np.zeros(tuple(n))
        L.setFF_Fpointer(Fr)
        L.setFF_Epointer(Er)
        if kind < 0:
            L.getLennardJonesFF(na, Rs, cLJ)
            F, E = oracle.lj_grid(n, cell, Rs, cLJ, gridE=np.zeros(tuple(n)))
        else:
            L.getCoulombFF(na, Rs, kqq, kind)
            F, E = oracle.coulomb_grid(n, cell, Rs, kqq, kind, gridE=np.zeros(tuple(n)))
        assert np.array_equal(F, Fr) and np.array_equal(E, Er), kind
    FF = np.clip(Fr, -3, 3).copy()
    L.setFF_Fpointer(FF)
    for maxit, dt, alg, ps in ((300, 0.5, 1, 1), (50, 0.2, 0, 0), (0, 0.5, 1, -1), (1, 0.3, 1, 1)):
        L.setRelax(maxit, 1e-8, dt, 0.1)
        L.setFIRE(1.1, 0.5, 0.99)
        L.setTip(3.5, 15 / -oracle.eVA_Nm, np.array([0.2, -0.1, 0.0]), np.array([0.3, 0.3, 0]) / -oracle.eVA_Nm)
        tip = oracle.tip_params(3.5, 15 / -oracle.eVA_Nm, [0.2, -0.1, 0], np.array([0.3, 0.3, 0]) / -oracle.eVA_Nm)
        prm = oracle.relax_param_vector(tip, maxIters=maxit, convF2=1e-8, dt=dt, damping=0.1)
        rT = np.zeros((3, 4, 7, 3))
        rT[..., 0] = rng.uniform(0, 6, (3, 4, 1))
        rT[..., 1] = rng.uniform(0, 6, (3, 4, 1))
        rT[..., 2] = np.linspace(9.0, 8.2, 7)
        rs = np.zeros_like(rT)
        fs = np.zeros_like(rT)
        L.relaxTipStrokes_omp(3, 4, ps, alg, 7, rT, rs, fs, None)
        rs2, fs2, _, _ = oracle.relax_strokes(n, cell, FF, prm, rT, probeStart=ps, relaxAlg=alg)
        assert np.array_equal(rs, rs2) and np.array_equal(fs, fs2), (maxit, dt, alg, ps)
    # radial tip spline (forceRSpline): 7 knots (the reference's halving search skips some
    # intervals when the count is not a power of two), a stiff radial force around l0 = 3.5
    import ctypes

    class SplineParams(ctypes.Structure):
        _fields_ = [("rff_n", ctypes.c_int), ("rff_xs", ctypes.POINTER(ctypes.c_double)), ("rff_ydys", ctypes.POINTER(ctypes.c_double))]

    xs = np.linspace(2.0, 5.0, 7)
    k = 15 / -oracle.eVA_Nm
    ydys = np.ascontiguousarray(np.column_stack([k * (xs - 3.5) + 0.05 * (xs - 3.5) ** 3, k + 0.15 * (xs - 3.5) ** 2]))
    sp = SplineParams(len(xs), xs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ydys.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    L.setRelax(300, 1e-8, 0.5, 0.1)
    for ps in (1, 0):
        rs = np.zeros_like(rT)
        fs = np.zeros_like(rT)
        L.relaxTipStrokes_omp(3, 4, ps, 1, 7, rT, rs, fs, ctypes.cast(ctypes.pointer(sp), ctypes.c_void_p))
        prm = oracle.relax_param_vector(tip, maxIters=300, convF2=1e-8, dt=0.5, damping=0.1)
        rs2, fs2, _, _ = oracle.relax_strokes(n, cell, FF, prm, rT, probeStart=ps, relaxAlg=1, spline=(xs, ydys))
        assert np.array_equal(rs, rs2) and np.array_equal(fs, fs2), ps
        rs3, _, _, _ = oracle.relax_strokes(n, cell, FF, prm, rT, probeStart=ps, relaxAlg=1)
        assert not np.array_equal(rs3, rs2)  # the spline is in effect


def test_poisson_plane_wave_skewed_cell(oracle):
    """rho = cos(G.r), G a reciprocal-lattice vector of a skewed cell: V = 4 pi k cos(G.r)/|G|^2."""
    dims = (12, 10, 9)
    cell = np.array([[7.0, 0, 0], [1.5, 6.0, 0], [0.3, 0.4, 5.5]])
    lv = np.vstack([np.zeros(3), cell])
    Bm = 2 * np.pi * np.linalg.inv(cell).T
    for m in ((1, 0, 0), (2, -1, 3), (0, 4, -2)):
        Gv = m[0] * Bm[0] + m[1] * Bm[1] + m[2] * Bm[2]
        f = np.stack(np.meshgrid(*[np.arange(dims[k]) / dims[k] for k in range(3)], indexing="ij"), axis=-1)
        rho = np.cos((f @ cell) @ Gv)
        V = oracle.poisson_hartree(rho, lv)
        assert np.allclose(V, 4 * np.pi * oracle.CoulombConst * rho / (Gv @ Gv), atol=1e-12 * np.abs(V).max())


def test_gaussian_density_kat(oracle):
    """A normalised Gaussian on a grid node: peak w/((2 pi)^1.5 s^3), integral w, periodic wrap."""
    L, n, s, w = 10.0, 50, 0.7, 3.0
    lv = np.array([[0.0, 0, 0], [L, 0, 0], [0, L, 0], [0, 0, L]])
    rho = oracle.gaussian_density((n, n, n), lv, [[0.0, 0.0, 0.2 * 9, s, w]])
    k = 9  # z index of the atom
    assert np.isclose(rho[0, 0, k], w / ((2 * np.pi) ** 1.5 * s**3), rtol=1e-12)
    assert np.isclose(rho.sum() * (L / n) ** 3, w, rtol=1e-6)
    assert np.isclose(rho[1, 0, k], rho[-1, 0, k], rtol=1e-12)  # minimum image across x = 0


def test_mlp_oracle_gradient_finite_differences():
    """The float64 restatement's backward against central differences of its loss."""
    from oracle import mlp_oracle as MO

    rng = np.random.default_rng(0)
    P = rng.normal(0, 0.2, MO.NPARAM)
    X = rng.normal(0, 1, (5, MO.IN))
    X[:, MO.IN - 6 :] = 0
    T = rng.normal(0, 1, (5, 4))
    _, G = MO.loss_and_grad(P, X, T, bf=False)
    for i in rng.choice(MO.NPARAM, 40, replace=False):
        d = np.zeros_like(P)
        d[i] = 1e-6
        fd = (MO.loss_and_grad(P + d, X, T, False)[0] - MO.loss_and_grad(P - d, X, T, False)[0]) / 2e-6
        assert abs(fd - G[i]) <= 1e-5 * (abs(G[i]) + 1e-3)


def test_interp_at_known_answers(oracle):
    """interp_at restatement: node values at nodes, exact on a linear function inside the grid,
    and the periodic wrap between the last and the first node."""
    n = (8, 6, 10)
    lv = np.array([[-1.0, 0.5, 2.0], [4.0, 0, 0], [0, 3.0, 0], [0, 0, 5.0]])
    h = np.diag(lv[1:]) / n
    g = np.stack(np.meshgrid(*[lv[0][k] + np.arange(n[k]) * h[k] for k in range(3)], indexing="ij"), axis=-1)
    lin = (0.3 * g[..., 0] - 0.7 * g[..., 1] + 0.2 * g[..., 2]).astype(np.float32)
    # at the nodes themselves
    out = oracle.interp_at(lin, lv, n, lv[0], np.diag(h))
    assert np.allclose(out, lin, atol=1e-5)
    # half-way points of the interior: the mean of the neighbours, i.e. the linear function
    o2 = lv[0] + 0.5 * h
    out = oracle.interp_at(lin, lv, (7, 5, 9), o2, np.diag(h))
    want = 0.3 * (g[:7, :5, :9, 0] + 0.5 * h[0]) - 0.7 * (g[:7, :5, :9, 1] + 0.5 * h[1]) + 0.2 * (g[:7, :5, :9, 2] + 0.5 * h[2])
    assert np.allclose(out, want, atol=1e-5)
    # periodic wrap: a quarter step before the origin along x mixes node n-1 (1/4) and node 0 (3/4)
    o3 = lv[0] - np.array([0.25 * h[0], 0, 0])
    out = oracle.interp_at(lin, lv, (1, n[1], n[2]), o3, np.diag(h))
    assert np.allclose(out[0], 0.25 * lin[-1] + 0.75 * lin[0], atol=1e-5)


def test_hartree_tip_density_plane_wave(oracle):
    """Hartree route with a tip density: V = cos(G.r) on the force-field grid correlated with an
    s-density of charge c gives E = c exp(-s^2 |G|^2 / 2) cos(G.r) and F = -grad E by centred
    differences."""
    n = (16, 16, 16)
    L, h, s, c = 8.0, 0.5, 0.7, -0.3
    lv = np.array([[0.0, 0, 0], [L, 0, 0], [0, L, 0], [0, 0, L]])
    x = np.arange(n[0]) * h
    G = 2 * np.pi / L
    pot = np.broadcast_to(np.cos(G * x)[:, None, None], n).astype(np.float32)
    FE = oracle.hartree_ff(n, lv, pot, lv, {"s": c}, s, np.zeros((0, 3)), np.zeros((0, 2)), np.eye(3), np.zeros(3))
    FE = FE.transpose(2, 1, 0, 3)  # -> [nx, ny, nz, 4]
    damp = c * np.exp(-(s * G) ** 2 / 2)
    E = damp * np.cos(G * x)
    Fx = damp * np.sin(G * x) * np.sin(G * h) / h
    assert np.allclose(FE[:, 3, 5, 3], E, atol=1e-6)
    assert np.allclose(FE[:, 3, 5, 0], Fx, atol=1e-6)
    assert np.abs(FE[..., 1:3]).max() < 1e-6


def test_hartree_point_charge_tip_known_answers(oracle):
    """Hartree route with the point-charge tip (no atoms): the field of V on the force-field grid
    sampled at the tip charges' heights (periodically on the force-field grid).  Same grid:
    periodic centred differences of a plane-wave potential; other grid: the exact gradient of
    a linear potential (interpolated at +-0.05 A inside the potential's grid)."""
    n = (16, 12, 20)
    lv = np.array([[0.0, 0, 0], [8.0, 0, 0], [0, 6.0, 0], [0, 0, 10.0]])
    h = 0.5
    kx, kz = 2 * np.pi / 8.0, 2 * 2 * np.pi / 10.0
    x, z = np.arange(n[0]) * h, np.arange(n[2]) * h
    V = (np.sin(kx * x)[:, None, None] + 0.5 * np.cos(kz * z)[None, None, :]) * np.ones(n)
    Qs, QZs = [1.0, -2.0, 0, 0], [0.0, 1.0, 0, 0]
    none = (np.zeros((0, 3)), np.zeros((0, 2)))
    FE = oracle.hartree_ff_point_charges(n, lv, V.astype(np.float32), lv, *none, Qs, QZs).transpose(2, 1, 0, 3)

    def field(zs):
        ex = -np.cos(kx * x)[:, None, None] * np.sin(kx * h) / h * np.ones(n)
        ez = 0.5 * np.sin(kz * zs)[None, None, :] * np.sin(kz * h) / h * np.ones(n)
        w = np.sin(kx * x)[:, None, None] + 0.5 * np.cos(kz * zs)[None, None, :]
        return ex, ez, w * np.ones(n)

    e0, e1 = field(z), field(z + 1.0)  # QZ = 1 A = two steps (periodic)
    assert np.allclose(FE[..., 0], e0[0] - 2 * e1[0], atol=1e-5)
    assert np.abs(FE[..., 1]).max() < 1e-5
    assert np.allclose(FE[..., 2], e0[1] - 2 * e1[1], atol=1e-5)
    assert np.allclose(FE[..., 3], e0[2] - 2 * e1[2], atol=1e-5)
    # a linear potential on a larger grid of its own: field (-a, -b, -c), so F = (1 - 2)(-a, -b, -c)
    a, b, cz = 0.3, -0.2, 0.5
    lvp = np.array([[-1.0, -1.0, -2.0], [12.0, 0, 0], [0, 10.0, 0], [0, 0, 16.0]])
    npot = (24, 20, 32)
    gp = [lvp[0][k] + np.arange(npot[k]) * 0.5 for k in range(3)]
    Vp = (a * gp[0][:, None, None] + b * gp[1][None, :, None] + cz * gp[2][None, None, :]).astype(np.float32)
    FE = oracle.hartree_ff_point_charges(n, lv, Vp, lvp, *none, Qs, QZs).transpose(2, 1, 0, 3)
    assert np.allclose(FE[..., 0], a, atol=2e-3) and np.allclose(FE[..., 1], b, atol=2e-3) and np.allclose(FE[..., 2], cz, atol=2e-3)
    # the tip charges sample the field on the force-field grid, periodic over its cell
    def Vff(zs):
        return a * x[:, None, None] + b * (np.arange(n[1]) * h)[None, :, None] + cz * zs[None, None, :]

    assert np.allclose(FE[..., 3], Vff(z) - 2 * Vff((z + 1.0) % 10.0), atol=1e-4)


def _gaussian_on(shape, lvec):
    """A unit-width Gaussian at the origin of a periodic grid (wrapped), the form of the
    reference's tests/test_datagrid.py make_gaussian."""
    xyz = np.stack(np.meshgrid(*[np.linspace(-0.5, 0.5, shape[i], endpoint=False) for i in range(3)], indexing="ij"), axis=-1)
    xyz = xyz.dot(np.asarray(lvec, np.float64)[1:].T)
    a = np.exp(-0.5 * (xyz**2).sum(axis=-1))
    return np.roll(a, (-np.array(shape) / 2).astype(int), axis=(0, 1, 2))


def test_interp_tip_at_gaussian(oracle):
    """The tip-density resampling restatement against the analytic Gaussian on the new grid
    (the reference's test_tip_interp at smaller sizes), and zero beyond half of the input cell."""
    lv1 = np.array([[0.0, 0, 0], [10, 0, 0], [0, 10, 0], [0, 0, 10]])
    lv2 = np.array([[0.0, 0, 0], [12, 0, 0], [0, 8, 0], [0, 0, 15]])
    g1 = _gaussian_on((100, 100, 100), lv1).astype(np.float32)
    out = oracle.interp_tip_at(g1, lv1, (72, 48, 90), lv2)
    g2 = _gaussian_on((72, 48, 90), lv2)
    assert np.allclose(out, g2, atol=3e-3, rtol=3e-3)
    # beyond |x| > 5 A (half of the 10 A input cell) along x: zero; the 12 A grid has such points
    x = np.arange(72)
    x = np.where(x > 36, x - 72, x) * (12 / 72)
    assert (out[np.abs(x) > 5.0 + 1e-6] == 0).all()


def test_hartree_pz_tip_density_sign(oracle):
    """An odd tip density fixes correlation against convolution: V = cos(G z) with a pz
    density c (z / s) g(r) gives E = -c s G exp(-s^2 G^2 / 2) sin(G z) (a convolution would give
    the opposite sign)."""
    n = (8, 8, 20)
    lv = np.array([[0.0, 0, 0], [4.0, 0, 0], [0, 4.0, 0], [0, 0, 10.0]])
    h, s, c = 0.5, 0.7, 0.2
    z = np.arange(n[2]) * h
    G = 2 * 2 * np.pi / 10.0
    pot = np.broadcast_to(np.cos(G * z)[None, None, :], n).astype(np.float32)
    FE = oracle.hartree_ff(n, lv, pot, lv, {"pz": c}, s, np.zeros((0, 3)), np.zeros((0, 2)), np.eye(3), np.zeros(3)).transpose(2, 1, 0, 3)
    a = -c * s * G * np.exp(-(s * G) ** 2 / 2)
    assert np.allclose(FE[2, 3, :, 3], a * np.sin(G * z), atol=1e-6)
    assert np.allclose(FE[2, 3, :, 2], -a * np.cos(G * z) * np.sin(G * h) / h, atol=1e-6)
