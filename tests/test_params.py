"""Simulation parameters (common.PpafmParameters, restating ppafm/common.py:26-160): the
reference's own test (tests/test_common.py test_ppafm_parameters) on its parameter file, with
the parsed values and the defaults compared to what the reference itself produced
(tests/golden/params/, made by tests/golden/make_golden.py)."""

import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "params")


def test_ppafm_parameters(tmp_path):
    from ppafm_gb300 import common

    ref = json.load(open(os.path.join(GOLD, "parsed.json")))
    p_default = common.PpafmParameters()
    assert p_default.model_dump() == ref["default"]
    assert p_default.PBC is True and p_default.nPBC == [1, 1, 1] and p_default.probeType == "O"
    assert p_default.gridN == [-1, -1, -1] and np.isclose(p_default.klat, 0.5) and p_default.vdWDampKind == 2

    p_ini = common.PpafmParameters.from_file(os.path.join(GOLD, "test_params.ini"))
    assert p_ini.model_dump() == ref["parsed"]
    assert p_ini.PBC is False and p_ini.nPBC == [2, 3, 4] and p_ini.probeType == "Xe"
    assert np.isclose(p_ini.charge, 0.5) and p_ini.ffModel == "Morse" and np.isclose(p_ini.gridN, [10, 20, 30]).all()
    assert np.isclose(p_ini.scanStep, [0.1, 0.2, 0.3]).all() and np.isclose(p_ini.Amplitude, 8.0) and p_ini.vdWDampKind == 3

    p_ini.to_file(tmp_path / "test_params.toml")
    assert common.PpafmParameters.from_file(tmp_path / "test_params.toml") == p_ini

    # gridN from the cell when the file does not give it; unknown keys and bad values raise
    (tmp_path / "a.ini").write_text("gridA 12.0 0 0\ngridB 0 8.5 0\ngridC 0 0 20.0\n")
    assert common.PpafmParameters.from_file(tmp_path / "a.ini").gridN == [120, 85, 200]
    (tmp_path / "b.ini").write_text("nosuchkey 1\n")
    with pytest.raises(ValueError):
        common.PpafmParameters.from_file(tmp_path / "b.ini")
    (tmp_path / "c.ini").write_text("scanMin 1.0 2.0\n")
    with pytest.raises(ValueError):
        common.PpafmParameters.from_file(tmp_path / "c.ini")
    with pytest.raises(ValueError):
        common.PpafmParameters.from_file(tmp_path / "missing.ini")


def test_parameters_drive_the_host_helpers():
    """A PpafmParameters object where the pipeline functions take parameters (attribute access)."""
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import common

    p = common.PpafmParameters(probeType="8", charge=-0.05, r0Probe=[0.0, 0.0, 4.0], klat=0.25, krad=20.0)
    assert HL._get(p, "probeType") == "8" and HL._get(p, "charge") == -0.05
    v = HL.tip_vector(p, dict(maxIters=300, convF2=1e-8, dt=0.5, damping=0.1))
    assert np.isfinite(v).all()


def test_afmulator_parameter_files(tmp_path):
    """AFMulator.from_params / save_params / load_params (AFMulator.py:483-565): the values a
    params.ini sets, a save and reload, and the scan-window check (no GPU work involved)."""
    import warnings

    from ppafm_gb300.AFMulator import AFMulator

    (tmp_path / "params.ini").write_text(
        "probeType 8\ntip dz2\ncharge -0.1\nsigma 0.71\nstiffness 0.25 0.25 20.0\nr0Probe 0.0 0.0 3.0\n"
        "PBC True\nnPBC 1 1 0\ngridA 16.0 0 0\ngridB 0 16.0 0\ngridC 0 0 20.0\n"
        "scanMin 2.0 2.0 7.0\nscanMax 14.0 14.0 10.0\nscanStep 0.1 0.1 0.1\nAmplitude 1.0\n"
    )
    afm = AFMulator.from_params(tmp_path / "params.ini")
    assert afm.iZPP == 8 and afm.rho == {"dz2": -0.1} and np.isclose(afm.sigma, 0.71)
    assert afm.scan_dim == (121, 121, 30) and afm.df_steps == 10 and tuple(afm.npbc) == (1, 1, 0)
    assert np.allclose(afm.sample_lvec, np.diag([16.0, 16.0, 20.0]))
    assert np.allclose(afm.stiffness * -16.0217662, [0.25, 0.25, 0.0, 20.0], rtol=1e-6)
    afm.save_params(tmp_path / "saved.ini")
    b = AFMulator.from_params(tmp_path / "saved.ini")
    assert b.scan_dim == afm.scan_dim and b.df_steps == afm.df_steps and b.rho == afm.rho
    assert np.allclose(b.lvec, afm.lvec) and np.array_equal(b.nDim, afm.nDim)
    assert np.allclose(b.stiffness, afm.stiffness, rtol=1e-6) and np.allclose(b.tipR0, afm.tipR0)
    c = AFMulator()
    c.load_params(tmp_path / "saved.ini")
    assert c.scan_dim == afm.scan_dim and np.allclose(c.lvec, afm.lvec) and c.rho == afm.rho
    # scan window reaching past the non-periodic z edge of the force-field grid
    c.setScanWindow(((2.0, 2.0, 7.0), (14.0, 14.0, 60.0)), (121, 121, 30))
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        c.check_scan_window()
    assert any("boundary of the force-field grid" in str(x.message) for x in w)
    # a symbol as probe type
    (tmp_path / "xe.ini").write_text("probeType Xe\n")
    assert AFMulator.from_params(tmp_path / "xe.ini").iZPP == 54
    # no plotting: plot_images saves the stack (heights top-down) with its tip heights
    X = np.arange(121 * 121 * 21, dtype=np.float32).reshape(121, 121, 21)
    with warnings.catch_warnings(record=True):
        warnings.simplefilter("always")
        afm.plot_images(X, outdir=str(tmp_path / "img"))
    z = np.load(tmp_path / "img" / "df.npz")
    assert np.array_equal(z["X"], X[:, :, ::-1]) and len(z["zTips"]) == 21 and np.isclose(z["zTips"][0], 7.0 + afm.amplitude / 2)
    afm.setRhoDelta(None)
    with pytest.raises(NotImplementedError):
        afm.setRhoDelta({"s": 1.0})
    with pytest.raises(NotImplementedError):
        afm.setBPauli(1.2)


def test_load_geometry_vs_reference():
    """io.loadGeometry (io.py:398-503) on an xyz with charges, a POSCAR in direct coordinates and
    an FHI-aims geometry.in: atoms, grid size, lattice and the parameters it sets, as the
    reference parsed them (tests/golden/stages/geometry.json)."""
    from ppafm_gb300 import common, io

    gold = os.path.join(HERE, "golden", "stages")
    ref = json.load(open(os.path.join(gold, "geometry.json")))
    for name, r in ref.items():
        p = common.PpafmParameters.from_file(os.path.join(gold, "params.ini"))
        atoms, nD, lv = io.loadGeometry(os.path.join(gold, name), parameters=p)
        assert [int(z) for z in atoms[0]] == [int(z) for z in r["atoms"][0]], name
        for k in range(1, 5):
            assert np.allclose(atoms[k], r["atoms"][k], rtol=1e-12, atol=1e-12), (name, k)
        assert list(nD) == r["nDim"] and np.allclose(lv, r["lvec"], rtol=1e-7) and p.PBC == r["PBC"], name
        assert [int(x) for x in p.gridN] == r["gridN"]
        assert np.allclose([p.gridO, p.gridA, p.gridB, p.gridC], r["lvec"], rtol=1e-7)
    # a zero cell vector: made to enclose the scan window with 3 A padding, PBC off
    p = common.PpafmParameters.from_file(os.path.join(gold, "params.ini"))
    p.gridC = [0.0, 0.0, 0.0]
    _, nD, lv = io.loadGeometry(os.path.join(gold, "mol.xyz"), parameters=p)
    assert p.PBC is False and np.isclose(lv[3, 2], (7.0 - 4.0) - (5.0 - 4.0) + 6.0) and np.isclose(lv[0, 2], 5.0 - 4.0 - 3.0)
    head = io.primcoords2Xsf([6, 8], [[0.0, 1.0], [0.5, 1.5], [0.25, 0.75]], lv)
    assert "PRIMCOORD\n2 1\n6 0.000000 0.500000 0.250000\n8 1.000000 1.500000 0.750000\n" in head


def test_common_helpers_vs_reference():
    """Rotations, sphere frames, image replication, wrapping and pair parameters of
    ppafm/common.py against the reference's own outputs (tests/golden/helpers.npz), and the
    reference's test_sphere_tangent_space vectors."""
    from ppafm_gb300 import common as C

    g = np.load(os.path.join(HERE, "golden", "helpers.npz"))
    FF = C.loadSpecies()
    assert np.allclose(C.rotation_matrix(g["axis"], 0.7), g["rot"], rtol=0, atol=1e-14)
    rots = C.genRotations(g["axis"], g["thetas"])
    assert np.allclose(rots, g["rots"], rtol=0, atol=1e-14)
    assert np.allclose(C.sphereTangentSpace(11), g["sphere"], rtol=0, atol=1e-14)
    assert np.allclose(
        C.sphereTangentSpace(2),
        [[[-0.0, 1.0, 0.0], [-0.5, -0.0, 0.8660254], [0.8660254, 0.0, 0.5]], [[-0.67549029, -0.73736888, 0.0], [-0.36868444, 0.33774515, 0.8660254], [-0.63858018, 0.58499175, -0.5]]],
    )
    i, h = C.maxAlongDir(g["Rs"], g["hdir"])
    i2, h2, e2 = C.maxAlongDirEntropy(g["Rs"], g["hdir"], beta=0.7)
    assert np.allclose([i, h, i2, h2, e2], g["maxdir"], rtol=1e-14)
    z, r, q, c = C.multRot(g["Zs"], g["Rs"], g["Qs"], g["cLJs"], rots, cog=(0.5, -0.5, 0.2))
    assert np.array_equal(z, g["mr_Z"]) and np.allclose(r, g["mr_R"], rtol=0, atol=1e-13) and np.array_equal(q, g["mr_Q"]) and np.array_equal(c, g["mr_c"])
    z, r, q, c = C.PBCAtoms3D(g["Zs"], g["Rs"], g["Qs"], g["cLJs"], g["lvec3"], npbc=[1, 1, 0])
    assert np.array_equal(z, g["p3_Z"]) and np.allclose(r, g["p3_R"], rtol=0, atol=1e-13) and np.array_equal(q, g["p3_Q"]) and np.array_equal(c, g["p3_c"])
    W = g["Rs"].copy()
    C.wrapAtomsCell(W, 0.25, -0.1, g["lvec3"][0], g["lvec3"][1])
    assert np.allclose(W, g["wrapped"], rtol=0, atol=1e-12)
    assert np.array_equal(C.getSampleAtomsREA(g["Zs"], FF), g["sREA"])
    assert np.array_equal(C.getAtomsRE(8, g["Zs"], FF), g["RE"])
    R = np.array(C.makeRotJitter())
    assert R.shape == (50, 3, 3) and np.allclose(R @ R.transpose(0, 2, 1), np.eye(3), atol=1e-12)


def test_cube_and_xsf_geometry_files(tmp_path):
    """Gaussian cube reading (io.py:291-395, 643-675) against the reference's readers on a
    skewed-voxel file (tests/golden/cube/), loadGeometry of it, and the XSF geometry writer
    with the PRIMCOORD header parser."""
    from ppafm_gb300 import common, io

    gold = os.path.join(HERE, "golden", "cube")
    g = np.load(os.path.join(gold, "parsed.npz"))
    path = os.path.join(gold, "dens.cube")
    F, lvec, nD, head = io.loadCUBE(path)
    assert np.array_equal(F, g["F"]) and np.array_equal(lvec, g["lvec"]) and list(nD) == list(g["nD"])
    Fx, _, nDx, _ = io.loadCUBE(path, xyz_order=True)
    assert np.array_equal(Fx, g["Fx"]) and list(nDx) == list(g["nDx"])
    assert np.array_equal(np.array(io.loadAtomsCUBE(path), dtype=np.float64), g["atoms"])
    assert np.array_equal(np.array(io.loadCellCUBE(path)), g["cell"]) and io.loadNCUBE(path) == list(g["ncube"])
    p = common.PpafmParameters()
    atoms, n, lv = io.loadGeometry(path, parameters=p)
    assert np.array_equal(np.array(atoms, dtype=np.float64), g["g_atoms"]) and np.array_equal(np.array(n), g["g_n"]) and np.array_equal(lv, g["g_lvec"])
    # XSF geometry: written, read back by loadXSFGeom and by the header parser
    xyz = np.array([[0.5, 1.0, 1.5], [2.0, -1.0, 0.25]])
    cell = np.diag([6.0, 7.0, 8.0])
    io.saveGeomXSF(str(tmp_path / "g.xsf"), [6, 8], xyz, cell)
    with open(tmp_path / "g.xsf", "a") as f:
        f.write("BEGIN_BLOCK_DATAGRID_3D\nx\nBEGIN_DATAGRID_3D_x\n2 2 2\n0 0 0\n6 0 0\n0 7 0\n0 0 8\n")
    (Zs, x, y, z, _), _, _ = io.loadXSFGeom(str(tmp_path / "g.xsf"))
    assert Zs == [6, 8] and np.allclose(np.column_stack([x, y, z]), xyz)
    Zh, Rh = io.getFromHead_PRIMCOORD(open(tmp_path / "g.xsf").read().split("\n"))
    assert list(Zh) == [6, 8] and np.allclose(Rh, xyz)


def test_species_table_is_the_reference_default():
    """The built-in per-element table equals the reference's defaults/atomtypes.ini as the
    reference loads it (all 118 species), and loadSpeciesLines reads the same format."""
    from ppafm_gb300 import common

    g = np.load(os.path.join(HERE, "golden", "params", "species.npz"))
    sp = common.loadSpecies()
    for k in ("rmin", "epsilon", "alpha", "atom", "symbol"):
        assert np.array_equal(sp[k], g[k]), k
    lines = [f"{r} {e} {a} {z} {s.decode()}\n" for r, e, a, z, s in zip(g["rmin"], g["epsilon"], g["alpha"], g["atom"], g["symbol"])]
    sp2 = common.loadSpeciesLines(lines + ["short line\n"])
    assert len(sp2) == len(sp) and np.array_equal(sp2["rmin"], sp["rmin"]) and np.array_equal(sp2["symbol"], sp["symbol"])


def test_wsxm_writers(tmp_path):
    """WSxM ASCII XYZ slices (io.py:680-706): the header, then x, y and the value at every
    pixel of the slice in meshgrid order, the layout of the reference's writer."""
    from ppafm_gb300 import io

    data = np.arange(4 * 3 * 2, dtype=np.float64).reshape(4, 3, 2)
    io.saveWSxM_3D(str(tmp_path / "df"), data, [0.0, 3.0, 1.0, 2.0])
    lines = open(tmp_path / "df_001.xyz").read().split("\n")
    assert lines[:4] == ["WSxM file copyright Nanotec Electronica", "WSxM ASCII XYZ file", "X[A]  Y[A]  df[Hz]", ""]
    v = np.loadtxt(tmp_path / "df_001.xyz", skiprows=4)
    Xs, Ys = np.meshgrid(np.linspace(0, 3, 4), np.linspace(1, 2, 3))
    assert np.allclose(v[:, 0], Xs.ravel()) and np.allclose(v[:, 1], Ys.ravel()) and np.allclose(v[:, 2], data[:, :, 1].ravel())
