"""Host side of the ML generator: the xyz reader/writer (ppafm/io.py:19-110, the cases of
the reference's tests/test_io.py) and the rotation helpers of ppafm/ml/Generator.py."""

import numpy as np
import pytest


def test_xyz_roundtrip(tmp_path):
    from ppafm_gb300.io import loadXYZ, saveXYZ
    from ppafm_gb300.species import SYMBOL_TO_Z

    rng = np.random.default_rng(0)
    N = 20
    xyzs = 10 * rng.random((N, 3))
    Zs = rng.integers(1, 87, N)
    qs = (rng.random(N) - 0.5) / N
    f = tmp_path / "io_test.xyz"
    saveXYZ(f, xyzs, Zs, qs, "test comment")
    xyzs_, Zs_, qs_, comment_ = loadXYZ(f)
    assert np.allclose(xyzs, xyzs_, atol=1e-6) and np.array_equal(Zs, Zs_) and np.allclose(qs, qs_, atol=1e-6)
    assert comment_ == "test comment"
    saveXYZ(f, xyzs, Zs, qs=None)
    _, _, qs_, _ = loadXYZ(f)
    assert np.all(qs_ == 0)
    # element given by its atomic number
    f.write_text("2\n\n6 0 0 0\nO 1 2 3 -0.5\n".replace("6 0 0 0", "6 0 0 0 0.5"))
    x, Z, q, _ = loadXYZ(f)
    assert list(Z) == [6, SYMBOL_TO_Z["O"]] and np.allclose(q, [0.5, -0.5]) and np.allclose(x[1], [1, 2, 3])


def test_xyz_bad_files(tmp_path):
    from ppafm_gb300.io import loadXYZ

    f = tmp_path / "bad.xyz"
    f.write_text("two\n\nC 0 0 0\n")
    with pytest.raises(ValueError, match="number of atoms"):
        loadXYZ(f)
    f.write_text("1\n\nC 0 0\n")
    with pytest.raises(ValueError, match="interpret"):
        loadXYZ(f)


def test_ase_charge_column():
    from ppafm_gb300.io import _charges

    rng = np.random.default_rng(1)
    extra = (rng.random((10, 2)) - 0.5) / 10
    cols = [[str(e[0]), str(e[1])] for e in extra]
    assert np.allclose(_charges('Properties=species:S:1:pos:R:3:tags:I:1:initial_charges:R:1 pbc="F F F"', cols), extra[:, 1])
    assert np.allclose(_charges('Properties=species:S:1:pos:R:3:initial_charges:R:1:tags:I:1 pbc="F F F"', cols), extra[:, 0])
    assert np.all(_charges('Properties=species:S:1:pos:R:3:tags:I:1 pbc="F F F"', [[c[0]] for c in cols]) == 0)
    assert np.allclose(_charges("plain comment", cols), extra[:, 0])


def test_rotation_helpers():
    from ppafm_gb300.ml.Generator import getRandomUniformDisk, rotate, sortRotationsByEntropy

    np.random.seed(0)
    pts = np.array([getRandomUniformDisk() for _ in range(200)])
    assert np.all(np.hypot(pts[:, 0], pts[:, 1]) <= 1.0)
    xyz = np.random.rand(7, 3)
    Rz = np.array([[0.0, -1, 0], [1, 0, 0], [0, 0, 1]])
    out = rotate(xyz, [np.eye(3), Rz])
    assert np.allclose(out[0], xyz) and np.allclose(out[1][:, 0], -xyz[:, 1])
    flat = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    up, side = np.eye(3), np.array([[0.0, 0, 1], [0, 1, 0], [1, 0, 0]])
    # looking down z every atom is at the top (entropy 3); down x only one is
    assert sortRotationsByEntropy(flat, [side, up])[0] is up


def _xsf_inputs():
    import os

    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "xsf", "inputs.npz"))
    return d["S"], d["V"], d["lvec"]


def test_xsf_files_match_the_reference(tmp_path):
    """Byte-identical XSF files (scalar, vector, default orthogonal cell) and identical loads of
    the files the reference wrote (tests/golden/xsf, made by tests/golden/make_golden.py)."""
    import os

    from ppafm_gb300 import io as pio

    g = os.path.join(os.path.dirname(__file__), "golden", "xsf")
    S, V, lvec = _xsf_inputs()
    pio.saveXSFData(tmp_path / "scal.xsf", S, lvec)
    assert (tmp_path / "scal.xsf").read_text() == open(os.path.join(g, "scal.xsf")).read()
    pio.saveXSFData(tmp_path / "ortho.xsf", S[:, :, :2], dd=[0.1, 0.2, 0.3])
    assert (tmp_path / "ortho.xsf").read_text() == open(os.path.join(g, "ortho.xsf")).read()
    pio.save_vec_field(str(tmp_path / "vec"), V, lvec, data_format="xsf")
    for c in "xyz":
        assert (tmp_path / f"vec_{c}.xsf").read_text() == open(os.path.join(g, f"vec_{c}.xsf")).read()
    F, lv, n, head = pio.loadXSFData(os.path.join(g, "scal.xsf"))
    assert np.allclose(F, S, rtol=1e-5, atol=1e-5) and np.allclose(lv, lvec) and list(n) == list(S.shape)
    assert any("BEGIN_DATAGRID_3D" in h for h in head)
    FF, lv, n, _ = pio.load_vec_field(os.path.join(g, "vec"), "xsf")
    assert FF.shape == V.shape and np.allclose(FF, V, rtol=1e-5, atol=1e-5)
    FF, lv, n, info = pio.load_vec_field(os.path.join(g, "vec"), "npy")
    assert np.array_equal(FF, V) and np.array_equal(lv, lvec) and np.array_equal(info[1], lvec)
    D, lv, n, info = pio.load_scal_field(os.path.join(g, "scal"), "npy")
    assert np.array_equal(D, S)
    # npz written here loads with the same keys
    pio.save_vec_field(str(tmp_path / "v2"), V, lvec, data_format="npy")
    ref = np.load(os.path.join(g, "vec.npz"))
    got = np.load(tmp_path / "v2.npz")
    assert sorted(ref.files) == sorted(got.files) and all(np.array_equal(ref[k], got[k]) for k in ref.files)
    with pytest.raises(ValueError):
        pio.load_vec_field(str(tmp_path / "v2"), "cube")


def test_limit_vec_field_golden(golden):
    from ppafm_gb300 import io as pio

    g = golden("clamp")
    G = g["G"].copy()
    pio.limit_vec_field(G, Fmax=10.0)
    assert np.array_equal(G, g["Gc"])
