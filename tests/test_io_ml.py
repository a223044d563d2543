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
