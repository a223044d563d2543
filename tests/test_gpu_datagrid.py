"""The grid classes of the Hartree route on the GPU (ppafm_gb300.field, restating
ppafm/ocl/field.py:115-704): the reference's own tests/test_datagrid.py (power_positive against
numpy, the tip-density resampling against an analytic Gaussian, hard and soft clamp, add_mult),
the interpolations and the gradient against the oracle, XSF round trip, and the AFMulator with a
tip density given on a grid other than the force field's."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _eye_lvec():
    return np.concatenate([np.zeros((1, 3)), np.eye(3)], axis=0)


def test_power_positive(gpulib):
    from ppafm_gb300.field import DataGrid

    rng = np.random.default_rng(0)
    p = 1.5
    a = (rng.random((120, 110, 100)) - 0.25).astype(np.float32)
    data = DataGrid(a, _eye_lvec())
    b = a.astype(np.float64)
    Q = b.sum()
    b[b < 0] = 0
    b *= Q / b.sum()  # handleNegativeDensity
    want = b**p
    out = data.power_positive(p=p, in_place=False)
    assert np.allclose(out.array, want, rtol=1e-5, atol=1e-6)
    assert np.array_equal(data.array, a)  # not in place: the input is unchanged
    data.power_positive(p=p, in_place=True)
    assert np.allclose(data.array, want, rtol=1e-5, atol=1e-6)
    raw = DataGrid(a, _eye_lvec()).power_positive(p=p, normalize=False, in_place=False)
    assert np.allclose(raw.array, np.maximum(a, 0).astype(np.float64) ** p, rtol=1e-5, atol=1e-6)


def test_tip_interp(gpulib, oracle):
    from ppafm_gb300.field import TipDensity
    from tests.test_oracle import _gaussian_on

    lv1 = np.array([[0, 0, 0], [10, 0, 0], [0, 10, 0], [0, 0, 10]], dtype=np.float64)
    rho = TipDensity(_gaussian_on((200, 200, 200), lv1), lv1)
    lv2 = np.array([[0, 0, 0], [12, 0, 0], [0, 8, 0], [0, 0, 15]], dtype=np.float64)
    out = rho.interp_at(lv2, (150, 100, 140))
    assert isinstance(out, TipDensity) and out.shape == (150, 100, 140)
    assert np.allclose(out.array, _gaussian_on((150, 100, 140), lv2), atol=1e-3, rtol=1e-3)  # the reference's bar
    want = oracle.interp_tip_at(rho.array, lv1, (150, 100, 140), lv2)
    assert np.abs(out.array - want).max() <= 1e-5


def test_clamp(gpulib):
    from ppafm_gb300.field import DataGrid

    array = np.array([-1.0, 0.0, 1.0, 2.0])[None, None]
    g = DataGrid(array, _eye_lvec())
    new = g.clamp(minimum=0.0, maximum=1.0, clamp_type="hard", in_place=False)
    assert np.allclose(new.array, [0.0, 0.0, 1.0, 1.0])
    assert np.allclose(g.array, array)
    new = g.clamp(maximum=1.0, clamp_type="hard", in_place=False)
    assert np.allclose(new.array, [-1.0, 0.0, 1.0, 1.0])
    g.clamp(maximum=1.0, clamp_type="soft", in_place=True)
    assert (g.array < 2.0).all()
    v = np.array([-1.0, 0.0, 1.0, 2.0])
    assert np.allclose(g.array.ravel(), (v - 1.0) / (1 + np.exp(v - 1.0)) + 1.0, rtol=1e-6)
    with pytest.raises(ValueError):
        g.clamp(clamp_type="medium")


def test_add_mult(gpulib):
    from ppafm_gb300.field import DataGrid

    g1 = DataGrid(np.array([0.0, 1.0, 2.0])[None, None], _eye_lvec())
    g2 = DataGrid(np.array([1.0, 0.0, 1.0])[None, None], _eye_lvec())
    g1.add_mult(g2, scale=2.0, in_place=True)
    assert np.allclose(g1.array, [2.0, 1.0, 4.0])


def test_interp_at_and_grad_vs_oracle(gpulib, oracle):
    """DataGrid.interp_at with a rotation against the float32 restatement; grad against periodic
    centred differences; an XSF round trip of a grid and of its gradient."""
    import os
    import tempfile

    from ppafm_gb300.field import DataGrid, HartreePotential

    rng = np.random.default_rng(4)
    lv = np.array([[-1.0, 0.5, -2.0], [9.0, 0, 0], [0, 8.0, 0], [0, 0, 10.0]])
    a = rng.normal(size=(36, 32, 40)).astype(np.float32)
    g = HartreePotential(a, lv)
    c, s_ = np.cos(0.4), np.sin(0.4)
    rot = np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1.0]])
    lv2 = np.array([[0.0, 0.0, -1.0], [6.0, 0, 0], [0, 5.0, 0], [0, 0, 7.0]])
    out = g.interp_at(lv2, (30, 25, 35), rot=rot, rot_center=np.array([3.0, 2.5, 1.0]))
    assert isinstance(out, HartreePotential)
    want = oracle.interp_at(a, lv, (30, 25, 35), lv2[0], lv2[1:] / np.array([30, 25, 35])[:, None], rot, np.array([3.0, 2.5, 1.0]))
    assert np.abs(out.array - want).max() <= 1e-5 * np.abs(a).max()
    G = g.grad(scale=[-1.0, -1.0, -1.0, 1.0])
    h = np.diag(g.step)
    for k in range(3):
        fd = -0.5 * (np.roll(a, -1, axis=k) - np.roll(a, 1, axis=k)) / h[k]
        assert np.allclose(G.array[..., k], fd, atol=1e-5)
    assert np.array_equal(G.array[..., 3], a)
    d = tempfile.mkdtemp()
    g.to_file(os.path.join(d, "pot.xsf"))
    g2, _, _ = DataGrid.from_file(os.path.join(d, "pot.xsf"))
    assert g2.shape == g.shape and np.allclose(g2.array, a, rtol=1e-5, atol=1e-5) and np.allclose(g2.lvec, lv)
    G.to_file(os.path.join(d, "field.xsf"))
    assert all(os.path.exists(os.path.join(d, f)) for f in ("field_x.xsf", "field_y.xsf", "field_z.xsf", "field_w.xsf"))


def test_afmulator_tip_density_on_other_grid_vs_oracle(gpulib, oracle):
    """A tip density given on its own grid (a dz2 multipole made by the restatement on a
    12 x 12 x 16 A, 60 x 60 x 80 grid) is resampled onto the force-field grid; images against the
    oracle with the same resampling."""
    from ppafm_gb300.AFMulator import AFMulator, HartreePotential, TipDensity
    from tests.test_gpu_pipeline import _hartree_case

    xyzs, Zs, pot, lvp = _hartree_case(oracle)
    lvt = np.array([[0.0, 0, 0], [12.0, 0, 0], [0, 12.0, 0], [0, 0, 16.0]])
    nt = (60, 60, 80)
    L = np.diag(lvt[1:])
    coords = []
    for a in range(3):
        c = np.linspace(0, L[a] * (1 - 1 / nt[a]), nt[a])
        c[c >= L[a] / 2] -= L[a]
        coords.append(c)
    X, Y, Z = np.meshgrid(*coords, indexing="ij")
    rho_t = oracle.getProbeDensity(lvt, X, Y, Z, L / np.array(nt), sigma=0.71, multipole_dict={"dz2": -0.1}).astype(np.float32)
    kw = dict(pixPerAngstrome=10, scan_dim=(32, 28, 24), scan_window=((4.0, 4.0, 7.0), (12.0, 11.0, 9.4)), df_steps=8, npbc=(1, 1, 0))
    afm = AFMulator(rho=TipDensity(rho_t, lvt), **kw)
    X_gpu = afm.eval(xyzs, Zs, HartreePotential(pot, lvp))
    FE = afm.downloadFF()
    from ppafm_gb300 import species

    FFp = np.array([(r[0], r[1], r[2]) for r in species.loadSpecies()])
    Xo, aux = oracle.AFMulator(FFp, **kw).eval(xyzs, Zs, None, pot=(pot, lvp), rho=(rho_t, lvt), return_all=True)
    FEo = aux["FE"].transpose(2, 1, 0, 3)
    m = np.linalg.norm(FEo[..., :3].astype(np.float64), axis=-1) < 10.0
    scale = np.abs(FEo[..., :3].astype(np.float64)).max()
    assert np.abs(FE[..., :3] - FEo[..., :3])[m].max() <= 1e-4 * min(scale, 10.0) + 1e-5
    d = np.abs(X_gpu - Xo)
    assert (d > 0.1).mean() < 0.01 and np.median(d) < 1e-2
    # plot_to_dir: no plotting here; the stack is saved instead, the result unchanged
    import os
    import tempfile

    out_dir = tempfile.mkdtemp()
    with pytest.warns(UserWarning):
        X2 = afm.eval(xyzs, Zs, HartreePotential(pot, lvp), plot_to_dir=out_dir)
    assert np.array_equal(X2, X_gpu) and np.array_equal(np.load(os.path.join(out_dir, "df.npy")), X2)
    # eval_ of a molecule object, and the force field saved as XSF (|F| clamped to 10 eV/A)
    from types import SimpleNamespace

    assert np.array_equal(afm.eval_(SimpleNamespace(xyzs=xyzs, Zs=Zs, qs=HartreePotential(pot, lvp))), X_gpu)
    afm.saveFF(prefix=os.path.join(out_dir, ""))
    from ppafm_gb300.io import loadXSFData

    Fz, _, _, _ = loadXSFData(os.path.join(out_dir, "FF_z.xsf"))
    F = afm.downloadFF()[..., :3].astype(np.float64)
    k = np.minimum(1.0, 10.0 / np.maximum(np.linalg.norm(F, axis=-1), 1e-30))
    assert np.allclose(Fz, F[..., 2] * k, rtol=1e-5, atol=1e-5)
