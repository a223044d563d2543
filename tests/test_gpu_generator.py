"""The ML generators on the GPU path: the reference's generator test (batch count and
shapes, tests/test_generator.py of ppafm), image-for-image equality with AFMulator.eval
for both the deferred (one copy per batch) and the per-image host-copy mode, and the
LJ+Hartree simulation type with one tip density per tip; every image is also compared with
the oracle's restatement of the AFMulator (oracle.AFMulator) for that image's molecule,
tip and scan window."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_generator_afm_trainer_batches(gpulib):
    from ppafm_gb300.AFMulator import AFMulator
    from ppafm_gb300.ml.Generator import GeneratorAFMtrainer

    n_sample, batch_size, n_atoms = 12, 5, 10
    rng = np.random.default_rng(0)
    np.random.seed(0)

    class TestTrainer(GeneratorAFMtrainer):
        def on_batch_start(self):
            self.randomize_tip(max_tilt=0.5)

        def on_afm_start(self):
            self.randomize_distance(delta=0.5)

    def generator():
        for _ in range(n_sample):
            yield {"xyzs": 10 * rng.random((n_atoms, 3)), "Zs": rng.integers(1, 16, n_atoms)}

    class Disks:  # a stand-in aux map (the reference's are OpenCL); follows the scan window
        scan_window = None

        def __call__(self, xyzqs, Zs, pot, rot):
            return np.full((100, 100), float(len(Zs)), dtype=np.float32)

    afmulator = AFMulator(scan_dim=(100, 100, 20), scan_window=((0, 0, 5), (10, 10, 7)))
    aux = Disks()
    trainer = TestTrainer(afmulator=afmulator, aux_maps=[aux], sample_generator=generator(), sim_type="LJ", batch_size=batch_size, iZPPs=[8, 54])
    i_batch = -1
    for i_batch, (Xs, Ys, mols, sws) in enumerate(trainer):
        nb = 5 if i_batch < 2 else 2
        assert Xs.shape == (nb, 2, 100, 100, 11)
        assert Ys.shape == (nb, 1, 100, 100)
        assert len(mols) == nb and all(m.shape == (n_atoms, 5) for m in mols)
        assert sws.shape == (nb, 2, 2, 3)
        assert np.isfinite(Xs).all() and np.abs(Xs).max() > 0
    assert i_batch == 2
    assert aux.scan_window is not None
    with pytest.raises(NotImplementedError):
        GeneratorAFMtrainer(afmulator, [], generator(), sim_type="FDBM")


def test_generator_hartree_matches_eval(gpulib, oracle):
    """LJ+Hartree samples with two tip densities (cached per tip on the device, the spectrum
    transformed again when the tip changes): every image equals AFMulator.eval with that tip
    density and scan window; the aux maps get the potential."""
    from ppafm_gb300.AFMulator import AFMulator, HartreePotential
    from ppafm_gb300.ml.Generator import GeneratorAFMtrainer
    from tests.test_gpu_pipeline import _hartree_case

    xyzs, Zs, pot, lvp = _hartree_case(oracle)
    HP = HartreePotential(pot, lvp)
    rhos = [{"dz2": -0.1}, {"s": 0.05, "pz": 0.02}]
    rng = np.random.default_rng(3)
    seen, pots = [], []

    def rotz(t):
        c, s_ = np.cos(t), np.sin(t)
        return np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1.0]])

    def samples():
        for _ in range(3):
            yield {"xyzs": xyzs, "Zs": Zs, "qs": HP, "rot": rotz(rng.uniform(0, 0.5))}

    class Recorder(GeneratorAFMtrainer):
        def on_afm_start(self):
            a = self.afmulator
            seen.append((a.iZPP, a.scan_window, a.rho, self.sample_dict["rot"].copy()))

    def aux(xyzqs, Zs_, pot_, rot):
        pots.append(pot_)
        return np.zeros((32, 28), dtype=np.float32)

    kw = dict(pixPerAngstrome=10, scan_dim=(32, 28, 24), scan_window=((4.0, 4.0, 7.0), (12.0, 11.0, 9.4)), df_steps=8, npbc=(1, 1, 0))
    tr = Recorder(AFMulator(**kw), [aux], samples(), sim_type="LJ+Hartree", batch_size=2, iZPPs=[8, 8], rhos=rhos)
    batches = [b for b in tr]  # (list() would ask the generator for its length)
    assert [b[0].shape for b in batches] == [(2, 2, 32, 28, 17), (1, 2, 32, 28, 17)]
    assert all(p is HP for p in pots) and len(pots) == 3
    assert all(np.array_equal(m[:, 3], np.zeros(len(Zs))) for b in batches for m in b[2])
    images = [Xs[s, t] for Xs, _, _, _ in batches for s in range(Xs.shape[0]) for t in range(2)]
    assert len(images) == len(seen) == 6
    assert [r for _, _, r, _ in seen] == rhos * 3
    FFp = _species_table()
    for img, (iZPP, sw, rho, rot) in zip(images, seen):
        ref = AFMulator(**{**kw, "scan_window": sw}, rho=rho)
        ref.iZPP = iZPP
        want = ref.eval(xyzs, Zs, HP, rot=rot)
        assert np.array_equal(img, want)
        # and against the oracle's restatement of the AFMulator (float64 FFTs)
        ora = oracle.AFMulator(FFp, **{**kw, "scan_window": sw}, iZPP=iZPP).eval(xyzs, Zs, None, pot=(pot, lvp), rho=rho, sigma=0.71, rot=rot)
        _close_images(img, ora)
    with pytest.raises(ValueError):
        next(iter(GeneratorAFMtrainer(AFMulator(**kw), [], iter([{"xyzs": xyzs, "Zs": Zs, "qs": np.zeros(len(Zs))}]), sim_type="LJ+Hartree", iZPPs=[8], rhos=rhos[:1])))


def _write_molecules(tmp_path, n, rng):
    from ppafm_gb300.io import saveXYZ

    paths = []
    for k in range(n):
        na = int(rng.integers(8, 20))
        xyz = np.c_[rng.random((na, 2)) * 8.0, rng.random(na) * 0.5]
        Zs = rng.choice([1, 6, 7, 8], na)
        q = rng.uniform(-0.3, 0.3, na)
        q -= q.mean()
        p = tmp_path / f"mol{k}.xyz"
        saveXYZ(p, xyz, Zs, q)
        paths.append(str(p))
    return paths


def _species_table():
    from ppafm_gb300 import species

    return np.array([(r[0], r[1], r[2]) for r in species.loadSpecies()])


def _close_images(img, ref):
    """The AFMulator tolerance against the oracle (tests/test_gpu_pipeline.py): float32 on both
    sides, trajectories agree to float rounding except at bistable pixels."""
    d = np.abs(img - ref)
    assert img.shape == ref.shape
    assert (d > 0.1).mean() < 0.01 and np.median(d) < 1e-2, ((d > 0.1).mean(), np.median(d))


@pytest.mark.parametrize("host_copy_each", [False, True])
def test_inverse_trainer_matches_eval(gpulib, oracle, tmp_path, host_copy_each):

    from ppafm_gb300.AFMulator import AFMulator
    from ppafm_gb300.ml.Generator import InverseAFMtrainer

    rng = np.random.default_rng(5)
    paths = _write_molecules(tmp_path, 5, rng)
    seen = []

    class Recorder(InverseAFMtrainer):
        def on_afm_start(self):  # what AFMulator.eval gets for this image
            seen.append((self.xyzs.copy(), self.Zs.copy(), self.qs.copy(), self.REAs.copy(), self.afmulator.iZPP, self.afmulator.Qs.copy(), self.afmulator.QZs.copy()))

    class HostEach(Recorder):
        def on_afm_end(self):
            assert isinstance(self.Xs, np.ndarray)
            self.host_images.append(self.Xs.copy())

    cls = HostEach if host_copy_each else Recorder
    afm = AFMulator(scan_dim=(64, 64, 20), scan_window=((2.0, 2.0, 7.0), (10.0, 10.0, 9.0)))
    tr = cls(afm, [], paths, batch_size=3, iZPPs=[8, 8], Qs=[[-10, 20, -10, 0], [0, 0, 0, 0]], QZs=[[0.1, 0, -0.1, 0], [0, 0, 0, 0]])
    tr.host_images = []
    assert len(tr) == 1
    batches = list(tr)
    assert [b[0][0].shape[0] for b in batches] == [3, 2]
    images = [X[t][s] for Xs, _, _ in batches for s in range(Xs[0].shape[0]) for t in range(2) for X in [Xs]]
    assert len(images) == len(seen) == 10
    ref = AFMulator(scan_dim=(64, 64, 20), scan_window=((2.0, 2.0, 7.0), (10.0, 10.0, 9.0)))
    FFp = _species_table()
    for img, (xyz, Zs, qs, REAs, iZPP, Qs, QZs) in zip(images, seen):
        ref.iZPP = iZPP
        ref.setQs(Qs, QZs)
        want = ref.eval(xyz, Zs, qs, REAs=REAs)
        assert np.array_equal(img, want)
        # and against the oracle's restatement of the AFMulator
        ora = oracle.AFMulator(FFp, scan_dim=(64, 64, 20), scan_window=((2.0, 2.0, 7.0), (10.0, 10.0, 9.0)), iZPP=iZPP, Qs=Qs, QZs=QZs)
        _close_images(img, ora.eval(xyz, Zs, qs, REAs=REAs))
    if host_copy_each:
        assert all(np.array_equal(a, b) for a, b in zip(tr.host_images, images))


@pytest.mark.parametrize("route", ["point_charges", "hartree"])
def test_overlap_mode_matches_plain(gpulib, route):
    """AFMulator.set_overlap (each image's force field on a second grid and stream beside the
    previous image's relaxation, as the generators queue them): images of a sequence of
    molecules, scan windows and tips equal the plain mode's bit for bit, on the point-charge
    route and on the Hartree route; the iteration counter agrees."""
    import torch

    from ppafm_gb300.AFMulator import AFMulator, HartreePotential

    rng = np.random.default_rng(3)
    mols = []
    for i in range(6):
        n = 8 + 3 * i
        xyz = np.column_stack([rng.uniform(2, 14, n), rng.uniform(2, 14, n), rng.uniform(-0.3, 0.3, n)])
        q = rng.uniform(-0.3, 0.3, n)
        mols.append((xyz, rng.choice([1, 6, 7, 8], n), q - q.mean()))
    pot = None
    if route == "hartree":
        n = (48, 48, 40)
        lv = np.array([[0.0, 0, -4], [16.0, 0, 0], [0, 16.0, 0], [0, 0, 12.0]])
        g = np.stack(np.meshgrid(*[np.arange(k) for k in n], indexing="ij"), -1).astype(np.float64)
        pot = HartreePotential((0.2 * np.cos(2 * np.pi * g[..., 0] / n[0]) * np.sin(2 * np.pi * g[..., 1] / n[1]) + 0.05 * g[..., 2] / n[2]).astype(np.float32), lv)
    windows = [((1.0 + 0.5 * i, 2.0, 6.5), (13.0 + 0.5 * i, 14.0, 9.5)) for i in range(len(mols))]
    tips = [([-10, 20, -10, 0], [0.1, 0, -0.1, 0]), ([-0.1, 0, 0, 0], [0, 0, 0, 0])]

    def run(overlap):
        afm = AFMulator(scan_dim=(96, 96, 24), scan_window=windows[0], df_steps=8, rho={"dz2": -0.1} if route == "hartree" else None)
        afm.set_overlap(overlap)
        nx, ny, nz = afm.scan_dim
        out = torch.empty((len(mols), len(tips), nx, ny, nz - 8 + 1), dtype=torch.float32, device="cuda")
        for i, (xyz, Zs, qs) in enumerate(mols):
            for t, (Q, QZ) in enumerate(tips):
                afm.setQs(Q, QZ)
                afm.setScanWindow(windows[i], afm.scan_dim, df_steps=8)
                afm.setLvec()
                afm.prepareFF(xyz, Zs, pot if pot is not None else qs)
                afm.evalAFM(out=out[i, t])
        afm.join()
        torch.cuda.synchronize()
        return out.cpu().numpy(), int(afm.counter.item())

    plain, it_plain = run(False)
    over, it_over = run(True)
    assert np.isfinite(plain).all() and np.abs(plain).max() > 0
    assert np.array_equal(plain, over)
    assert it_plain == it_over
