"""Parity at the benchmarked sizes: the small-molecule workload in full and the slab +
molecule workload (the headline: 800x800x500 grid, 18 540 atoms with images, 512x512x40
scan) by sampling, each against the oracle (the float64 restatement of the reference core,
bit-identical to it).

Force grids (``tests.conftest.check_ff``): every point within 1e-5 relative of the oracle
(|dF| <= 1e-5 * max(|F|, 1e-2 eV/A)), except where that is finer than float32 can resolve:
a float32 evaluation of a sum of pair terms carries an error of a few ulps of the terms'
magnitudes, sum_i |F_i|, so where the terms cancel (|F| << sum_i |F_i|: between atoms, and
inside the repulsive cores where the 10 eV/A clamp keeps only the direction of a large sum)
a point passes at |dF| <= 2^-20 sum_i |F_i| (16 float32 ulps of the summed magnitudes).  At
most 1 in 10^3 points may need that clause; their number and the float32 error of each grid
are printed (``-s``).

Relaxation, two comparisons.  Same force field: the oracle relaxes the GPU's own float32 grid
(values exact in float64), which isolates the relaxation arithmetic; bar of
``tests.test_gpu_relax._check_positions`` (no basin flips, every position within the
convergence ball, at most 1 in 10^4 pixel heights beyond 1e-3 A) and every Δf value within
0.1 Hz.  End to end: the oracle's float64 force field and relaxation on the same atoms; bar of
``_check_end_to_end`` (basin flips, where the float32 grid's error sends a bistable pixel into
its other minimum, at most 1 in 10^4 pixel heights; every other height within the ball; Δf
within 0.1 Hz at every pixel without a flip).  The fractions are printed.

The slab workload's samples: three whole z-planes (inside the slab's top layer, at the
molecule and in the scan region), compared point for point; two blocks of 4 x 4 pixels x 40
heights (over the molecule and at a seeded place), relaxed by the oracle on its own force
field filled on a box around each block (the probe stays inside the box: asserted) and
compared with the GPU scan's pixels; the GPU's float64 evaluation of the same sums on every
50th z-plane for the per-grid float32 error."""

import time

import numpy as np
import pytest

from tests.conftest import check_ff, rel_err
from tests.test_gpu_relax import _check_end_to_end, _check_positions

pytestmark = pytest.mark.gpu

FLOOR = 1e-2
DF_TOL = 0.1


def _check_ff(name, got, ref, coords, pl):
    return check_ff(name, got, ref, coords, pl.Rs0, pl.cLJs, pl.kqq, pl.Q)


def _relax_params(w):
    return dict(maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])


def _oracle_ff(oracle, n, cell, i0, ns, Rs0, cLJs, kqq, Q, nthreads=0):
    """clamp(F_LJ) + Q clamp(F_Coulomb) on the subgrid [i0, i0+ns) (the reference's
    computeLJ / computeELFF_pointCharge with the 10 eV/A clamp and perform_relaxation's sum).
    Atoms without charge add exactly +0.0 to the Coulomb sums, so only charged ones are passed."""
    Fl, _ = oracle.ff_subgrid(n, cell, i0, ns, Rs0, cLJs, -1, nthreads=nthreads)
    oracle.limit_vec_field(Fl, 10.0)
    q = kqq != 0.0
    if Q != 0.0 and q.any():
        Fe, _ = oracle.ff_subgrid(n, cell, i0, ns, Rs0[q], kqq[q], 0, nthreads=nthreads)
        oracle.limit_vec_field(Fe, 10.0)
        Fl += Q * Fe
    return Fl


def test_small_molecule_full_size(gpulib, oracle):
    """The whole 200^3 force field, 160x160x30 relaxed scan and Δf of the benchmarked
    small-molecule workload (seed 0)."""
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import common, workloads

    w = workloads.small_molecule(seed=0)
    relax = _relax_params(w)
    pl = HL.Pipeline(w["Zs"], w["Rs"], w["Qs"], w["lvec"], w["gridN"], w, relax=relax, want_iters=True)
    out = pl.run()
    Fg, _ = pl.ff.to_host()
    n = np.array(w["gridN"], np.int32)
    lv = w["lvec"]
    t0 = time.perf_counter()
    FF = _oracle_ff(oracle, n, lv[1:], (0, 0, 0), n, pl.Rs0, pl.cLJs, pl.kqq, pl.Q)
    dc = lv[1:4] / n[:, None]
    print()
    _check_ff(f"small_molecule 200^3 LJ+Coulomb force field ({pl.natoms} atoms)", Fg, FF, lambda idx: idx @ dc, pl)
    xT, yT, zT, _ = common.prepareScanGrids(w["scanMin"], w["scanMax"], w["scanStep"], w["r0Probe"])
    ppg = out["ppos"].cpu().numpy()
    dfg = out["df"].cpu().numpy()
    itg = out["iters"].cpu().numpy()

    def scan(FFgrid):
        fzs, pp, it = oracle.relaxed_scan(n, lv[1:], FFgrid, pl.prm, xT, yT, zT, lv[0])
        return pp, oracle.Fz2df(fzs, w["scanStep"][2], w["kCantilever"], w["f0Cantilever"], w["Amplitude"]), it

    # same force field: the GPU's float32 grid relaxed by the oracle
    pp, df, it = scan(Fg)
    dpos = np.linalg.norm(ppg - pp, axis=-1)
    ddf = np.abs(dfg - df)
    print(f"small_molecule scan {dpos.shape} on the GPU's force field: positions max {dpos.max():.2e} A ({(dpos > 1e-3).sum()} beyond 1e-3 A), Δf max {ddf.max():.2e} Hz, FIRE iterations per pixel height {itg.mean():.3f} (oracle {it.mean():.3f})")
    _check_positions(dpos)
    assert ddf.max() < DF_TOL
    assert abs(itg.mean() - it.mean()) < 0.01 * it.mean()
    # end to end: the oracle's float64 force field
    pp, df, it = scan(FF)
    dpos = np.linalg.norm(ppg - pp, axis=-1)
    ddf = np.abs(dfg - df)
    flips, pix = _check_end_to_end(dpos, ddf)
    rest = dpos[~flips]
    print(f"small_molecule scan end to end: {flips.sum()} pixel heights in another basin ({pix.sum()} pixels); others max {rest.max():.2e} A ({(rest > 1e-3).sum()} beyond 1e-3 A); Δf max {ddf[~pix].max():.2e} Hz without a flip, {ddf.max():.2e} Hz overall; oracle {time.perf_counter() - t0:.1f} s")


@pytest.fixture(scope="module")
def slab_run(gpulib):
    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import workloads

    w = workloads.slab_molecule(seed=0)
    relax = _relax_params(w)
    pl = HL.Pipeline(w["Zs"], w["Rs"], w["Qs"], w["lvec"], w["gridN"], w, relax=relax, want_iters=True)
    out = pl.run()
    host = {k: v.cpu().numpy() for k, v in out.items()}
    return w, pl, host


@pytest.mark.parametrize("iz", [285, 350, 440])
def test_slab_molecule_full_size_planes(slab_run, oracle, iz):
    """Whole z-planes of the 800x800x500 force field against the oracle: z = -0.25 A (the slab's
    top layer, forces clamped), 3.0 A (the molecule's plane) and 7.5 A (the scan region)."""
    w, pl, _ = slab_run
    n = np.array(w["gridN"], np.int32)
    g = pl.ff.grid4[:, :, iz, :3].cpu().numpy().astype(np.float64)
    t0 = time.perf_counter()
    FF = _oracle_ff(oracle, n, w["lvec"][1:], (0, 0, iz), (n[0], n[1], 1), pl.Rs0, pl.cLJs, pl.kqq, pl.Q)[:, :, 0]
    # the GPU's float64 evaluation of the same sums (the error oracle of the sampled test below)
    from ppafm_gb300.device import FF_LJC

    g64 = pl.ff.compute_subgrid((0, 0, iz), (n[0], n[1], 1), pl.atoms, pl.natoms, pl.ncharged, FF_LJC, Q=pl.Q, Fmax=10.0, f64=True)
    err64 = rel_err(g64.view(int(n[0]), int(n[1]), 4)[..., :3].cpu().numpy().astype(np.float64), FF, FLOOR)
    z = w["lvec"][0, 2] + iz * w["lvec"][3, 2] / n[2]
    dc = w["lvec"][1:4] / n[:, None]
    print(f"\nslab_molecule plane iz={iz} (z = {z:.2f} A; {n[0] * n[1]} points x {pl.natoms} atoms; oracle {time.perf_counter() - t0:.1f} s): GPU float64 sums {err64:.1e} relative")
    _check_ff(f"slab_molecule plane iz={iz}", g, FF, lambda idx: idx[:, 0:1] * dc[0] + idx[:, 1:2] * dc[1] + iz * dc[2], pl)
    assert err64 < 1e-6


def test_slab_molecule_full_size_fp32_error(slab_run):
    """The float32 error of the headline grid on a larger sample: every 50th z-plane against
    the GPU's float64 evaluation of the same sums (itself checked against the oracle on the
    whole-plane test's planes)."""
    from ppafm_gb300.device import FF_LJC

    w, pl, _ = slab_run
    n = np.array(w["gridN"], np.int32)
    dc = w["lvec"][1:4] / n[:, None]
    worst = 0.0
    print()
    for iz in range(0, int(n[2]), 50):
        ref = pl.ff.compute_subgrid((0, 0, iz), (n[0], n[1], 1), pl.atoms, pl.natoms, pl.ncharged, FF_LJC, Q=pl.Q, Fmax=10.0, f64=True)
        ref = ref.view(int(n[0]), int(n[1]), 4)[..., :3].cpu().numpy().astype(np.float64)
        g = pl.ff.grid4[:, :, iz, :3].cpu().numpy().astype(np.float64)
        worst = max(worst, _check_ff(f"slab_molecule plane iz={iz} vs the GPU float64 sums", g, ref, lambda idx, iz=iz: idx[:, 0:1] * dc[0] + idx[:, 1:2] * dc[1] + iz * dc[2], pl))
    print(f"slab_molecule 800x800x500 force field: float32 max rel err {worst:.2e} over {len(range(0, int(n[2]), 50))} whole z-planes")


def _block_case(w, pl, oracle, bx, by, nb=4):
    """Oracle relaxations of pixels [bx, bx+nb) x [by, by+nb), each on a force field filled on a
    box around the block (a lazily committed full-size grid: only the box is written): the
    oracle's own float64 field, and the GPU's float32 field copied from the device.  Returns
    per field (positions, Fz, iterations) in the GPU outputs' order (ascending heights, scan
    origin)."""
    n = np.array(w["gridN"], np.int32)
    lv = np.asarray(w["lvec"], np.float64)
    cell = lv[1:4]
    xs, ys, zs = pl.xs, pl.ys, pl.zs
    Z = len(zs)
    ds = np.linalg.norm(cell, axis=1) / n
    r0 = w["r0Probe"]
    lo = np.array([xs[bx : bx + nb].min() - 2.0, ys[by : by + nb].min() - 2.0, zs.min() - r0[2] - 2.0])
    hi = np.array([xs[bx : bx + nb].max() + 2.0, ys[by : by + nb].max() + 2.0, zs.max() - r0[2] + 2.0])
    i_lo = np.maximum(np.floor(lo / ds).astype(int), 0)
    i_hi = np.minimum(np.ceil(hi / ds).astype(int) + 1, n)
    ns = i_hi - i_lo
    box = tuple(slice(a, b) for a, b in zip(i_lo, i_hi))
    rT = np.zeros((nb, nb, Z, 3))
    rT[..., 0] = xs[bx : bx + nb][:, None, None]
    rT[..., 1] = ys[by : by + nb][None, :, None]
    rT[..., 2] = zs[None, None, :]
    out = {}
    for which in ("oracle", "gpu"):
        FFbox = np.zeros(tuple(n) + (3,))
        if which == "oracle":
            FFbox[box] = _oracle_ff(oracle, n, cell, i_lo, ns, pl.Rs0, pl.cLJs, pl.kqq, pl.Q)
        else:
            FFbox[box] = pl.ff.grid4[box + (slice(0, 3),)].cpu().numpy().astype(np.float64)
        rs, fs, _, iters = oracle.relax_strokes(n, cell, FFbox, pl.prm, rT)
        g = rs / ds
        assert (g > i_lo + 1).all() and (g < i_hi - 2).all(), "the probe left the box"
        del FFbox
        out[which] = (rs[:, :, ::-1] + lv[0], fs[:, :, ::-1, 2], iters.reshape(nb, nb, Z)[:, :, ::-1])
    return out


def test_slab_molecule_full_size_relaxation(slab_run, oracle):
    """Relaxed positions, Fz and Δf of two 4x4-pixel blocks (all 40 heights) of the headline
    scan against the oracle's relaxation on the GPU's force field (same field) and on its own
    float64 field (end to end)."""
    w, pl, host = slab_run
    nx, ny, _ = pl.scan_shape
    rng = np.random.default_rng(0)
    blocks = [(nx // 2 - 2, ny // 2 - 2), (int(rng.integers(40, nx - 44)), int(rng.integers(40, ny - 44)))]
    dW = lambda fz: oracle.Fz2df(fz, w["scanStep"][2], w["kCantilever"], w["f0Cantilever"], w["Amplitude"])  # noqa: E731
    same, e2e = [], []
    for bx, by in blocks:
        t0 = time.perf_counter()
        res = _block_case(w, pl, oracle, bx, by)
        sl = (slice(bx, bx + 4), slice(by, by + 4))
        gp, gdf, git = host["ppos"][sl], host["df"][sl], host["iters"][sl]
        for which, store in (("gpu", same), ("oracle", e2e)):
            pp, fz, it = res[which]
            dpos = np.linalg.norm(gp - pp, axis=-1)
            ddf = np.abs(gdf - dW(fz))
            store.append((dpos, ddf))
            print(f"\nslab_molecule block ({bx},{by}) on the {'GPU' if which == 'gpu' else 'oracle'}'s force field: positions max {dpos.max():.2e} A ({(dpos > 1e-3).sum()} beyond 1e-3 A), Δf max {ddf.max():.2e} Hz, iterations {git.sum()} (oracle {it.sum()})", end="")
            assert abs(int(git.sum()) - int(it.sum())) <= 0.05 * it.sum() + 5
        print(f"; oracle {time.perf_counter() - t0:.1f} s")
    dpos, ddf = (np.stack([a[k] for a in same]) for k in (0, 1))
    _check_positions(dpos)
    assert ddf.max() < DF_TOL
    dpos, ddf = (np.stack([a[k] for a in e2e]) for k in (0, 1))
    _check_end_to_end(dpos, ddf)
    # the rest of the scan: converged everywhere and finite
    assert np.isfinite(host["df"]).all() and np.isfinite(host["ppos"]).all()
    assert (host["iters"] < w["maxIters"]).mean() > 0.999
