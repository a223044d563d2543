"""The learned warm start on the batched relaxation.

1. The height-synchronous schedule without a network reproduces the flattened persistent
   kernel (plain FIRE from the height above) stroke for stroke.
2. Recorded training pairs are what they claim: the tanh-compressed forces at the 3x3x3 grid
   nodes around the start point (the tip plus the previous height's converged displacement),
   the point's offset from the middle node, that displacement and its change at the height
   above; the targets are the change of the converged displacement.
3. A network trained on plain-FIRE pairs of held-out molecules lowers the mean FIRE
   iterations per pixel height on other molecules, with every height converged to the same
   criterion and df within 0.1 Hz of plain FIRE (except at basin flips, which plain FIRE
   itself resolves by where it starts)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(nmol, seed, scale):
    from ppafm_gb300 import workloads

    systems = workloads.molecule_batch(seed=seed, nmol=nmol, scale=scale)
    w = systems[0]
    relax = dict(maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    return systems, w, relax


def test_layered_plain_matches_flattened(gpulib):
    import torch

    from ppafm_gb300.batch import BatchPipeline

    systems, params, relax = _batch(4, 21, 0.3)
    a = BatchPipeline(systems, params, relax=relax, want_iters=True)
    a.run()
    torch.cuda.synchronize()
    ref = [{k: v.clone() for k, v in a.outputs(j).items()} for j in range(len(systems))]
    a.run_layered()
    torch.cuda.synchronize()
    for j in range(len(systems)):
        o = a.outputs(j)
        assert o["iters"].equal(ref[j]["iters"]), j
        assert o["ppos"].equal(ref[j]["ppos"]), j
        assert o["df"].equal(ref[j]["df"]), j


def test_recorded_pairs(gpulib):
    import torch

    from ppafm_gb300 import common as PPU
    from ppafm_gb300.batch import BatchPipeline
    from ppafm_gb300.warmstart import NIN

    systems, params, relax = _batch(1, 23, 0.25)
    bp = BatchPipeline(systems, params, relax=relax, want_iters=True, tuning=(2, 32, 1, 32))
    nz = bp.systems[0]["scan_shape"][2]
    nstrokes = bp.strokes
    X = torch.zeros((nstrokes * nz, NIN), dtype=torch.bfloat16, device="cuda")
    T = torch.full((nstrokes * nz, 4), float("nan"), device="cuda")
    bp.run_layered(record=(1, X, T))
    torch.cuda.synchronize()
    s = bp.systems[0]
    nx, ny, _ = s["scan_shape"]
    w = systems[0]
    xT, yT, zT, _ = PPU.prepareScanGrids(w["scanMin"], w["scanMax"], w["scanStep"], w["r0Probe"])
    pp = s["out"]["ppos"].cpu().numpy().astype(np.float64)  # ascending z
    d_asc = pp - np.stack(np.meshgrid(xT, yT, zT, indexing="ij"), axis=-1)  # tip + d = ppos (origin 0)
    d_app = d_asc[:, :, ::-1]  # approach order
    Xn = X.float().cpu().numpy()
    Tn = T.cpu().numpy()
    rPP0 = np.array([0.0, 0.0, -4.0])
    FE = s["FE"].view(tuple(s["n"]) + (4,))[..., :3].cpu().numpy().astype(np.float64)
    n = np.array(s["n"])
    cell = np.asarray(w["lvec"])[1:].diagonal()
    rng = np.random.default_rng(0)
    checked = 0
    tw, th = 32, 1
    nty = (ny + th - 1) // th
    for _ in range(60):
        ix, iy, iz = int(rng.integers(nx)), int(rng.integers(ny)), int(rng.integers(0, nz))
        gs = ((ix // tw) * nty + iy // th) * (tw * th) + (ix % tw) * th + iy % th
        slot = gs * nz + iz
        if np.isnan(Tn[slot, 0]):
            continue
        dprev = rPP0 if iz == 0 else d_app[ix, iy, iz - 1]
        assert np.allclose(Tn[slot, :3], 10 * (d_app[ix, iy, iz] - dprev), atol=1e-4)
        # forces at the 3x3x3 grid nodes around the start point's nearest node, the offset
        # from that node, the displacement and its change at the height above
        p = np.array([xT[ix], yT[iy], zT[::-1][iz]]) + dprev
        g = p / cell * n
        fl = np.floor(g)
        if np.min(np.abs(g - fl - 0.5)) < 1e-4:
            continue  # halfway between nodes: float rounding decides the nearest one
        m = np.where(g - fl >= 0.5, fl + 1, fl).astype(int)
        q = np.array([FE[(m[0] + a) % n[0], (m[1] + b) % n[1], (m[2] + c) % n[2]] for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
        if iz == 0:
            dd = np.zeros(3)
        else:
            dd = d_app[ix, iy, iz - 1] - (rPP0 if iz == 1 else d_app[ix, iy, iz - 2])
        f = np.concatenate([np.tanh(2 * q.ravel()), 2 * (g - m), 10 * (dprev - rPP0), 10 * dd, np.zeros(6)])
        assert np.allclose(Xn[slot], f, rtol=1e-2, atol=1e-2), (slot, np.abs(Xn[slot] - f).max())
        checked += 1
    assert checked >= 30


def test_learned_warm_start_gain(gpulib):
    """Train on 16 held-out molecules, evaluate on 8 others (grids and scans at 0.35 scale)."""
    import torch

    from ppafm_gb300.batch import BatchPipeline
    from ppafm_gb300.warmstart import WarmStartNet, generate_pairs
    from tests.test_gpu_relax import _split_flips

    train_sys, params, relax = _batch(16, 1000, 0.35)
    X, T = generate_pairs(train_sys, params, relax, stride=1)
    assert X.shape[0] > 100000
    net = WarmStartNet(seed=0)
    log = net.train(X, T, steps=4000, batch=8192, lr=1e-3, log_every=1000)
    assert log[-1][1] < 0.5 * log[0][1], log
    test_sys, _, _ = _batch(8, 2000, 0.35)
    plain = BatchPipeline(test_sys, params, relax=relax, want_iters=True)
    plain.run()
    learned = BatchPipeline(test_sys, params, relax=relax, want_iters=True)
    learned.run_layered(net)
    torch.cuda.synchronize()
    it_p = np.concatenate([plain.outputs(j)["iters"].cpu().numpy().ravel() for j in range(len(test_sys))])
    it_l = np.concatenate([learned.outputs(j)["iters"].cpu().numpy().ravel() for j in range(len(test_sys))])
    # every height converged (no height hit the iteration cap that plain FIRE did not hit)
    assert (it_l >= relax["maxIters"]).sum() <= (it_p >= relax["maxIters"]).sum() + 2
    assert it_l.mean() < 0.75 * it_p.mean(), (it_l.mean(), it_p.mean())
    for j in range(len(test_sys)):
        a, b = plain.outputs(j), learned.outputs(j)
        dpos = np.linalg.norm(a["ppos"].cpu().numpy() - b["ppos"].cpu().numpy(), axis=-1)
        flips, _ = _split_flips(dpos)
        assert flips.mean() < 0.01
        ok = ~flips.any(axis=-1)
        ddf = np.abs(a["df"].cpu().numpy() - b["df"].cpu().numpy())[ok]
        assert np.mean(ddf < 0.1) > 0.995, (j, np.mean(ddf < 0.1), ddf.max())
