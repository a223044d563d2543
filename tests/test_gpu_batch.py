"""The batched persistent launch (many molecules, one kernel) against the single-system path
and the oracle.

The batched kernel runs the same force-field block and the same relaxation arithmetic as the
single-system kernels, so per system its force field and relaxed scan must equal those of
HighLevel.Pipeline: the force field bit for bit, positions to a few float32 ulps (1e-5 A) and
the same iteration counts.  One system is also checked against the oracle with the
tolerances of the single-system pipeline test."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(nmol=5, seed=3, scale=0.3):
    from ppafm_gb300 import workloads

    systems = workloads.molecule_batch(seed=seed, nmol=nmol, scale=scale)
    w = systems[0]
    relax = dict(maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    return systems, w, relax


def _single(w, params, relax):
    from ppafm_gb300 import HighLevel as HL

    p = dict(params)
    for k in ("scanMin", "scanMax", "scanStep"):
        p[k] = w[k]
    pl = HL.Pipeline(w["Zs"], w["Rs"], w["Qs"], w["lvec"], w["gridN"], p, relax=relax, want_iters=True)
    out = pl.run()
    return pl, out


def _compare(bp, systems, params, relax):
    for j, w in enumerate(systems):
        pl, out = _single(w, params, relax)
        s = bp.systems[j]
        assert s["FE"].view(-1, 4)[:, :3].equal(pl.ff.FE.view(-1, 4)[:, :3]), f"system {j}: force field differs"
        ob = bp.outputs(j)
        dpos = (ob["ppos"] - out["ppos"]).abs().max().item()
        assert dpos < 1e-5, (j, dpos)
        assert (ob["iters"] == out["iters"]).float().mean().item() > 0.999
        assert (ob["df"] - out["df"]).abs().max().item() < 1e-3
        assert (ob["fzs"] - out["fzs"]).abs().max().item() < 1e-5


def test_batch_matches_single_pipelines(gpulib):
    from ppafm_gb300.batch import BatchPipeline

    systems, params, relax = _batch()
    bp = BatchPipeline(systems, params, relax=relax, want_iters=True)
    bp.run()
    _compare(bp, systems, params, relax)
    # the counter counts FIRE moves; a converged height reports the index of its last move
    tot = sum(int(bp.outputs(j)["iters"].sum().item()) for j in range(len(systems)))
    assert tot <= bp.iterations() <= tot + bp.pixel_z


@pytest.mark.parametrize("tuning", [(1, 32, 1, 32), (2, 4, 8, 128), (2, 16, 2, 64), (1, 3, 5, 7)])
def test_batch_tunings_agree(gpulib, tuning):
    from ppafm_gb300.batch import BatchPipeline

    systems, params, relax = _batch(nmol=4, seed=5)
    ref = BatchPipeline(systems, params, relax=relax, want_iters=True)
    ref.run()
    bp = BatchPipeline(systems, params, relax=relax, want_iters=True, tuning=tuning)
    bp.run()
    for j in range(len(systems)):
        a, b = ref.outputs(j), bp.outputs(j)
        for k in ("fzs", "ppos", "df", "iters"):
            assert a[k].equal(b[k]), (tuning, j, k)


def test_batch_graph_replay(gpulib):
    import torch

    from ppafm_gb300.batch import BatchPipeline

    systems, params, relax = _batch(nmol=3, seed=7)
    bp = BatchPipeline(systems, params, relax=relax, want_iters=True)
    bp.run()
    torch.cuda.synchronize()
    first = [{k: v.clone() for k, v in bp.outputs(j).items()} for j in range(len(systems))]
    for j in range(len(systems)):
        for v in bp.outputs(j).values():
            v.zero_()
    bp.capture()
    bp.replay()
    bp.replay()
    torch.cuda.synchronize()
    for j in range(len(systems)):
        for k, v in bp.outputs(j).items():
            assert v.equal(first[j][k]), (j, k)


def test_batch_output_sets(gpulib):
    """Two output sets: each slot's launch (and graph) writes its own buffers, equal to the
    one-set pipeline's; running one slot leaves the other untouched."""
    import torch

    from ppafm_gb300.batch import BatchPipeline

    systems, params, relax = _batch(nmol=3, seed=9)
    ref = BatchPipeline(systems, params, relax=relax, want_iters=True)
    ref.run()
    bp = BatchPipeline(systems, params, relax=relax, want_iters=True, out_sets=2)
    bp.run(slot=1)
    torch.cuda.synchronize()
    for j in range(len(systems)):
        assert all(v.data_ptr() != w.data_ptr() for v, w in zip(bp.outputs(j, 0).values(), bp.outputs(j, 1).values()))
        for k, v in bp.outputs(j, 1).items():
            assert v.equal(ref.outputs(j)[k]), (j, k)
        for v in bp.outputs(j, 0).values():
            v.zero_()
    bp.capture()
    bp.replay(0)
    torch.cuda.synchronize()
    for j in range(len(systems)):
        for k, v in bp.outputs(j, 0).items():
            assert v.equal(ref.outputs(j)[k]), (j, k)
    bp.close()


def test_batch_system_vs_oracle(gpulib, oracle):
    from ppafm_gb300.batch import BatchPipeline
    from tests.conftest import check_ff, grid_coords
    from tests.test_gpu_pipeline import _oracle_pipeline
    from tests.test_gpu_relax import _check_positions

    systems, params, relax = _batch(nmol=2, seed=11, scale=0.25)
    bp = BatchPipeline(systems, params, relax=relax, want_iters=True)
    bp.run()
    w = systems[1]
    FF, fzs, pp, df, it = _oracle_pipeline(oracle, w, relax)
    s = bp.systems[1]
    Fg = s["FE"].view(tuple(s["n"]) + (4,))[..., :3].cpu().numpy()
    from ppafm_gb300 import HighLevel as HL

    Rs0, cLJs, kqq = HL.prepare_atoms(w["Zs"], w["Rs"], w["Qs"], w["lvec"], w)
    check_ff("batched system LJ+Coulomb force field", Fg.astype(np.float64), FF, grid_coords(s["n"], w["lvec"]), Rs0, cLJs, kqq, params["charge"])
    out = bp.outputs(1)
    _check_positions(np.linalg.norm(out["ppos"].cpu().numpy() - pp, axis=-1))
    assert np.abs(out["df"].cpu().numpy() - df).max() < 0.1


def test_batch_rejects_bad_systems(gpulib):
    from ppafm_gb300._lib import PPGPUError
    from ppafm_gb300.batch import BatchPipeline

    systems, params, relax = _batch(nmol=2, seed=13)
    skew = dict(systems[1])
    lv = np.array(skew["lvec"], dtype=np.float64)
    lv[2, 0] = 0.7
    skew["lvec"] = lv
    with pytest.raises(PPGPUError, match="orthogonal"):
        BatchPipeline([systems[0], skew], params, relax=relax)
    with pytest.raises(PPGPUError, match="tuning"):
        BatchPipeline(systems, params, relax=relax, tuning=(3, 8, 4, 64))


def test_autotune_small(gpulib):
    from ppafm_gb300.batch import autotune

    systems, params, relax = _batch(nmol=3, seed=17, scale=0.25)
    cands = [(1, 32, 1, 32), (2, 8, 4, 64)]
    best, times = autotune(systems, params, relax, candidates=cands, reps=1, use_cache=False)
    assert best in cands and set(times) == set(cands) and all(t > 0 for t in times.values())


def test_batch_wait_timeout_is_reported(gpulib):
    """Failure detection without a fault: one system's force field is held back on the host
    side (its strokes wait for one more published block than exists), the strokes' bounded
    wait runs out after a 50 ms limit, the launch ends, ppgpu_device_status reports
    PPGPU_ERR_DEVICE_TIMEOUT once, and the next launch on the same context runs normally."""
    import time

    import torch

    from ppafm_gb300 import _lib
    from ppafm_gb300.batch import BatchPipeline

    L = _lib.lib()
    systems, params, relax = _batch(nmol=3, seed=5, scale=0.25)
    bp = BatchPipeline(systems, params, relax=relax)
    bp.run()
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))
    ref = [bp.outputs(j)["fzs"].clone() for j in range(len(systems))]
    assert L.ppgpu_batch_set_wait(bp.handle, 0.0, -1) == _lib.PPGPU_ERR_ARG
    assert L.ppgpu_batch_set_wait(bp.handle, 1.0, len(systems)) == _lib.PPGPU_ERR_ARG
    _lib.check(L.ppgpu_batch_set_wait(bp.handle, 0.05, 1))
    for j in range(len(systems)):
        bp.outputs(j)["fzs"].fill_(float("nan"))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bp.run()
    st = L.ppgpu_device_status(_lib.stream_handle())
    dt = time.perf_counter() - t0
    assert st == _lib.PPGPU_ERR_DEVICE_TIMEOUT, (st, _lib.last_error())
    assert "bounded" in _lib.last_error()
    assert dt < 1.9, f"the launch took {dt:.2f} s: the 50 ms limit did not end the wait"
    assert torch.isnan(bp.outputs(1)["fzs"]).all()  # the held system's strokes gave up
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))  # reported once, then cleared
    # released: the same handle runs to the same results
    _lib.check(L.ppgpu_batch_set_wait(bp.handle, 2.0, -1))
    bp.run()
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))
    for j in range(len(systems)):
        assert torch.equal(bp.outputs(j)["fzs"], ref[j]), j
    bp.close()
