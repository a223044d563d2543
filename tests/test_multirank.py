"""Multi-rank host logic on CPU: world-size-2 gloo process groups (no GPU).

Covers what the bench and a multi-GPU user rely on: the max-over-ranks step time, the sum
of per-rank work, and the longest-processing-time sharding of a molecule batch (every
molecule on exactly one rank, loads balanced)."""

import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from ppafm_gb300 import ranks, workloads

        r, w, _ = ranks.dist_env()
        tmax = ranks.max_over_ranks([1.0 + r, 10.0 - r])
        tsum = ranks.sum_over_ranks([float(r + 1)])
        systems = workloads.molecule_batch(seed=1, nmol=12, scale=0.2)
        costs = [ranks.system_cost(s) for s in systems]
        parts, totals = ranks.shard_lpt(costs, w)
        mine = parts[r]
        # every rank computes the same assignment; gather the counts to check coverage
        cover = ranks.sum_over_ranks([float(len(mine))])
        q.put((r, tmax, tsum, mine, cover, totals))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for r, tmax, tsum, mine, cover, totals in res:
        assert tmax == [2.0, 10.0]
        assert tsum == [3.0]
        assert cover == [12.0]
    assert sorted(res[0][3] + res[1][3]) == list(range(12))
    totals = res[0][5]
    assert max(totals) / min(totals) < 1.5


def test_lpt_balance_and_identity():
    from ppafm_gb300 import ranks

    rng = np.random.default_rng(0)
    costs = list(rng.uniform(1, 10, 64))
    parts, totals = ranks.shard_lpt(costs, 4)
    assert sorted(i for p in parts for i in p) == list(range(64))
    assert max(totals) - min(totals) <= max(costs)
    parts1, _ = ranks.shard_lpt(costs, 1)
    assert parts1 == [list(range(64))]
    assert ranks.max_over_ranks([3.0]) == [3.0]  # no process group: identity


@pytest.mark.parametrize("world", [2, 3])
def test_lpt_every_item_once(world):
    from ppafm_gb300 import ranks

    parts, _ = ranks.shard_lpt([5.0, 1.0, 1.0, 1.0, 1.0, 1.0], world)
    assert sorted(i for p in parts for i in p) == list(range(6))
    assert parts[0] == [0] or any(p == [0] for p in parts)
