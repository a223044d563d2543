"""Host-side logic for several GPUs, one process per GPU.

The hot path shards without any exchange on the data path: molecules of a batch are
independent, and a single system's pixels are independent once every rank holds the force
field.  What remains for the host is (1) assigning work to ranks -- longest-processing-time
first over the estimated cost of each molecule (grid points x atoms for the force field plus
pixel heights for the relaxation) -- and (2) reporting: the wall time of a step is the
maximum over ranks.  Both run on any torch.distributed backend (gloo on CPU in the tests,
nccl on GPUs in the bench).
"""

import heapq
import os

import numpy as np


def dist_env():
    """(rank, world size, local rank) from the torchrun environment (1 process if unset)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def system_cost(w, atom_images=9):
    """Estimated cost of one molecule: force-field pairs + relaxed pixel heights (weighted by
    the measured ratio of the two on GB300: one pixel height ~ 1e3 pairs)."""
    npts = float(np.prod(w["gridN"]))
    pairs = npts * len(w["Zs"]) * atom_images
    nx = int(round((w["scanMax"][0] - w["scanMin"][0]) / w["scanStep"][0])) + 1
    ny = int(round((w["scanMax"][1] - w["scanMin"][1]) / w["scanStep"][1])) + 1
    nz = int(round((w["scanMax"][2] - w["scanMin"][2]) / w["scanStep"][2])) + 1
    return pairs + 1e3 * nx * ny * nz


def shard_lpt(costs, world):
    """Longest-processing-time-first assignment of items to `world` ranks.  Returns a list of
    index lists (one per rank, each in ascending order) and the per-rank cost totals."""
    order = sorted(range(len(costs)), key=lambda i: -costs[i])
    heap = [(0.0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        c, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (c + costs[i], r))
    totals = [0.0] * world
    for r in range(world):
        parts[r].sort()
        totals[r] = float(sum(costs[i] for i in parts[r]))
    return parts, totals


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of a list of floats over all ranks (identity without a process
    group)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def sum_over_ranks(values, device="cpu"):
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return [float(v) for v in t.tolist()]
