"""Partition of independent boxes (or requests) over ranks, one GPU each.

Boxes never exchange data, so a multi-GPU run is a set of independent
partitions with no collective on the data path; the only collectives are the
bench's barrier and its max/sum of timings. The partition balances cost
(interior cells x steps): longest-processing-time-first, each box to the
rank with the least cost so far, ties to the lower rank, which is
deterministic and within 4/3 of the optimal makespan.
"""
import heapq

import numpy as np


def box_cost(cells, nsteps=1):
    """Interior cells x steps of a box in the reference layout (NCMP, ...)."""
    return int(np.prod([s - 4 for s in cells.shape[1:]])) * int(nsteps)


def partition(costs, world):
    """List of index lists, one per rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    for p in parts:
        p.sort()
    return parts


def my_share(items, costs, rank, world):
    """The items of `rank` under partition()."""
    return [items[i] for i in partition(costs, world)[rank]]


def reduce_scalar(x, world, op="max", device="cpu"):
    """max or sum of a Python float over ranks (identity for one rank)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())
