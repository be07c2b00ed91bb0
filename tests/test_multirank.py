"""The N>1 path on CPU: cost-balanced partition of independent boxes over
ranks and the timing reductions, with world-size-2 gloo process groups."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from rhyme_gb300 import ic, shard


def test_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    costs = [int(c) for c in rng.integers(1, 1000, 97)]
    for world in (1, 2, 3, 8):
        parts = shard.partition(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        lower = max(max(costs), sum(costs) / world)
        assert max(loads) <= 4.0 / 3.0 * lower + max(costs)
    assert shard.partition(costs, 2) == shard.partition(list(costs), 2)  # deterministic


def test_box_cost_counts_interior_cells():
    cells = ic.empty_box(3, [8, 16, 24])
    assert shard.box_cost(cells, 10) == 8 * 16 * 24 * 10


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(1)
        boxes = [ic.batch_box(rng, edges=(8, 16))[0] for _ in range(9)]
        costs = [shard.box_cost(b) for b in boxes]
        mine = shard.partition(costs, world)[rank]
        load = sum(costs[i] for i in mine)
        total = shard.reduce_scalar(load, world, "sum")
        worst = shard.reduce_scalar(load, world, "max")
        out[rank] = (sorted(mine), load, total, worst)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_share_boxes():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    a, b = res[0], res[1]
    assert set(a[0]).isdisjoint(b[0]) and sorted(a[0] + b[0]) == list(range(9))
    assert a[2] == b[2] == a[1] + b[1]
    assert a[3] == b[3] == max(a[1], b[1])
