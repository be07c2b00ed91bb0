"""Autotuner of the mixed-precision sweeps: the chosen tile shapes come from
the candidate set, and the result of a step does not depend on the shape
(each face state and interface is computed by one thread from the same FP32
values with the same operations, and the accumulation rounds explicitly)."""
import numpy as np
import pytest

from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import MIXED, OUTFLOW, PERIODIC, REFLECTIVE, hydro_params

pytestmark = pytest.mark.gpu

# tiles: (cells along the axis, pencils)
CANDIDATES = {1: [(64, 1), (128, 1), (256, 1), (512, 1)],
              2: [(8, 32), (16, 16), (32, 8), (64, 4)],
              3: [(8, 32), (16, 16), (32, 8), (64, 4)]}


def _smooth_box(ndim, dims, seed):
    rng = np.random.default_rng(seed)
    cells = ic.empty_box(ndim, dims)
    shp = tuple(dims[::-1])
    grids = np.indices(shp)[::-1]
    rho = 1.0 + 0.2 * np.sin(2 * np.pi * (grids[0] + rng.uniform()) / max(dims))
    vel = [0.1 * np.cos(2 * np.pi * grids[a % ndim] / dims[a % ndim]) for a in range(ndim)]
    pr = 1.0 + 0.1 * rng.uniform(size=shp)
    cells[ic.interior(ndim, dims)] = ic.prim_to_cons(rho, vel, pr, 5.0 / 3.0)
    return cells


def _run(p, cells, dx, nsteps, tuning):
    c = cells.copy()
    with gpu.Context(dict(p, precision=MIXED, sweep_tuning=tuning)) as ctx:
        b = ctx.register_box(c)
        plan = ctx.sweep_plan(b, dx)
        ctx.run(b, dx, nsteps)
        fb = ctx.fallback_count(b)
        ctx.sync_to_host(b)
    return c, plan, fb


@pytest.mark.parametrize("ndim,dims", [(1, [700]), (2, [40, 72]), (3, [24, 8, 40]), (3, [64, 64, 64])])
def test_tuned_equals_fixed(ndim, dims):
    cells = _smooth_box(ndim, dims, seed=ndim)
    courant = {1: 0.8, 2: 0.5, 3: 0.3}[ndim]
    p = hydro_params(ndim, bc=[PERIODIC] * 6, courant=courant)
    dx = [1.0 / max(dims)] * ndim
    a, plan_a, fa = _run(p, cells, dx, 6, 0)
    b, plan_b, fb = _run(p, cells, dx, 6, 1)
    assert len(plan_a) == ndim and len(plan_b) == ndim
    assert all(s in CANDIDATES[ndim] for s in plan_a + plan_b), (plan_a, plan_b)
    assert fa == 0 and fb == 0
    assert np.array_equal(a, b), (plan_a, plan_b)
    print(ndim, dims, "tuned", plan_a, "fixed", plan_b)


def test_size_rule_small_boxes():
    """The size rule gives 8-cell tiles to 8-cell boxes."""
    cells = _smooth_box(3, [8, 8, 8], seed=0)
    with gpu.Context(hydro_params(3, precision=MIXED, sweep_tuning=1, courant=0.3)) as ctx:
        b = ctx.register_box(cells)
        assert ctx.sweep_plan(b, [1 / 8.0] * 3) == [(8, 32)] * 3


def test_batch_mixed_sizes_tuned():
    """A batch whose boxes fall in different size classes (different tile
    shapes per class) equals its boxes stepped alone."""
    rng = np.random.default_rng(4)
    items = []
    for dims in ([8, 8, 8], [64, 16, 8], [40, 40, 40], [8, 56, 24], [16, 16, 64]):
        cells = _smooth_box(3, dims, seed=int(rng.integers(0, 100)))
        bc = [int(rng.choice([REFLECTIVE, OUTFLOW])) for _ in range(6)]
        items.append((cells, [1.0 / 64] * 3, hydro_params(3, bc=bc, courant=0.3, precision=MIXED)))
    base = items[0][2]
    states = [c.copy() for c, _, _ in items]
    with gpu.Context(base) as ctx:
        boxes = []
        for st, (_, dx, p) in zip(states, items):
            bx = ctx.register_box(st)
            ctx.set_box_params(bx, bc=p["bc"], limiter=p["limiter"], omega=p["omega"])
            boxes.append(bx)
        plans = [ctx.sweep_plan(bx, dx) for bx, (_, dx, _) in zip(boxes, items)]
        with ctx.batch(boxes, [dx for _, dx, _ in items]) as bt:
            bt.run(5)
        for bx in boxes:
            ctx.sync_to_host(bx)
    for st, (cells, dx, p) in zip(states, items):
        alone = cells.copy()
        with gpu.Context(p) as ctx:
            bx = ctx.register_box(alone)
            ctx.run(bx, dx, 5)
            ctx.sync_to_host(bx)
        assert np.array_equal(st, alone)
    print("plans", plans)
