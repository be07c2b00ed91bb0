"""Batches of independent boxes (rhyme_gpu_batch_*): each box stepped inside
a batch, with its own boundary types, limiter, cell size and dt, equals the
same box stepped alone; FP64 bit for bit, mixed precision within 1e-12 (the
FP64 fix-up of queued interfaces adds with atomics)."""
import numpy as np
import pytest

from parity import field_errors

from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import FP64, MIXED, OUTFLOW, PERIODIC, REFLECTIVE, hydro_params

pytestmark = pytest.mark.gpu


def _boxes3d(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        cells, dx, p = ic.batch_box(rng, edges=(8, 12, 16, 20, 24))
        lim = int(rng.integers(1, 5))
        out.append((cells, dx, dict(p, limiter=lim)))
    return out


def _alone(p, cells, dx, nsteps):
    c = cells.copy()
    with gpu.Context(p) as ctx:
        box = ctx.register_box(c)
        dts = ctx.run(box, dx, nsteps)
        ctx.sync_to_host(box)
    return c, dts[-1]


def _batched(base, items, nsteps, chunks=(None,)):
    states = [c.copy() for c, _, _ in items]
    with gpu.Context(base) as ctx:
        boxes = []
        for st, (_, dx, p) in zip(states, items):
            b = ctx.register_box(st)
            ctx.set_box_params(b, bc=p["bc"], limiter=p["limiter"], omega=p["omega"])
            boxes.append(b)
        with ctx.batch(boxes, [dx for _, dx, _ in items]) as bt:
            done = 0
            for k in chunks:
                k = nsteps - done if k is None else k
                bt.run(k)
                done += k
            dts = bt.dts()
        for b in boxes:
            ctx.sync_to_host(b)
    return states, dts


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_batch_3d_equals_alone(precision):
    items = _boxes3d(7, seed=3)
    base = dict(items[0][2], precision=precision)
    got, dts = _batched(base, items, 6, chunks=(2, 1, 3))
    for i, (cells, dx, p) in enumerate(items):
        ref, dt = _alone(dict(p, precision=precision), cells, dx, 6)
        if precision == FP64:
            assert np.array_equal(got[i], ref), i
            assert dts[i] == dt
        else:
            errs = field_errors(got[i], ref, 3)
            assert max(e[0] for e in errs) <= 1e-12, (i, errs)
            assert abs(dts[i] - dt) <= 1e-12 * dt


@pytest.mark.parametrize("ndim", [1, 2])
def test_batch_low_dim_equals_alone(ndim):
    rng = np.random.default_rng(ndim)
    items = []
    for k in range(5):
        dims = [int(x) for x in rng.integers(6, 40, ndim)]
        cells = ic.empty_box(ndim, dims)
        shp = tuple(dims[::-1])
        rho = 1.0 + 0.3 * rng.uniform(size=shp)
        vel = [0.2 * rng.uniform(-1, 1, shp) for _ in range(ndim)]
        pr = 1.0 + 0.3 * rng.uniform(size=shp)
        cells[ic.interior(ndim, dims)] = ic.prim_to_cons(rho, vel, pr, 5.0 / 3.0)
        bc = [int(rng.choice([REFLECTIVE, OUTFLOW, PERIODIC])) for _ in range(6)]
        p = hydro_params(ndim, limiter=int(rng.integers(1, 5)), bc=bc, courant=0.4)
        items.append((cells, [1.0 / (10 + k)] * ndim, p))
    got, dts = _batched(items[0][2], items, 8)
    for i, (cells, dx, p) in enumerate(items):
        ref, dt = _alone(p, cells, dx, 8)
        assert np.array_equal(got[i], ref), i
        assert dts[i] == dt


def test_batch_survives_single_steps_in_between():
    """A box stepped on its own between batch runs keeps the batch correct."""
    items = _boxes3d(3, seed=9)
    base = items[0][2]
    states = [c.copy() for c, _, _ in items]
    with gpu.Context(base) as ctx:
        boxes = []
        for st, (_, dx, p) in zip(states, items):
            b = ctx.register_box(st)
            ctx.set_box_params(b, bc=p["bc"], limiter=p["limiter"])
            boxes.append(b)
        with ctx.batch(boxes, [dx for _, dx, _ in items]) as bt:
            bt.run(2)
            ctx.run(boxes[1], items[1][1], 1)
            bt.run(2)
        for b in boxes:
            ctx.sync_to_host(b)
    for i, (cells, dx, p) in enumerate(items):
        ref, _ = _alone(p, cells, dx, 5 if i == 1 else 4)
        assert np.array_equal(states[i], ref), i
