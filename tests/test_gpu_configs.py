"""Parity and size-independent properties at the benchmark configurations'
full sizes (the smaller boxes of the other files cover the code paths; these
cover the sizes): the 256^3 sphere box in plain FP64 against the CPU oracle
bit for bit; conservation of mass, momentum and energy of that periodic box
in both precisions; real boxes of the 4096-box batch stepped as a batch
against the oracle bit for bit."""
import os

import numpy as np
import pytest

import oracle
from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import FP64, MIXED

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

NTHREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def spheres256():
    return ic.spheres_3d(n=256, seed=0)


def test_spheres_256_fp64_bitwise(spheres256):
    cells, dx, p = spheres256
    got = cells.copy()
    with gpu.Context(dict(p, precision=FP64)) as ctx:
        b = ctx.register_box(got)
        dts = ctx.run(b, dx, 3)
        ctx.sync_to_host(b)
    ref = cells.copy()
    dref = oracle.run(p, ref, dx, 3, nthreads=NTHREADS)
    assert np.array_equal(dts, dref)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("precision,tol", [(FP64, 1e-13), (MIXED, 1e-8)])
def test_spheres_256_conservation(spheres256, precision, tol):
    """Periodic box: the interior sums of every conserved field change only
    by rounding (relative to the sum of magnitudes)."""
    cells, dx, p = spheres256
    c = cells.copy()
    inner = (slice(None),) + (slice(2, -2),) * 3
    s0 = c[inner].reshape(5, -1).sum(axis=1)
    m0 = np.abs(c[inner]).reshape(5, -1).sum(axis=1)
    with gpu.Context(dict(p, precision=precision)) as ctx:
        b = ctx.register_box(c)
        ctx.run(b, dx, 10)
        ctx.sync_to_host(b)
    s1 = c[inner].reshape(5, -1).sum(axis=1)
    rel = np.abs(s1 - s0) / m0
    assert rel.max() <= tol, rel


def test_batch4096_boxes_fp64_bitwise():
    """Eight of the 4096 config-2 boxes (the same seeded draw), stepped as one
    batch with their own BCs and dt, against the oracle box by box."""
    items = ic.batch_boxes(4096, seed=0)
    pick = [0, 1, 2, 3, 1000, 2048, 3000, 4095]
    boxes = [items[i] for i in pick]
    states = [c.copy() for c, _, _ in boxes]
    with gpu.Context(dict(boxes[0][2], precision=FP64)) as ctx:
        hs = []
        for st, (_, dx, p) in zip(states, boxes):
            h = ctx.register_box(st)
            ctx.set_box_params(h, bc=p["bc"], limiter=p["limiter"], omega=p["omega"])
            hs.append(h)
        with ctx.batch(hs, [dx for _, dx, _ in boxes]) as bt:
            bt.run(10)
            dts = bt.dts()
        for h in hs:
            ctx.sync_to_host(h)
    for i, (st, (cells, dx, p)) in enumerate(zip(states, boxes)):
        ref = cells.copy()
        dref = oracle.run(p, ref, dx, 10, nthreads=NTHREADS)
        assert dts[i] == dref[-1], pick[i]
        assert np.array_equal(st, ref, equal_nan=True), pick[i]
