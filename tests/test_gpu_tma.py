"""TMA staging of the mixed sweeps.

Where a box's FP32 mirror has rows of a multiple of 16 bytes (x extent plus
ghosts a multiple of 4 cells), each single-box sweep tile stages its slab
with one cp.async.bulk.tensor copy; elsewhere, and with RHYME_GPU_TMA=0 in
the environment, with coalesced loads. Both must give the same bits, in the
whole-box step and in the pipelined solve of a page-locked box in slabs
(whose tiles address the whole box's map at an offset)."""
import os

import numpy as np
import pytest

from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import MIXED

pytestmark = pytest.mark.gpu


def _run(cells, dx, p, steps, tma, drop_in=False):
    old = os.environ.get("RHYME_GPU_TMA")
    os.environ["RHYME_GPU_TMA"] = "1" if tma else "0"
    try:
        c = cells.copy()
        n0 = gpu.tma_launches()
        with gpu.Context(dict(p, precision=MIXED)) as ctx:
            b = ctx.register_box(c)
            if drop_in:
                ctx.set_host_writeback(b)
                dts = []
                for _ in range(steps):
                    ctx.sync_to_device(b)
                    dt = ctx.cfl_time_step(b, dx)
                    ctx.set_boundaries(b)
                    ctx.muscl_hancock_solve(b, dx, dt)
                    ctx.sync_to_host(b)
                    dts.append(dt)
            else:
                dts = ctx.run(b, dx, steps)
            ctx.sync_to_host(b)
        return c, np.asarray(dts), gpu.tma_launches() - n0
    finally:
        if old is None:
            del os.environ["RHYME_GPU_TMA"]
        else:
            os.environ["RHYME_GPU_TMA"] = old


@pytest.mark.parametrize("case", ["spheres3d_60", "spheres3d_28", "slab2d_124", "slab2d_odd"])
def test_tma_staging_equals_coalesced_loads(case):
    if case.startswith("spheres3d"):
        n = int(case.split("_")[1])
        cells, dx, p = ic.spheres_3d(n=n, nspheres=4, seed=2)
    elif case == "slab2d_124":
        cells, dx, p = ic.slab_2d(n=124, seed=2)
    else:
        cells, dx, p = ic.slab_2d(n=61, seed=2)  # 65 cells per row: no tensor copies
    a, da, na = _run(cells, dx, p, 8, tma=True)
    b, db, nb = _run(cells, dx, p, 8, tma=False)
    assert nb == 0
    if case == "slab2d_odd":
        assert na == 0
    else:
        assert na > 0
    assert np.array_equal(da, db)
    assert np.array_equal(a, b)


def test_tma_staging_in_the_pipelined_drop_in_loop():
    """A 3-D box of more than 16 MiB solved in slabs with host write-back:
    the slab tiles offset their tensor coordinates by the slab's first row."""
    cells, dx, p = ic.spheres_3d(n=76, nspheres=4, seed=9)
    a, da, na = _run(cells, dx, p, 3, tma=True, drop_in=True)
    b, db, nb = _run(cells, dx, p, 3, tma=False, drop_in=True)
    assert na > 0 and nb == 0
    assert np.array_equal(da, db)
    assert np.array_equal(a, b)
