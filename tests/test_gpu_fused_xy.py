"""The x and y sweeps of a 3-D mixed box as one kernel (sweep_xy_kernel)
against the two per-axis sweeps (RHYME_GPU_XY=0): the fused kernel performs
the same operations (the FIRST and MID accumulations with the same
roundings), so the states and dts of a resident run must be bit-identical,
for a box whose extents are multiples of the 16 x 16 tile and for one whose
x and y extents are not. A box whose mirror rows are not a multiple of 16
bytes cannot take the plane's tensor copy and runs the per-axis sweeps; the
profile then reports them separately."""
import os

import numpy as np
import pytest

from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import MIXED

pytestmark = pytest.mark.gpu


def run(cells, dx, p, steps, fuse):
    old = os.environ.get("RHYME_GPU_XY")
    os.environ["RHYME_GPU_XY"] = "1" if fuse else "0"
    try:
        c = cells.copy()
        with gpu.Context(dict(p, precision=MIXED)) as ctx:
            b = ctx.register_box(c)
            dts = list(ctx.run(b, dx, steps))
            phases = ctx.profile_steps(b, dx, 2)
            dts += list(ctx.run(b, dx, 2))
            fb = ctx.fallback_count(b)
            ctx.sync_to_host(b)
    finally:
        if old is None:
            del os.environ["RHYME_GPU_XY"]
        else:
            os.environ["RHYME_GPU_XY"] = old
    return c, np.asarray(dts), phases, fb


def boxes():
    cells, dx, p = ic.spheres_3d(n=48, nspheres=6, seed=4)
    yield "48^3", cells, dx, p, True
    # interior 40 x 36 x 20: partial tiles along y
    yield "40x36x20", np.ascontiguousarray(cells[:, :24, :40, :44]), [1.0 / 48] * 3, p, True
    # interior 37 x 36 x 20: rows of 41 floats, not a multiple of 16 bytes
    yield "37x36x20", np.ascontiguousarray(cells[:, :24, :40, :41]), [1.0 / 48] * 3, p, False


@pytest.mark.parametrize("case", list(boxes()), ids=lambda c: c[0])
def test_fused_xy_equals_two_sweeps(case):
    _, cells, dx, p, fusable = case
    a, da, pa, fa = run(cells, dx, p, 6, True)
    b, db, pb, fb = run(cells, dx, p, 6, False)
    assert fa == fb == 0
    assert np.array_equal(da, db)
    assert np.array_equal(a, b)
    assert ("sweep_xy" in pa) == fusable
    assert "sweep_xy" not in pb and "sweep_y" in pb
