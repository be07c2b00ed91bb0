"""The drop-in loop with overlapped copies against the device-resident run.

A 2-/3-D mixed-precision box of 16 MiB or more with a page-locked host array
is uploaded in slabs of rows of its outermost axis, each slab's CFL maximum
taken as it arrives (rhyme_gpu_sync_to_device), and with host write-back on
it is solved in slabs whose finished rows are copied back while the next
slab is solved (rhyme_gpu_set_host_writeback, rhyme_gpu_mh_solve). The
loop sync_to_device -> cfl_time_step -> set_boundaries -> solve ->
sync_to_host must give the state and the dt of every step that
rhyme_gpu_run (whole-box kernels, CUDA graph) gives: bit for bit when no
interface goes to the FP64 fallback, whose double atomics may add the two
corrections of a cell in either order.
"""
import numpy as np
import pytest

from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import FP64, MINMOD, MIXED, OUTFLOW, hydro_params

pytestmark = pytest.mark.gpu


def drop_in(p, cells, dx, nsteps, writeback=True):
    host = cells.copy()
    dts = []
    with gpu.Context(p) as ctx:
        box = ctx.register_box(host)
        ctx.set_host_writeback(box, writeback)
        for _ in range(nsteps):
            ctx.sync_to_device(box)
            dt = ctx.cfl_time_step(box, dx)
            ctx.set_boundaries(box)
            ctx.muscl_hancock_solve(box, dx, dt)
            ctx.sync_to_host(box)
            dts.append(dt)
        fb = ctx.fallback_count(box)
    return host, np.array(dts), fb


def resident(p, cells, dx, nsteps):
    c = cells.copy()
    with gpu.Context(p) as ctx:
        box = ctx.register_box(c)
        dts = ctx.run(box, dx, nsteps)
        fb = ctx.fallback_count(box)
        ctx.sync_to_host(box)
    return c, dts, fb


def test_overlapped_drop_in_matches_run_3d():
    # 76^3 cells with ghosts x 5 components x 8 B = 17.6 MB: above the
    # threshold of the slab path
    cells, dx, p = ic.spheres_3d(n=72, nspheres=8, seed=3)
    q = dict(p, precision=MIXED)
    a, da, fa = resident(q, cells, dx, 6)
    b, db, fb = drop_in(q, cells, dx, 6, writeback=True)
    c, dc, fc = drop_in(q, cells, dx, 6, writeback=False)
    assert fa == fb == fc == 0
    assert np.array_equal(da, db) and np.array_equal(da, dc)
    assert np.array_equal(a, b)
    assert np.array_equal(a, c)


def test_fp64_write_back_matches_run():
    """Plain FP64 (no slab path): the solve's write-back is one copy after it,
    and the drop-in loop still equals the resident run bit for bit."""
    cells, dx, p = ic.spheres_3d(n=32, nspheres=4, seed=6)
    q = dict(p, precision=FP64)
    a, da, _ = resident(q, cells, dx, 4)
    b, db, _ = drop_in(q, cells, dx, 4, writeback=True)
    assert np.array_equal(da, db)
    assert np.array_equal(a, b)


def test_overlapped_drop_in_matches_run_2d():
    # 2-D: slabs of rows along y; 1028 x 1028 x 4 x 8 B = 33.8 MB
    n = 1024
    rng = np.random.default_rng(5)
    g = 5.0 / 3.0
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    rho = 1.0 + 0.3 * np.exp(-((X - 0.4) ** 2 + (Y - 0.6) ** 2) / 0.02) + 0.01 * rng.random((n, n))
    pr = 1.0 + 0.5 * np.exp(-((X - 0.6) ** 2 + (Y - 0.3) ** 2) / 0.01)
    cells = ic.empty_box(2, [n, n])
    cells[:, 2:-2, 2:-2] = ic.prim_to_cons(rho, [0.2 * np.ones_like(rho), -0.1 * np.ones_like(rho)], pr, g)
    p = hydro_params(2, limiter=MINMOD, bc=[OUTFLOW] * 4, courant=0.5, precision=MIXED)
    a, da, fa = resident(p, cells, [1.0 / n] * 2, 4)
    b, db, fb = drop_in(p, cells, [1.0 / n] * 2, 4)
    assert fa == fb == 0
    assert np.array_equal(da, db)
    assert np.array_equal(a, b)


def test_overlapped_solve_fallback_at_slab_boundary():
    """Receding states along z beyond the vacuum-generation limit (the 1-D
    near-vacuum case of the mixed tests, extruded over 64 x 64) with the
    discontinuity between cells 48 and 49. With the size-rule tile shapes
    (16 cells along z) the slabs hold 16 rows, so that interface lies
    between two slabs: the second slab queues its FP64 fix-up, which
    corrects a row the first slab finished; that row must be copied back
    after the correction."""
    nx, ny, nz = 64, 64, 96
    g = 5.0 / 3.0
    cells = ic.empty_box(3, [nx, ny, nz])
    z = np.arange(nz)[:, None, None] * np.ones((1, ny, nx))
    rho = np.ones((nz, ny, nx))
    w = np.where(z < 48, -3.0, 3.0)
    pr = np.full((nz, ny, nx), 0.4)
    zero = np.zeros_like(rho)
    cells[:, 2:-2, 2:-2, 2:-2] = ic.prim_to_cons(rho, [zero, zero, w], pr, g)
    p = hydro_params(3, limiter=MINMOD, bc=[OUTFLOW] * 6, vac_rho=1e-8, vac_p=1e-10, courant=0.3,
                     precision=MIXED, sweep_tuning=1)
    dx = [1.0 / nz] * 3
    a, da, fa = resident(p, cells, dx, 12)
    b, db, fb = drop_in(p, cells, dx, 12)
    assert fa > 0 and fb > 0
    assert np.isfinite(a).all() and np.isfinite(b).all()
    # whole arrays, ghosts included, relative to the density's L1 norm (the x
    # and y momenta are rounding noise of the FP64 fix-up, about 1e-16); a
    # correction lost or applied after its row was copied would show as an
    # error of order 1e-3
    scale = np.abs(a[0]).sum()
    for k in range(5):
        assert np.abs(b[k] - a[k]).sum() <= 1e-12 * max(scale, np.abs(a[k]).sum()), k
    assert np.max(np.abs(db - da) / da) <= 1e-12


@pytest.mark.parametrize("split", [[12], [5, 7], [1, 1, 10]])
def test_resident_run_carries_the_cfl_pass(split):
    """In mixed precision the resident run carries the CFL pass: the last
    sweep of a step writes the next state's FP32 mirror and folds its signal
    speeds, and the next step only forms dt from that maximum. The dts and
    states must equal those of the step-by-step loop (whole CFL pass every
    step) bit for bit, across run calls split anywhere and with the state
    downloaded and uploaded again between calls (which drops the carry)."""
    cells, dx, p = ic.spheres_3d(n=44, nspheres=5, seed=12)
    q = dict(p, precision=MIXED)
    a = cells.copy()
    dts = []
    with gpu.Context(q) as ctx:
        box = ctx.register_box(a)
        for k, n in enumerate(split):
            dts.extend(ctx.run(box, dx, n))
            if k == 1:
                ctx.sync_to_host(box)
                ctx.sync_to_device(box)
        assert ctx.fallback_count(box) == 0
        ctx.sync_to_host(box)
    b = cells.copy()
    ref = []
    with gpu.Context(q) as ctx:
        box = ctx.register_box(b)
        for _ in range(sum(split)):
            dt = ctx.cfl_time_step(box, dx)
            ctx.set_boundaries(box)
            ctx.muscl_hancock_solve(box, dx, dt)
            ref.append(dt)
        ctx.sync_to_host(box)
    assert np.array_equal(np.asarray(dts), np.asarray(ref))
    assert np.array_equal(a, b)
