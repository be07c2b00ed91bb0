"""One box decomposed into slabs along its outermost axis on the GPU: the
slabs are boxes of one context, their halo faces of type HALO filled by
rhyme_gpu_get_rows / rhyme_gpu_set_rows, dt the minimum of the slabs' dt
(rhyme_gb300.slabs.run_local). The slabs' interior rows and every dt equal
the whole box's, bit for bit, in plain FP64 and in mixed precision (none of
these steps sends an interface to the FP64 fallback, whose atomics could
add two corrections of a cell in either order)."""
import numpy as np
import pytest

from rhyme_gb300 import gpu, ic, slabs
from rhyme_gb300.params import FP64, MIXED, OUTFLOW, PERIODIC

pytestmark = pytest.mark.gpu


def whole(cells, dx, p, nsteps):
    c = cells.copy()
    with gpu.Context(p) as ctx:
        b = ctx.register_box(c)
        dts = []
        for _ in range(nsteps):
            dt = ctx.cfl_time_step(b, dx)
            ctx.set_boundaries(b)
            ctx.muscl_hancock_solve(b, dx, dt)
            dts.append(dt)
        fb = ctx.fallback_count(b) if p["precision"] == MIXED else 0
        ctx.sync_to_host(b)
    return c, np.array(dts), fb


def decomposed(cells, dx, p, nsteps, parts):
    nz = cells.shape[1] - 4
    rows = slabs.split_rows(nz, parts)
    arrays = [slabs.slab_cells(cells, a, c) for a, c in rows]
    periodic = p["bc"][4] == PERIODIC and p["bc"][5] == PERIODIC
    with gpu.Context(p) as ctx:
        ss = []
        for r, arr in enumerate(arrays):
            b = ctx.register_box(arr)
            ctx.set_box_params(b, bc=slabs.slab_bc(p["bc"], 3, r, parts), limiter=p["limiter"], omega=p["omega"])
            ss.append((ctx, b))
        dts = slabs.run_local(ss, [c for _, c in rows], nsteps, slabs.GpuOps(dx), periodic)
        fb = sum(ctx.fallback_count(b) for _, b in ss) if p["precision"] == MIXED else 0
        for _, b in ss:
            ctx.sync_to_host(b)
    return rows, arrays, dts, fb


@pytest.mark.parametrize("precision,parts,bc_z", [(MIXED, 3, PERIODIC), (FP64, 2, PERIODIC), (MIXED, 4, OUTFLOW)])
def test_slabs_equal_whole_box(precision, parts, bc_z):
    cells, dx, p = ic.spheres_3d(n=48, nspheres=6, seed=4)
    p = dict(p, precision=precision, bc=[PERIODIC] * 4 + [bc_z, bc_z])
    ref, dref, fa = whole(cells, dx, p, 8)
    rows, arrays, d, fb = decomposed(cells, dx, p, 8, parts)
    assert fa == 0 and fb == 0
    assert np.array_equal(d, dref)
    for (a, c), arr in zip(rows, arrays):
        assert np.array_equal(arr[:, 2:2 + c], ref[:, 2 + a:2 + a + c])


class DeviceRowOps(slabs.GpuOps):
    """The halo rows through CUDA tensors (device to device), as run_rank
    does under NCCL."""

    def get_rows(self, s, row0, n):
        import torch
        out = torch.empty(self.rows_shape(s, n), dtype=torch.float64, device="cuda")
        self.rows_into(s, row0, n, out)
        return out


def test_rows_through_cuda_tensors():
    """get_rows into / set_rows from device memory equal the host copies."""
    torch = pytest.importorskip("torch")
    cells, dx, p = ic.spheres_3d(n=24, nspheres=2, seed=1)
    with gpu.Context(dict(p, precision=FP64)) as ctx:
        b = ctx.register_box(cells.copy())
        host = ctx.get_rows(b, 3, 2)
        dev = torch.empty(ctx.rows_shape(b, 2), dtype=torch.float64, device="cuda")
        ctx.get_rows(b, 3, 2, out=dev)
        assert np.array_equal(dev.cpu().numpy(), host)
        ctx.set_rows(b, 0, dev * 2.0)
        assert np.array_equal(ctx.get_rows(b, 0, 2), 2.0 * host)


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_slabs_with_device_rows_equal_whole_box(precision):
    cells, dx, p = ic.spheres_3d(n=40, nspheres=5, seed=6)
    p = dict(p, precision=precision, bc=[PERIODIC] * 6)
    ref, dref, _ = whole(cells, dx, p, 6)
    nz = cells.shape[1] - 4
    rows = slabs.split_rows(nz, 3)
    arrays = [slabs.slab_cells(cells, a, c) for a, c in rows]
    with gpu.Context(p) as ctx:
        ss = []
        for r, arr in enumerate(arrays):
            b = ctx.register_box(arr)
            ctx.set_box_params(b, bc=slabs.slab_bc(p["bc"], 3, r, 3), limiter=p["limiter"], omega=p["omega"])
            ss.append((ctx, b))
        d = slabs.run_local(ss, [c for _, c in rows], 6, DeviceRowOps(dx), True)
        for _, b in ss:
            ctx.sync_to_host(b)
    assert np.array_equal(d, dref)
    for (a, c), arr in zip(rows, arrays):
        assert np.array_equal(arr[:, 2:2 + c], ref[:, 2 + a:2 + a + c])
