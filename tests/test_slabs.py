"""One box decomposed into slabs along its outermost axis (rhyme_gb300.slabs),
on the CPU with the oracle standing in for each slab's GPU: in one process
(1-, 2- and 3-D) and as gloo ranks (world sizes 2 and 3, periodic and
outflow along the axis), the slabs' interior rows and every dt equal the
whole box's, bit for bit."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle
from rhyme_gb300 import ic, slabs
from rhyme_gb300.params import HALO, OUTFLOW, PERIODIC, REFLECTIVE, SUPERBEE, hydro_params


class OracleOps:
    """A slab is (params, cells) stepped by the oracle."""

    def __init__(self, dx):
        self.dx = dx

    def dt(self, s):
        p, cells = s
        return oracle.cfl_time_step(p, cells, self.dx)

    def fill(self, s):
        p, cells = s
        oracle.set_boundaries(p, cells)

    def get_rows(self, s, row0, n):
        p, cells = s
        return cells[:p["ndim"] + 2, row0:row0 + n].copy()

    def set_rows(self, s, row0, rows):
        p, cells = s
        cells[:p["ndim"] + 2, row0:row0 + rows.shape[1]] = rows

    def solve(self, s, dt):
        p, cells = s
        oracle.mh_solve(p, cells, self.dx, dt, nthreads=1)


def box(bc_z, seed=0):
    """A 3-D 12 x 10 x 20 box with a seeded random state."""
    nx, ny, nz = 12, 10, 20
    rng = np.random.default_rng(seed)
    g = 5.0 / 3.0
    shp = (nz, ny, nx)
    rho = 1.0 + 0.3 * rng.random(shp)
    vel = [0.2 * (rng.random(shp) - 0.5) for _ in range(3)]
    pr = 1.0 + 0.5 * rng.random(shp)
    cells = ic.empty_box(3, [nx, ny, nz])
    cells[:, 2:-2, 2:-2, 2:-2] = ic.prim_to_cons(rho, vel, pr, g)
    p = hydro_params(3, limiter=SUPERBEE, bc=[PERIODIC, REFLECTIVE, OUTFLOW, PERIODIC, bc_z, bc_z],
                     courant=0.4)
    return cells, [1.0 / nz] * 3, p


def whole(cells, dx, p, nsteps):
    c = cells.copy()
    d = oracle.run(p, c, dx, nsteps, nthreads=1)
    return c, d


def test_split_and_boundary_types():
    assert slabs.split_rows(10, 3) == [(0, 4), (4, 3), (7, 3)]
    with pytest.raises(ValueError):
        slabs.split_rows(5, 3)
    bc = [1, 2, 2, 1, PERIODIC, PERIODIC]
    assert slabs.slab_bc(bc, 3, 0, 1) == bc
    assert slabs.slab_bc(bc, 3, 0, 3)[4:] == [HALO, HALO]
    bc = [1, 2, 2, 1, OUTFLOW, REFLECTIVE]
    assert slabs.slab_bc(bc, 3, 0, 3)[4:] == [OUTFLOW, HALO]
    assert slabs.slab_bc(bc, 3, 1, 3)[4:] == [HALO, HALO]
    assert slabs.slab_bc(bc, 3, 2, 3)[4:] == [HALO, REFLECTIVE]
    assert slabs.slab_bc([PERIODIC] * 4, 2, 1, 2)[2:4] == [HALO, HALO]
    assert slabs.neighbours(0, 3, True) == (2, 1)
    assert slabs.neighbours(0, 3, False) == (None, 1)
    assert slabs.neighbours(2, 3, False) == (1, None)
    assert slabs.neighbours(0, 2, True) == (1, 1)


@pytest.mark.parametrize("bc_z,parts", [(PERIODIC, 3), (OUTFLOW, 3), (PERIODIC, 2), (REFLECTIVE, 4)])
def test_local_slabs_equal_whole_box(bc_z, parts):
    cells, dx, p = box(bc_z)
    ref, dref = whole(cells, dx, p, 6)
    nz = cells.shape[1] - 4
    parts_rows = slabs.split_rows(nz, parts)
    ss = [(dict(p, bc=slabs.slab_bc(p["bc"], 3, r, parts)), slabs.slab_cells(cells, a, c))
          for r, (a, c) in enumerate(parts_rows)]
    d = slabs.run_local(ss, [c for _, c in parts_rows], 6, OracleOps(dx), periodic=(bc_z == PERIODIC))
    assert np.array_equal(d, dref)
    for (a, c), (_, sc) in zip(parts_rows, ss):
        assert np.array_equal(sc[:, 2:2 + c], ref[:, 2 + a:2 + a + c])


def box_nd(ndim, bc_last, seed=2):
    """A 1-D (40 cells) or 2-D (14 x 24) box with a seeded random state; the
    outermost axis is the last one."""
    dims = {1: [40], 2: [14, 24]}[ndim]
    rng = np.random.default_rng(seed)
    shp = tuple(dims[::-1])
    rho = 1.0 + 0.3 * rng.random(shp)
    vel = [0.2 * (rng.random(shp) - 0.5) for _ in range(ndim)]
    pr = 1.0 + 0.5 * rng.random(shp)
    cells = ic.empty_box(ndim, dims)
    cells[ic.interior(ndim, dims)] = ic.prim_to_cons(rho, vel, pr, 5.0 / 3.0)
    bc = [REFLECTIVE, OUTFLOW][:2 * ndim - 2] + [bc_last, bc_last]
    p = hydro_params(ndim, limiter=SUPERBEE, bc=bc, courant=0.5)
    return cells, [1.0 / max(dims)] * ndim, p


@pytest.mark.parametrize("ndim,bc_last,parts", [(1, PERIODIC, 3), (1, OUTFLOW, 2), (2, PERIODIC, 3), (2, REFLECTIVE, 4)])
def test_local_slabs_equal_whole_box_1d_2d(ndim, bc_last, parts):
    cells, dx, p = box_nd(ndim, bc_last)
    ref, dref = whole(cells, dx, p, 8)
    n = cells.shape[1] - 4
    rows = slabs.split_rows(n, parts)
    ss = [(dict(p, bc=slabs.slab_bc(p["bc"], ndim, r, parts)), slabs.slab_cells(cells, a, c))
          for r, (a, c) in enumerate(rows)]
    d = slabs.run_local(ss, [c for _, c in rows], 8, OracleOps(dx), periodic=(bc_last == PERIODIC))
    assert np.array_equal(d, dref)
    for (a, c), (_, sc) in zip(rows, ss):
        assert np.array_equal(sc[:, 2:2 + c], ref[:, 2 + a:2 + a + c])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, bc_z, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cells, dx, p = box(bc_z, seed=1)
        nz = cells.shape[1] - 4
        a, c = slabs.split_rows(nz, world)[rank]
        s = (dict(p, bc=slabs.slab_bc(p["bc"], 3, rank, world)), slabs.slab_cells(cells, a, c))
        d = slabs.run_rank(s, c, 5, OracleOps(dx), bc_z == PERIODIC, rank, world)
        out[rank] = (a, c, s[1][:, 2:2 + c].copy(), d)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(180)
@pytest.mark.parametrize("world,bc_z", [(2, PERIODIC), (3, OUTFLOW)])
def test_gloo_ranks_equal_whole_box(world, bc_z):
    port = _free_port()
    # the manager process is spawned too: this process runs OpenMP threads
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, port, bc_z, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    cells, dx, p = box(bc_z, seed=1)
    ref, dref = whole(cells, dx, p, 5)
    for r in range(world):
        a, c, interior, d = res[r]
        assert np.array_equal(d, dref)
        assert np.array_equal(interior, ref[:, 2 + a:2 + a + c])
