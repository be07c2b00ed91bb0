"""The Riemann solver's vacuum branches and the reference's full box layout
on the GPU, against the CPU oracle.

Vacuum: rhyme_riemann_problem_solve.f90:28-67 takes three branches when the
density on one or both sides is at or below the vacuum density (vacuum on
the right, on the left, on both sides), each with its own sampling of the
fan and the vacuum state. They are fed here element by element (every
sub-branch, at x/t = 0 and elsewhere) and inside whole steps of 1-D boxes
with a vacuum region, in plain FP64 (bit for bit) and in the mixed form,
whose sweeps hand every vacuum interface to the FP64 fix-up.

Layout: rhyme_samr_init_box.f90:32 allocates cells(..., NCMP) with
NCMP = NDIM + 3 + NSPE (cmake/CalcNumberOfComponents.cmake:4-5), NDIM + 6
with the default three species. The library moves and updates only the
NDIM + 2 hydro blocks; the temperature and species blocks are the host's
and must come back untouched through every path: register, upload (whole or
in slabs from a page-locked array), the step, host write-back and download.
"""
import numpy as np
import pytest

import oracle
from parity import assert_fp64_parity
from refcheck import GAMMA

from rhyme_gb300 import gpu, ic
from rhyme_gb300.metrics import field_errors
from rhyme_gb300.params import FP64, MIXED, hydro_params

pytestmark = pytest.mark.gpu

VAC_RHO, VAC_P = 1e-3, 1e-6


def _vacuum_rows(rng, n, ndim, g):
    """Left/right conserved states: a third with vacuum on the right, a
    third on the left, a third on both sides (densities 0, below and at
    VAC_RHO), the other side's gas in motion either way."""
    rho = 10 ** rng.uniform(-1, 1, (2, n))
    vel = rng.uniform(-2, 2, (2, ndim, n))
    pr = 10 ** rng.uniform(-1, 1, (2, n))
    kind = np.arange(n) % 3  # 0: right vacuum, 1: left vacuum, 2: both
    vac = rng.choice([0.0, 0.5 * VAC_RHO, VAC_RHO], n)
    vac2 = rng.choice([0.0, 0.25 * VAC_RHO, VAC_RHO], n)
    rho[1] = np.where(kind != 1, vac, rho[1])
    rho[0] = np.where(kind == 1, vac, np.where(kind == 2, vac2, rho[0]))
    U = []
    for s in range(2):
        u = ic.prim_to_cons(rho[s], list(vel[s]), np.where(rho[s] <= VAC_RHO, 0.5 * VAC_P, pr[s]), g).T.copy()
        U.append(u)
    return U, kind


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_riemann_vacuum_branches_vs_oracle(ndim):
    rng = np.random.default_rng(31 + ndim)
    g = GAMMA["monatomic"]
    n = 6000
    U, kind = _vacuum_rows(rng, n, ndim, g)
    p = hydro_params(ndim, gamma=g, vac_rho=VAC_RHO, vac_p=VAC_P)
    hit = set()
    with gpu.Context(p) as ctx:
        for axis in range(ndim):
            for dx, dt in ((0.0, 1.0), (2.5, 1.0), (-2.5, 1.0), (6.0, 1.0), (-6.0, 1.0), (0.7, 2.0)):
                a = ctx.riemann_problem_solve(U[0], U[1], dx, dt, axis)
                b = oracle.riemann_solve(p, U[0], U[1], dx, dt, axis)
                assert np.array_equal(a, b, equal_nan=True), (axis, dx)
                # which sub-branch each row took (the sampling tests of
                # rhyme_riemann_problem_solve.f90:28-67)
                s = dx / dt
                gm1 = g - 1.0
                for side, k in ((0, 0), (1, 1)):
                    live = U[side][kind == k]
                    v = live[:, 1 + axis] / live[:, 0]
                    pl = oracle.eos(ndim, g, p["kb_amu"], live, 0)
                    cs = pl[2]
                    if k == 0:  # gas on the left: vacuum beyond v - 2cs/gm1, fan beyond v - cs
                        hit |= {("right", "vacuum")} if np.any(s > v - 2 * cs / gm1) else set()
                        hit |= {("right", "fan")} if np.any((s <= v - 2 * cs / gm1) & (s > v - cs)) else set()
                        hit |= {("right", "state")} if np.any(s <= v - cs) else set()
                    else:  # gas on the right
                        hit |= {("left", "state")} if np.any(s > v + cs) else set()
                        hit |= {("left", "fan")} if np.any((s <= v + cs) & (s > v + 2 * cs / gm1)) else set()
                        hit |= {("left", "vacuum")} if np.any(s <= v + 2 * cs / gm1) else set()
    assert {("right", "vacuum"), ("right", "state"), ("left", "state"), ("left", "vacuum")} <= hit, hit


def _vacuum_box_1d(n=96, flip=False):
    """Gas | vacuum (rho = VAC_RHO/2) | gas, the gas moving; flipped, the
    vacuum borders the gas from the other side."""
    g = GAMMA["monatomic"]
    rho = np.full(n, 1.0)
    pr = np.full(n, 1.0)
    u = np.zeros(n)
    a, b = n // 3, 2 * n // 3
    rho[a:b], pr[a:b] = 0.5 * VAC_RHO, 0.5 * VAC_P
    rho[b:], pr[b:], u[b:] = 0.5, 0.5, -0.3
    u[:a] = 0.2
    if flip:
        rho, pr, u = rho[::-1].copy(), pr[::-1].copy(), -u[::-1]
    c = ic.empty_box(1, [n])
    c[ic.interior(1, [n])] = ic.prim_to_cons(rho, [u], pr, g)
    return c


@pytest.mark.parametrize("flip", [False, True])
@pytest.mark.parametrize("limiter", [1, 2, 3, 4])
def test_vacuum_box_steps(flip, limiter):
    """Vacuum interfaces inside whole steps: FP64 bit for bit against the
    oracle; the mixed form sends them to its FP64 fix-up and stays close to
    the FP64 result."""
    n, steps = 96, 20
    p = hydro_params(1, limiter=limiter, bc=[2, 2], vac_rho=VAC_RHO, vac_p=VAC_P, courant=0.5)
    cells = _vacuum_box_1d(n, flip)
    dx = [1.0 / n]
    ref = cells.copy()
    dref = oracle.run(p, ref, dx, steps)
    out = {}
    for prec in (FP64, MIXED):
        c = cells.copy()
        with gpu.Context(dict(p, precision=prec)) as ctx:
            b = ctx.register_box(c)
            dts = ctx.run(b, dx, steps)
            if prec == MIXED:
                assert ctx.fallback_count(b) > 0
            ctx.sync_to_host(b)
        out[prec] = (c, np.asarray(dts))
    got, dts = out[FP64]
    assert np.array_equal(got, ref) and np.array_equal(dts, dref)
    assert_fp64_parity(got, ref, 1, dts, dref)
    mixed, _ = out[MIXED]
    assert np.all(np.isfinite(mixed))
    errs = field_errors(mixed, got, 1)
    assert errs[0][0] <= 1e-5, errs


def _with_extra_components(cells, ndim, rng):
    """The hydro blocks of `cells` followed by temperature and three species
    blocks of sentinel values (NCMP = NDIM + 6)."""
    extra = rng.uniform(-7.0, 7.0, (4,) + cells.shape[1:])
    return np.ascontiguousarray(np.concatenate([cells, extra], axis=0))


@pytest.mark.parametrize("ndim", [1, 2, 3])
@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_full_component_layout_resident_run(ndim, precision):
    rng = np.random.default_rng(ndim)
    if ndim == 1:
        cells, dx, p = ic.riemann_1d(n=200, seed=3)
    elif ndim == 2:
        cells, dx, p = ic.slab_2d(n=48, seed=3)
    else:
        cells, dx, p = ic.spheres_3d(n=20, nspheres=3, seed=3)
    full = _with_extra_components(cells, ndim, rng)
    sentinels = full[ndim + 2:].copy()
    steps = 6
    with gpu.Context(dict(p, precision=precision)) as ctx:
        b = ctx.register_box(full)
        dts = ctx.run(b, dx, steps)
        ctx.sync_to_host(b)
        ctx.sync_to_device(b)  # a second upload, from the downloaded host array
        dts2 = ctx.run(b, dx, 2)
        ctx.sync_to_host(b)
    assert np.array_equal(full[ndim + 2:], sentinels)
    ref = cells.copy()
    dref = oracle.run(p, ref, dx, steps + 2)
    if precision == FP64:
        assert np.array_equal(full[:ndim + 2], ref)
        assert np.array_equal(np.concatenate([dts, dts2]), dref)
    else:
        alone = cells.copy()
        with gpu.Context(dict(p, precision=MIXED)) as ctx:
            b = ctx.register_box(alone)
            ctx.run(b, dx, steps)
            ctx.sync_to_host(b)
            ctx.sync_to_device(b)
            ctx.run(b, dx, 2)
            ctx.sync_to_host(b)
        assert np.array_equal(full[:ndim + 2], alone)


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_full_component_layout_drop_in_loop(precision):
    """The drop-in loop with host write-back (the shim's default) on a 3-D box
    of more than 16 MiB of hydro state: in mixed precision the upload and the
    solve's write-back run in slabs from the page-locked host array, whose
    component stride then spans NDIM + 6 blocks."""
    rng = np.random.default_rng(5)
    cells, dx, p = ic.spheres_3d(n=72, nspheres=4, seed=5)
    full = _with_extra_components(cells, 3, rng)
    sentinels = full[5:].copy()
    ref = cells.copy()
    p = dict(p, precision=precision)
    with gpu.Context(p) as ctx:
        b = ctx.register_box(ref)
        dref = ctx.run(b, dx, 3)
        ctx.sync_to_host(b)
    with gpu.Context(p) as ctx:
        b = ctx.register_box(full)
        ctx.set_host_writeback(b)
        for k in range(3):
            ctx.sync_to_device(b)
            dt = ctx.cfl_time_step(b, dx)
            ctx.set_boundaries(b)
            ctx.muscl_hancock_solve(b, dx, dt)
            ctx.sync_to_host(b)
            assert dt == dref[k]
    assert np.array_equal(full[5:], sentinels)
    assert np.array_equal(full[:5], ref)
    if precision == FP64:
        oref = cells.copy()
        oracle.run(dict(p, precision=FP64), oref, dx, 3)
        assert np.array_equal(full[:5], oref)
