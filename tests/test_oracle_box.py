"""Box-level checks of the CPU oracle: ghost fill, CFL, whole steps (CPU only).

The ghost-fill and CFL cases restate rhyme_samr_bc_set_*_boundary_test.f90
and rhyme_cfl_dt_test.f90; the whole-step cases check properties the
reference's solve tests leave unpinned (conservation, symmetry, agreement of
the two solver orderings, Sod against its analytic solution).
"""
import numpy as np
import pytest

import oracle
from refcheck import GAMMA, KB_AMU_SI, to_be

from rhyme_gb300 import ic


def _params(ndim, bc, limiter=2, solver_type=2, gamma=GAMMA["monatomic"]):
    return dict(ndim=ndim, gamma=gamma, kb_amu=KB_AMU_SI, courant=0.8, limiter=limiter,
                omega=0.0, vac_rho=0.0, vac_p=0.0, tol=1e-6, n_iter=100, bc=list(bc),
                solver_type=solver_type)


def _random_box(ndim, dims, seed=1):
    rng = np.random.default_rng(seed)
    shape = (ndim + 2,) + tuple(d + 4 for d in dims[::-1])
    cells = np.zeros(shape)
    interior = (slice(None),) + tuple(slice(2, d + 2) for d in dims[::-1])
    rho = rng.uniform(0.5, 2.0, shape[1:])
    vel = rng.uniform(-0.5, 0.5, (ndim,) + shape[1:])
    p = rng.uniform(0.5, 2.0, shape[1:])
    full = np.zeros(shape)
    full[0] = rho
    full[1:ndim + 1] = rho * vel
    full[ndim + 1] = 0.5 * rho * (vel * vel).sum(0) + p / (GAMMA["monatomic"] - 1.0)
    cells[interior] = full[interior]
    return cells


def _face(cells, ndim, axis, idx):
    """Slice of ghost/interior layer `idx` (Fortran index) along `axis`,
    restricted to interior transverse positions."""
    sl = [slice(None)]
    for a in range(ndim - 1, -1, -1):
        if a == axis:
            sl.append(idx + 1)
        else:
            sl.append(slice(2, cells.shape[1 + (ndim - 1 - a)] - 2))
    return cells[tuple(sl)]


@pytest.mark.parametrize("ndim,dims", [(1, [16]), (2, [16, 8]), (3, [16, 8, 4])])
@pytest.mark.parametrize("bctype", [1, 2, 3])
def test_set_boundaries(ndim, dims, bctype):
    """rhyme_samr_bc_set_{left,right,...}_boundary_test.f90: exact copies,
    negated normal momentum for reflective, wrap for periodic; corners kept."""
    cells = _random_box(ndim, dims)
    before = cells.copy()
    oracle.set_boundaries(_params(ndim, [bctype] * 6), cells)
    for axis in range(ndim):
        N = dims[axis]
        for ghost, src_refl, src_per in ((0, 1, N), (-1, 2, N - 1), (N + 1, N, 1), (N + 2, N - 1, 2)):
            g = _face(cells, ndim, axis, ghost)
            src = _face(cells, ndim, axis, src_per if bctype == 3 else src_refl)
            exp = src.copy()
            if bctype == 1:
                exp[1 + axis] = -exp[1 + axis]
            assert to_be(g, exp) or np.array_equal(g, exp)
    # corners (ghost in two axes) untouched
    if ndim >= 2:
        assert np.array_equal(cells[:, 0, 0], before[:, 0, 0])
        assert np.array_equal(cells[:, 1, 1], before[:, 1, 1])


@pytest.mark.parametrize("ndim,dims", [(1, [16]), (2, [16, 8]), (3, [16, 8, 4])])
def test_set_inflow_boundaries(ndim, dims):
    """rhyme_samr_bc_set_{left,...,front}_boundary_test.f90 (inflow): both
    ghost layers of an inflow face hold the face's cons_inflows (rho 1.23,
    every momentum 2.34, e_tot 3.45); here each face gets its own values
    (offset by the face index) so that a face written from another face's
    values would show."""
    cells = _random_box(ndim, dims)
    before = cells.copy()
    inflow = [[1.23 + f, *([2.34 + f] * ndim), 3.45 + f] for f in range(6)]
    oracle.set_boundaries(dict(_params(ndim, [4] * 6), inflow=inflow), cells)
    for axis in range(ndim):
        N = dims[axis]
        for side, ghosts in ((0, (0, -1)), (1, (N + 1, N + 2))):
            face = 2 * axis + side
            for ghost in ghosts:
                g = _face(cells, ndim, axis, ghost)
                for c in range(ndim + 2):
                    assert np.all(g[c] == inflow[face][c]), (axis, side, ghost, c)
    interior = (slice(None),) + tuple(slice(2, d + 2) for d in dims[::-1])
    assert np.array_equal(cells[interior], before[interior])
    if ndim >= 2:
        assert np.array_equal(cells[:, 0, 0], before[:, 0, 0])


def _fill_1d_reference_order(c, n, bctype):
    """The statements of rhyme_samr_bc_set_left_boundary.f90 then
    _set_right_boundary.f90 (rhyme_samr_bc_set_boundaries.f90:9-10) for a
    1-D box, on c[comp, i + 1] = cells(i, comp), i = -1 .. n + 2, in the
    reference's order: left copies, left momentum sign, right copies, right
    momentum sign."""
    at = lambda i: i + 1  # noqa: E731
    if bctype == 3:
        c[:, at(0)] = c[:, at(n)]
        c[:, at(-1)] = c[:, at(n - 1)]
    else:
        c[:, at(0)] = c[:, at(1)]
        c[:, at(-1)] = c[:, at(2)]
        if bctype == 1:
            c[1, at(0)] = -c[1, at(1)]
            c[1, at(-1)] = -c[1, at(2)]
    if bctype == 3:
        c[:, at(n + 1)] = c[:, at(1)]
        c[:, at(n + 2)] = c[:, at(2)]
    else:
        c[:, at(n + 1)] = c[:, at(n)]
        c[:, at(n + 2)] = c[:, at(n - 1)]
        if bctype == 1:
            c[1, at(n + 1)] = -c[1, at(n)]
            c[1, at(n + 2)] = -c[1, at(n - 1)]
    return c


@pytest.mark.parametrize("n", [1, 2, 3])
@pytest.mark.parametrize("bctype", [1, 2, 3])
def test_ghost_fill_order_on_short_boxes(n, bctype):
    """With fewer than 4 interior cells a face's ghost layers read cells
    that the other face writes (for n = 1 the left face's outer ghost reads
    the right face's inner ghost before that face is filled), so the result
    depends on the reference's statement order, which the oracle keeps."""
    rng = np.random.default_rng(n * 10 + bctype)
    cells = rng.uniform(0.5, 2.0, (3, n + 4))   # ghosts hold distinct old values
    want = _fill_1d_reference_order(cells.copy(), n, bctype)
    oracle.set_boundaries(_params(1, [bctype] * 6), cells)
    assert np.array_equal(cells, want)


@pytest.mark.parametrize("ndim,dims", [(1, [32]), (2, [16, 8]), (3, [8, 8, 4])])
def test_cfl_time_step(ndim, dims):
    """rhyme_cfl_dt_test.f90:58-73: dt = c*min(dx)/max(|v|+cs)."""
    cells = _random_box(ndim, dims)
    dx = [1.0 / d for d in dims]
    p = _params(ndim, [2] * 6)
    dt = oracle.cfl_time_step(p, cells, dx)
    interior = (slice(None),) + tuple(slice(2, d + 2) for d in dims[::-1])
    u = cells[interior].reshape(ndim + 2, -1).T
    _, _, cs = oracle.eos(ndim, p["gamma"], KB_AMU_SI, u, 0)
    s = np.zeros(u.shape[0])
    for a in range(ndim):
        s = s + u[:, 1 + a] * u[:, 1 + a]
    v = np.sqrt(s) / u[:, 0] + cs
    exp = 0.8 * min(dx) / v.max()
    assert to_be(dt, exp)


def test_uniform_state_is_steady():
    cells = np.zeros((5, 12, 12, 12))
    cells[0] = 1.0
    cells[1] = 0.3
    cells[4] = 3.0
    interior = (slice(None), slice(2, 10), slice(2, 10), slice(2, 10))
    ref = cells[interior].copy()
    oracle.run(_params(3, [3] * 6), cells, [1 / 8] * 3, 5)
    assert np.allclose(cells[interior], ref, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("limiter", [1, 2, 3, 4])
def test_periodic_conservation(limiter):
    p = _params(2, [3] * 4 + [2, 2], limiter=limiter)
    cells, dx, _ = ic.slab_2d(n=32, seed=3)
    interior = (slice(None), slice(2, 34), slice(2, 34))
    tot0 = cells[interior].sum(axis=(1, 2))
    oracle.run(p, cells, dx, 20)
    tot1 = cells[interior].sum(axis=(1, 2))
    assert np.allclose(tot1, tot0, rtol=1e-13, atol=1e-13)


def test_solver_orderings_agree():
    """memory_intensive vs cpu_intensive differ only in rounding order."""
    a, dx, _ = ic.slab_2d(n=32, seed=5)
    b = a.copy()
    oracle.run(_params(2, [3] * 4 + [2, 2], solver_type=2), a, dx, 10)
    oracle.run(_params(2, [3] * 4 + [2, 2], solver_type=1), b, dx, 10)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-13)


def test_1d_embedded_in_3d():
    """A state varying along x only evolves identically in 1-D and 3-D."""
    c1, dx, p1 = ic.riemann_1d(n=64, seed=7)
    p1 = dict(p1)
    c3 = np.zeros((5, 8, 8, 68))
    c3[0] = c1[0]
    c3[1] = c1[1]
    c3[4] = c1[2]
    c3[:, :2] = 0.0
    c3[:, -2:] = 0.0
    c3[:, :, :2] = 0.0
    c3[:, :, -2:] = 0.0
    p3 = dict(p1)
    p3["ndim"] = 3
    p3["bc"] = [2, 2, 3, 3, 3, 3]
    oracle.run(p1, c1, [1 / 64], 20)
    oracle.run(p3, c3, [1 / 64] * 3, 20)
    for k in range(2, 6):
        for j in range(2, 6):
            assert np.allclose(c3[0, k, j, 2:-2], c1[0, 2:-2], rtol=1e-13, atol=1e-14)
            assert np.allclose(c3[4, k, j, 2:-2], c1[2, 2:-2], rtol=1e-13, atol=1e-14)


def test_sod_against_analytic(golden_dir):
    """1-D Sod (gamma=1.4) evolved to t~0.2 matches the analytic density
    profile to first-order accuracy near discontinuities (L1 < 1e-2)."""
    import os
    n = 500
    g = GAMMA["diatomic"]
    cells = np.zeros((3, n + 4))
    x = -0.5 + (np.arange(n) + 0.5) / n
    rho = np.where(x < 0, 1.0, 0.125)
    pr = np.where(x < 0, 1.0, 0.1)
    cells[0, 2:-2] = rho
    cells[2, 2:-2] = pr / (g - 1.0)
    p = _params(1, [2] * 6, limiter=1, gamma=g)
    p["tol"], p["n_iter"] = 1e-8, 1000
    t = 0.0
    while t < 0.2:
        dt = oracle.run(p, cells, [1.0 / n], 1)[0]
        t += dt
    ref = np.loadtxt(os.path.join(golden_dir, "sod_t0.2_analytical.csv"), delimiter=",", comments="#")
    rho_ref = np.interp(x, ref[:, 0] * (t / 0.2), ref[:, 1])
    assert np.mean(np.abs(cells[0, 2:-2] - rho_ref)) < 1e-2


def _advection_box(ndim, grid, axis, g=GAMMA["diatomic"]):
    """rhyme_muscl_hancock_advection_factory.f90: square density waves
    (1.2 where mod(i, N/4) >= N/8 along the axis, 1.0 elsewhere) moving at
    v = 0.01 along the axis under p = 0.1, diatomic gas, periodic along the
    axis and outflow across it."""
    shp = tuple(grid[::-1])
    lam = grid[axis] // 4
    i = np.indices(shp)[ndim - 1 - axis] + 1
    rho = np.where(i % lam >= lam // 2, 1.2, 1.0)
    vel = [np.zeros(shp) for _ in range(ndim)]
    vel[axis] = np.full(shp, 0.01)
    cells = ic.empty_box(ndim, grid)
    cells[ic.interior(ndim, grid)] = ic.prim_to_cons(rho, vel, np.full(shp, 0.1), g)
    bc = [2] * 6
    bc[2 * axis] = bc[2 * axis + 1] = 3
    return cells, bc[:2 * ndim]


@pytest.mark.parametrize("solver", [1, 2])
@pytest.mark.parametrize("limiter", [1, 2, 3, 4])
@pytest.mark.parametrize("ndim,grid", [(1, [128]), (2, [32, 32]), (3, [16, 16, 16])])
def test_contact_advection(ndim, grid, limiter, solver):
    """The reference's advection set-up, which its solve tests step without
    expectations (and at dt = dx / v, a Courant number near 38), here at a
    stable Courant number for 20 steps. A pure contact: with equal pressure
    and velocity on both sides the exact solver returns that pressure and
    velocity, so velocity and pressure stay uniform to rounding, the
    transverse velocities stay exactly zero, mass is conserved and the
    density keeps within its initial range."""
    g = GAMMA["diatomic"]
    for axis in range(ndim):
        cells, bc = _advection_box(ndim, grid, axis)
        p = dict(_params(ndim, bc, limiter=limiter, solver_type=solver, gamma=g),
                 courant=0.8 if ndim == 1 else 0.4)
        inner = ic.interior(ndim, grid)
        m0 = cells[inner][0].sum()
        oracle.run(p, cells, [1.0 / n for n in grid], 20, nthreads=1)
        u = cells[inner]
        rho = u[0]
        v = u[1:1 + ndim] / rho
        pr = (g - 1.0) * (u[ndim + 1] - 0.5 * rho * (v * v).sum(0))
        assert np.max(np.abs(v[axis] - 0.01)) <= 1e-13 * 0.01
        assert all(np.all(v[a] == 0.0) for a in range(ndim) if a != axis)
        assert np.max(np.abs(pr - 0.1)) <= 1e-14 * 0.1
        assert abs(rho.sum() - m0) <= 1e-14 * m0
        assert rho.min() >= 1.0 - 1e-14 and rho.max() <= 1.2 + 1e-14
        assert rho.max() - rho.min() > 0.1   # the waves are still there
