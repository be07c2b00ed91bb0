"""Symmetries of the CPU oracle's algorithm (CPU only): properties that hold
for any input, checked on seeded random states, beside the reference's
golden vectors.

* The exact Riemann solver (rhyme_riemann_problem_solve.f90 with the
  rhyme_irs_* iteration), for two non-vacuum sides, is mirror-symmetric and
  Galilean-invariant, vacuum generation included. Its vacuum-left and
  vacuum-right branches (rhyme_riemann_problem_solve.f90:28-65) are not
  mirror images of each other: they take the side's wave speeds with the
  signs opposite to those of Toro, section 4.6, so a fan against vacuum is
  never sampled.
  The oracle keeps that behaviour; it is checked here in closed form.
* The limited slope (rhyme_slope_limiter.f90:62-82 and the four limiter
  files) commutes with scaling by a power of two and with negation, bit for
  bit. Only van Leer's ξ(r) = min(2r/(1+r), ξR(r)) is unchanged under
  r -> 1/r; minmod, van Albada and superbee as the reference writes them
  (Toro's ξ(r) applied to the average slope 0.5(Δ_L + Δ_R)) are not
  mirror-symmetric.
* Hence a whole MUSCL-Hancock step with van Leer, on a box reflected along
  an axis, is the reflection of the step on the box; with any limiter, a box
  whose axes are permuted (equal cell sizes) steps to the permuted box. The
  memory-intensive order sums the per-axis flux differences before the
  update (rhyme_muscl_hancock_solve_memory_intensive.f90), so in 2-D that
  permutation is exact.
"""
import numpy as np
import pytest

import oracle
from rhyme_gb300 import ic
from rhyme_gb300.params import (CPU_INTENSIVE, MEMORY_INTENSIVE, MINMOD, OUTFLOW, PERIODIC,
                                REFLECTIVE, SUPERBEE, VAN_ALBADA, VAN_LEER, hydro_params)


def random_sides(ndim, n, seed, g):
    """n left and n right conserved states: ρ and p log-uniform over three
    decades, every velocity component uniform in [-3, 3] (about 3% of the
    pairs generate vacuum)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(2):
        rho = 10 ** rng.uniform(-2, 1, n)
        v = rng.uniform(-3, 3, (n, ndim))
        p = 10 ** rng.uniform(-2, 1, n)
        u = np.zeros((n, ndim + 2))
        u[:, 0] = rho
        u[:, 1:1 + ndim] = rho[:, None] * v
        u[:, ndim + 1] = 0.5 * rho * np.sum(v * v, axis=1) + p / (g - 1.0)
        out.append(u)
    return out


def row_err(a, b):
    """Largest difference per row, relative to the row's largest magnitude."""
    scale = np.maximum(np.max(np.abs(a), axis=1), np.finfo(np.float64).tiny)
    return np.max(np.abs(a - b), axis=1) / scale


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_riemann_mirror_symmetry(ndim):
    p = hydro_params(ndim, tol=1e-10, n_iter=1000)
    for axis in range(ndim):
        l, r = random_sides(ndim, 2000, 7 + axis, p["gamma"])

        def mirror(u):
            m = u.copy()
            m[:, 1 + axis] = -m[:, 1 + axis]
            return m

        for x in (0.0, 0.37, -0.21):
            u = oracle.riemann_solve(p, l, r, x, 1.0, axis)
            um = mirror(oracle.riemann_solve(p, mirror(r), mirror(l), -x, 1.0, axis))
            assert np.any(u[:, 0] == 0.0)      # vacuum generation sampled
            assert np.max(row_err(u, um)) <= 1e-13, (axis, x)


def _side_speeds(u, ndim, axis, g):
    rho = u[:, 0]
    v = u[:, 1:1 + ndim] / rho[:, None]
    p = (g - 1.0) * (u[:, ndim + 1] - 0.5 * rho * np.sum(v * v, axis=1))
    return v[:, axis], np.sqrt(g * p / rho)


@pytest.mark.parametrize("ndim", [1, 3])
def test_riemann_vacuum_side_branches(ndim):
    """Vacuum on one side (ρ = 0 below the vacuum density's successor).
    rhyme_riemann_problem_solve.f90:47-65 (vacuum left): the right state
    where x/t > v_R + c_R, else W_0 (its fan test, x/t > v_R + 2c_R/(γ-1),
    lies inside the first one). :28-46 (vacuum right): W_0 where
    x/t > v_L - 2c_L/(γ-1), else the left state (its fan test,
    x/t > v_L - c_L, lies inside the first one). Thresholds within 1e-9 of
    x/t are skipped."""
    p = hydro_params(ndim, tol=1e-10, n_iter=1000)
    g = p["gamma"]
    for axis in range(ndim):
        side, _ = random_sides(ndim, 2000, 21 + axis, g)
        vac = np.zeros_like(side)
        v, c = _side_speeds(side, ndim, axis, g)
        for x in (-1.0, 0.0, 0.6):
            got_l = oracle.riemann_solve(p, vac, side, x, 1.0, axis)
            got_r = oracle.riemann_solve(p, side, vac, x, 1.0, axis)
            for got, edge in ((got_l, v + c), (got_r, v - 2.0 * c / (g - 1.0))):
                keep = np.abs(edge - x) > 1e-9
                state = (x > edge) if got is got_l else (x <= edge)
                a = got[keep & state]
                assert np.max(row_err(side[keep & state], a)) <= 1e-14
                assert np.all(got[keep & ~state] == 0.0)
            # the two branches are not mirror images: the side state shows
            # on the vacuum-left side for v_R + c_R < x/t <= v_R + 2c_R/(γ-1)
            if x == 0.0:
                mirror_r = side.copy()
                mirror_r[:, 1 + axis] = -mirror_r[:, 1 + axis]
                got_m = oracle.riemann_solve(p, mirror_r, vac, -x, 1.0, axis)
                differ = (got_l[:, 0] > 0.0) != (got_m[:, 0] > 0.0)
                assert np.any(differ)


def _prim(u, ndim, g):
    rho = u[:, 0]
    v = u[:, 1:1 + ndim] / np.where(rho > 0.0, rho, 1.0)[:, None]
    p = (g - 1.0) * (u[:, ndim + 1] - 0.5 * rho * np.sum(v * v, axis=1))
    return np.column_stack([rho, v, p])


@pytest.mark.parametrize("ndim", [1, 3])
def test_riemann_galilean_invariance(ndim):
    """Both sides moved by w along the axis, sampled at x/t + w: the same
    density and pressure, the velocity moved by w. The vacuum state is at
    rest in the box frame (rhyme_riemann_problem_solve.f90 returns
    w_vacuum), so vacuum rows are only checked to stay vacuum."""
    p = hydro_params(ndim, tol=1e-12, n_iter=1000)
    g = p["gamma"]
    for axis in range(ndim):
        l, r = random_sides(ndim, 2000, 11 + axis, g)
        for w in (0.75, -1.5):
            def boost(u):
                m = u.copy()
                m[:, ndim + 1] += u[:, 1 + axis] * w + 0.5 * u[:, 0] * w * w
                m[:, 1 + axis] += u[:, 0] * w
                return m

            for x in (0.0, 0.4):
                a = _prim(oracle.riemann_solve(p, l, r, x, 1.0, axis), ndim, g)
                b = _prim(oracle.riemann_solve(p, boost(l), boost(r), x + w, 1.0, axis), ndim, g)
                vac = a[:, 0] == 0.0
                assert vac.any() and np.array_equal(vac, b[:, 0] == 0.0)
                b[:, 1 + axis] -= w
                scale = np.maximum(np.max(np.abs(a), axis=1), 1.0)
                err = np.max(np.abs(a - b), axis=1) / scale
                assert np.max(err[~vac]) <= 1e-11, (axis, w, x)


def _limiter_rows(n, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-2.0, 2.0, (n, 5))
    ul = u + rng.uniform(-1.0, 1.0, (n, 5))
    ur = u + rng.uniform(-1.0, 1.0, (n, 5))
    return ul, u, ur


@pytest.mark.parametrize("limiter", [VAN_LEER, MINMOD, VAN_ALBADA, SUPERBEE])
@pytest.mark.parametrize("omega", [0.0, 0.5, -0.3])
def test_limiter_scale_and_sign(limiter, omega):
    ul, u, ur = _limiter_rows(4000, limiter)
    d = oracle.slope_limiter(3, limiter, omega, ul, u, ur)
    assert np.any(d != 0.0) and np.any(d == 0.0)
    for c in (0.25, 2.0, 1024.0):
        assert np.array_equal(oracle.slope_limiter(3, limiter, omega, c * ul, c * u, c * ur), c * d)
    assert np.array_equal(oracle.slope_limiter(3, limiter, omega, -ul, -u, -ur), -d)


def test_limiter_mirror():
    """Data read backwards: Δ_L' = -Δ_R, Δ_R' = -Δ_L, so r' = 1/r."""
    ul, u, ur = _limiter_rows(4000, 5)
    d = oracle.slope_limiter(3, VAN_LEER, 0.0, ul, u, ur)
    dm = oracle.slope_limiter(3, VAN_LEER, 0.0, ur, u, ul)
    scale = np.maximum(np.abs(ur - ul), 1.0)
    assert np.max(np.abs(d + dm) / scale) <= 1e-15
    # minmod with Δ_L = 1, Δ_R = 2: r = 1/2 gives r Δ_avg = 0.75; backwards,
    # r = 2 gives min(1, ξR(2)) Δ_avg = (2/3)(-1.5) = -1
    one = np.ones((1, 5))
    assert to_list(oracle.slope_limiter(3, MINMOD, 0.0, 0 * one, one, 3 * one)) == [0.75] * 5
    assert to_list(oracle.slope_limiter(3, MINMOD, 0.0, 3 * one, one, 0 * one)) == [-1.0] * 5


def to_list(a):
    return [float(x) for x in a.ravel()]


def rand_box(ndim, dims, seed, g=5.0 / 3.0):
    rng = np.random.default_rng(seed)
    shp = tuple(dims[::-1])
    rho = 1.0 + 0.5 * rng.random(shp)
    vel = [0.3 * (rng.random(shp) - 0.5) for _ in range(ndim)]
    pr = 1.0 + 0.5 * rng.random(shp)
    cells = ic.empty_box(ndim, dims)
    cells[ic.interior(ndim, dims)] = ic.prim_to_cons(rho, vel, pr, g)
    return cells


def reflect(cells, ndim, axis):
    """The box read backwards along axis (numpy axis ndim - axis), its
    momentum along axis negated."""
    idx = [slice(None)] * (ndim + 1)
    idx[ndim - axis] = slice(None, None, -1)
    c = cells[tuple(idx)].copy()
    c[1 + axis] = -c[1 + axis]
    return c


def permute(cells, ndim, perm):
    """New axis a is old axis perm[a]; momentum components follow."""
    np_axes = [0] + [ndim - perm[ndim - 1 - k] for k in range(ndim)]
    t = np.transpose(cells, np_axes)
    return np.ascontiguousarray(np.stack([t[0]] + [t[1 + perm[a]] for a in range(ndim)] + [t[ndim + 1]]))


def field_err(a, b, ndim, dims):
    inner = ic.interior(ndim, dims)
    axes = tuple(range(1, ndim + 1))
    scale = np.max(np.abs(a[inner]), axis=axes, keepdims=True)
    return float(np.max(np.abs(a[inner] - b[inner]) / scale))


BC = [OUTFLOW, REFLECTIVE, PERIODIC, PERIODIC, REFLECTIVE, OUTFLOW]


@pytest.mark.parametrize("ndim,dims", [(1, [24]), (2, [16, 12]), (3, [10, 8, 12])])
@pytest.mark.parametrize("solver", [MEMORY_INTENSIVE, CPU_INTENSIVE])
def test_box_reflection_van_leer(ndim, dims, solver):
    p = hydro_params(ndim, limiter=VAN_LEER, bc=BC[:2 * ndim], courant=0.5, solver_type=solver)
    dx = [1.0 / max(dims)] * ndim
    c0 = rand_box(ndim, dims, 3)
    a = c0.copy()
    da = np.array(oracle.run(p, a, dx, 6, nthreads=1))
    for axis in range(ndim):
        bc = list(p["bc"])
        bc[2 * axis], bc[2 * axis + 1] = bc[2 * axis + 1], bc[2 * axis]
        b = reflect(c0, ndim, axis)
        db = np.array(oracle.run(dict(p, bc=bc), b, dx, 6, nthreads=1))
        assert np.max(np.abs(da - db) / da) <= 1e-14
        assert field_err(a, reflect(b, ndim, axis), ndim, dims) <= 1e-12, axis


@pytest.mark.parametrize("limiter", [VAN_LEER, MINMOD, VAN_ALBADA, SUPERBEE])
@pytest.mark.parametrize("ndim,dims,perm", [(2, [14, 10], [1, 0]), (3, [8, 10, 6], [1, 2, 0]),
                                            (3, [8, 10, 6], [2, 0, 1])])
def test_box_axis_permutation(limiter, ndim, dims, perm):
    p = hydro_params(ndim, limiter=limiter, bc=BC[:2 * ndim], courant=0.5)
    bc = []
    for a in range(ndim):
        bc += [p["bc"][2 * perm[a]], p["bc"][2 * perm[a] + 1]]
    dx = [1.0 / 16.0] * ndim
    c0 = rand_box(ndim, dims, 5)
    a = c0.copy()
    da = np.array(oracle.run(p, a, dx, 6, nthreads=1))
    b = permute(c0, ndim, perm)
    db = np.array(oracle.run(dict(p, bc=bc), b, dx, 6, nthreads=1))
    pa = permute(a, ndim, perm)
    dims_b = [dims[perm[k]] for k in range(ndim)]
    if ndim == 2:
        inner = ic.interior(ndim, dims_b)
        assert np.array_equal(da, db) and np.array_equal(pa[inner], b[inner])
    else:
        assert np.max(np.abs(da - db) / da) <= 1e-14
        assert field_err(pa, b, ndim, dims_b) <= 1e-13
