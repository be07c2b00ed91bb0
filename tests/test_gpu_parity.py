"""GPU parity of the plain FP64 path against the CPU oracle and the
reference's golden vectors, all through the C-ABI (librhyme_gpu.so).

The oracle runs with the C library's pow, as the compiled reference calls it
for every real `**`, and the CUDA kernels with its restatement
(libm_pow.h), so every box run is compared bit for bit: the whole array,
ghosts included, and every dt. That also covers the stated bar (<= 1e-12
relative L1/Linf per field, dt <= 1e-14), which is asserted beside it, and
the shear-layer workload, where a single flipped bit in one cell would grow
to ~1e-10 relative in 500 steps."""
import json
import os

import numpy as np
import pytest

import oracle
from parity import assert_fp64_parity, field_errors
from refcheck import GAMMA, KB_AMU_SI, within

from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import hydro_params

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


def ctx_for(p):
    return gpu.Context(p)


# ---------------------------------------------------------------- elements --
def test_irs_exec_p_stars(golden_dir):
    """rhyme_irs_exec_test.f90:36-57 on the GPU: 1000 golden p* to 6 s.f."""
    rows = np.loadtxt(os.path.join(golden_dir, "p_stars_1000.csv"), delimiter=",", comments="#")
    g1 = float(np.float32(5.0) / np.float32(3.0))
    l_rho, l_v, l_p, r_rho, r_v, r_p, exp = rows.T
    states = np.stack([l_rho, l_v, l_p, np.sqrt(g1 * l_p / l_rho), r_rho, r_v, r_p,
                       np.sqrt(g1 * r_p / r_rho)], axis=1)
    p = hydro_params(1, gamma=GAMMA["monatomic"], tol=1e-10, n_iter=100000)
    with ctx_for(p) as ctx:
        out = ctx.irs_exec(states)
    ref = oracle.irs_exec(GAMMA["monatomic"], 1e-10, 100000, states)
    bad = [i for i in range(1000) if not within(out[i, 0], exp[i], 6)]
    assert not bad, bad[:10]
    assert np.array_equal(out, ref)


def _toro(golden_dir):
    with open(os.path.join(golden_dir, "toro_star_cases.json")) as f:
        return json.load(f)["cases"]


def _cons(case, side, g):
    s = case[side]
    return np.array([s["rho"], s["rho"] * s["u"], 0.5 * s["rho"] * (s["u"] * s["u"]) + s["p"] / (g - 1.0)])


def test_riemann_sampling_sod(golden_dir):
    """rhyme_riemann_problem_sampling_test.f90:37-66 through the GPU
    rhyme_riemann_problem_solve: Sod at t = 0.2, 500 samples of x/t."""
    g = GAMMA["diatomic"]
    case = [c for c in _toro(golden_dir) if c["name"] == "Sod"][0]
    p = hydro_params(1, gamma=g, tol=1e-8, n_iter=1000, kb_amu=KB_AMU_SI)
    ref = np.loadtxt(os.path.join(golden_dir, "sod_t0.2_analytical.csv"), delimiter=",", comments="#")
    xs = -0.5 + np.arange(500, dtype=np.float64) / 499.0
    L = np.repeat(_cons(case, "left", g)[None], 500, 0)
    R = np.repeat(_cons(case, "right", g)[None], 500, 0)
    with ctx_for(p) as ctx:
        u = np.stack([ctx.riemann_problem_solve(L[i:i + 1], R[i:i + 1], xs[i], 0.2, 0)[0]
                      for i in range(500)])
    pr = dict(p)
    uo = np.stack([oracle.riemann_solve(pr, L[i:i + 1], R[i:i + 1], xs[i], 0.2, 0)[0] for i in range(500)])
    np.testing.assert_allclose(u, uo, rtol=1e-14, atol=1e-15)
    _, pres, _ = oracle.eos(1, g, KB_AMU_SI, u, 0)
    for i in range(500):
        x, rho, v, pe = ref[i]
        assert within(rho, u[i, 0], 15), ("rho", i)
        assert within(rho * v, u[i, 1], 14), ("rho_u", i)
        assert within(pe, pres[i], 15), ("p", i)


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_riemann_solve_random_vs_oracle(ndim):
    """Random interface pairs on every axis, including strong shocks,
    rarefactions and vacuum generation, sampled at x/t = 0 and elsewhere."""
    rng = np.random.default_rng(11 + ndim)
    n = 20000
    g = GAMMA["monatomic"]
    rho = 10 ** rng.uniform(-2, 2, (2, n))
    vel = rng.uniform(-3, 3, (2, ndim, n))
    pr = 10 ** rng.uniform(-2, 2, (2, n))
    U = [ic.prim_to_cons(rho[s], list(vel[s]), pr[s], g).T.copy() for s in range(2)]
    p = hydro_params(ndim, gamma=g, tol=1e-6, n_iter=100)
    with ctx_for(p) as ctx:
        for axis in range(ndim):
            for dx, dt in ((0.0, 1.0), (0.3, 1.0), (-0.7, 2.0)):
                a = ctx.riemann_problem_solve(U[0], U[1], dx, dt, axis)
                b = oracle.riemann_solve(p, U[0], U[1], dx, dt, axis)
                assert np.array_equal(a, b)


@pytest.mark.parametrize("limiter", [1, 2, 3, 4])
def test_slope_limiter_and_half_step_bitwise(limiter):
    rng = np.random.default_rng(limiter)
    ndim, n = 3, 5000
    ul, u, ur = (rng.uniform(0.5, 2.0, (n, 5)) for _ in range(3))
    ur[::7] = u[::7]  # |ur - u| < tiny branch
    p = hydro_params(ndim, limiter=limiter, omega=0.25 if limiter == 1 else 0.0)
    with ctx_for(p) as ctx:
        d = ctx.slope_limiter_run(ul, u, ur)
        l, r = ctx.half_step_extrapolation(u, d, 1, 0.01, 0.003)
    do = oracle.slope_limiter(ndim, limiter, p["omega"], ul, u, ur)
    lo, ro = oracle.half_step(ndim, p["gamma"], u, do, 1, 0.01, 0.003)
    assert np.array_equal(d, do)
    assert np.array_equal(l, lo) and np.array_equal(r, ro)


# ------------------------------------------------------------------- boxes --
def _random_box(ndim, dims, seed, vac=False):
    """Smooth random fields (a few low modes) plus one density/pressure jump,
    so every limiter and Riemann branch is exercised without driving the
    scheme out of its positive regime."""
    rng = np.random.default_rng(seed)
    g = GAMMA["monatomic"]
    shp = tuple(dims[::-1])
    grids = np.meshgrid(*[(np.arange(n) + 0.5) / n for n in dims[::-1]], indexing="ij")
    def smooth(amp):
        f = np.zeros(shp)
        for _ in range(3):
            k = rng.integers(1, 3, ndim)
            ph = rng.uniform(0, 2 * np.pi)
            f = f + amp * np.sin(sum(2 * np.pi * k[a] * grids[a] for a in range(ndim)) + ph)
        return f
    jump = grids[-1] > rng.uniform(0.3, 0.7)
    rho = np.exp(smooth(0.15)) * np.where(jump, rng.uniform(0.2, 0.6), 1.0)
    pr = np.exp(smooth(0.15)) * np.where(jump, rng.uniform(0.2, 0.6), 1.0)
    vel = [smooth(0.1) for _ in range(ndim)]
    if vac:
        low = grids[0] < 0.25
        rho = np.where(low, 1e-5, rho)
        pr = np.where(low, 1e-7, pr)
    cells = ic.empty_box(ndim, dims)
    cells[ic.interior(ndim, dims)] = ic.prim_to_cons(rho, vel, pr, g)
    return cells


def oracle_run(p, cells, dx, nsteps, nthreads=NTHREADS):
    """(result, dts) of the oracle with the C library's pow."""
    b = cells.copy()
    db = oracle.run(p, b, dx, nsteps, nthreads=nthreads)
    return b, db


def assert_bitwise(got, dts, ref, dts_ref):
    assert np.array_equal(got, ref, equal_nan=True), "max |diff| %.3e" % np.nanmax(np.abs(got - ref))
    assert np.array_equal(np.asarray(dts), np.asarray(dts_ref))


def _gpu_steps(p, cells, dx, nsteps, use_run):
    c = cells.copy()
    with ctx_for(p) as ctx:
        box = ctx.register_box(c)
        if use_run:
            dts = ctx.run(box, dx, nsteps)
        else:
            dts = []
            for _ in range(nsteps):
                dt = ctx.cfl_time_step(box, dx)
                ctx.set_boundaries(box)
                ctx.muscl_hancock_solve(box, dx, dt)
                dts.append(dt)
        ctx.sync_to_host(box)
    return c, np.asarray(dts)


CASES = []
for nd, dims in ((1, [24]), (2, [12, 9]), (3, [7, 6, 5])):
    for lim in (1, 2, 3, 4):
        for bc in (1, 2, 3):
            CASES.append((nd, dims, lim, bc))


# Courant numbers inside the multi-D stability limit of the unsplit step.
COURANT = {1: 0.8, 2: 0.5, 3: 0.3}


@pytest.mark.parametrize("ndim,dims,limiter,bc", CASES)
def test_box_steps_vs_oracle(ndim, dims, limiter, bc):
    p = hydro_params(ndim, limiter=limiter, bc=[bc] * 6, courant=COURANT[ndim])
    cells = _random_box(ndim, dims, seed=ndim * 100 + limiter * 10 + bc)
    dx = [1.0 / dims[0]] * ndim
    ref, dts_ref = oracle_run(p, cells, dx, 12)
    got, dts = _gpu_steps(p, cells, dx, 12, use_run=(limiter % 2 == 0))
    # whole array, ghosts included: the ghost faces equal the reference
    # array's (filled from U^n) and the corners stay untouched
    assert_bitwise(got, dts, ref, dts_ref)
    assert_fp64_parity(got, ref, ndim, dts, dts_ref)


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_mixed_bcs_cpu_order_and_omega(ndim):
    dims = [10, 7, 6][:ndim]
    bc = [1, 2, 3, 3, 2, 1][:2 * ndim] + [2] * (6 - 2 * ndim)
    p = hydro_params(ndim, limiter=1, omega=0.3, bc=bc, solver_type=1, courant=COURANT[ndim])
    cells = _random_box(ndim, dims, seed=5)
    dx = [0.1, 0.07, 0.05][:ndim]
    ref, dts_ref = oracle_run(p, cells, dx, 10)
    got, dts = _gpu_steps(p, cells, dx, 10, use_run=True)
    assert_bitwise(got, dts, ref, dts_ref)
    assert_fp64_parity(got, ref, ndim, dts, dts_ref)


@pytest.mark.parametrize("n", [1, 2, 3])
@pytest.mark.parametrize("bc", [1, 2, 3])
def test_tiny_boxes(n, bc):
    """Edges of 1-3 cells, where ghost sources overlap ghosts of the other
    side and the fill order of rhyme_samr_bc_set_boundaries matters."""
    for ndim in (1, 2):
        dims = [n, n + 1][:ndim]
        p = hydro_params(ndim, limiter=2, bc=[bc] * 6, courant=COURANT[ndim])
        cells = _random_box(ndim, dims, seed=n * 7 + bc)
        ref, dts_ref = oracle_run(p, cells, [0.5] * ndim, 3)
        got, dts = _gpu_steps(p, cells, [0.5] * ndim, 3, use_run=False)
        assert_bitwise(got, dts, ref, dts_ref)
        assert_fp64_parity(got, ref, ndim, dts, dts_ref)


def test_vacuum_and_inflow():
    ndim, dims = 2, [16, 12]
    inflow = [[0.0] * 5 for _ in range(6)]
    inflow[0][:4] = [2.0, 0.5, 0.0, 4.0]
    p = hydro_params(ndim, limiter=3, bc=[4, 2, 1, 2, 2, 2], vac_rho=1e-6, vac_p=1e-8, inflow=inflow,
                     courant=0.5)
    cells = _random_box(ndim, dims, seed=9, vac=True)
    ref, dts_ref = oracle_run(p, cells, [0.1, 0.1], 8)
    got, dts = _gpu_steps(p, cells, [0.1, 0.1], 8, use_run=True)
    assert_bitwise(got, dts, ref, dts_ref)
    assert_fp64_parity(got, ref, ndim, dts, dts_ref)


def test_status_word_reports_bad_cells():
    """A cell with negative pressure (NaN sound speed) is skipped by the dt
    maximum as in the reference, and reported through the status word."""
    p = hydro_params(1, limiter=2, bc=[2] * 6)
    cells = _random_box(1, [16], seed=1)
    cells[2, 8] = -1.0  # negative total energy -> negative pressure
    ref = cells.copy()
    dt_ref = oracle.cfl_time_step(p, ref, [0.1])
    with ctx_for(p) as ctx:
        box = ctx.register_box(cells)
        assert ctx.box_status(box) == 0
        dt = ctx.cfl_time_step(box, [0.1])
        assert ctx.box_status(box) == 1
        assert ctx.box_status(box) == 0
    assert dt == dt_ref


def test_ghost_fill_and_cfl_direct():
    ndim, dims = 3, [9, 8, 7]
    p = hydro_params(ndim, bc=[1, 3, 2, 1, 3, 2])
    cells = _random_box(ndim, dims, seed=2)
    ref = cells.copy()
    dx = [0.1, 0.2, 0.05]
    with ctx_for(p) as ctx:
        box = ctx.register_box(cells)
        dt = ctx.cfl_time_step(box, dx)
        ctx.set_boundaries(box)
        ctx.sync_to_host(box)
    oracle.set_boundaries(p, ref)
    assert np.array_equal(cells, ref)
    assert dt == oracle.cfl_time_step(p, ref, dx)


def test_default_courant_3d_few_steps():
    """The reference default courant 0.8 in 3-D, for the steps before the
    unsplit scheme departs from its positive regime."""
    p = hydro_params(3, limiter=4, bc=[3] * 6)
    cells = _random_box(3, [8, 7, 6], seed=21)
    ref, dts_ref = oracle_run(p, cells, [0.1] * 3, 3)
    got, dts = _gpu_steps(p, cells, [0.1] * 3, 3, use_run=True)
    assert_bitwise(got, dts, ref, dts_ref)
    assert_fp64_parity(got, ref, 3, dts, dts_ref)


def test_run_equals_stepwise():
    p = hydro_params(2, limiter=2, bc=[3] * 4)
    cells, dx, _ = ic.slab_2d(n=32, seed=4)
    a, da = _gpu_steps(p, cells, dx, 7, use_run=True)
    b, db = _gpu_steps(p, cells, dx, 7, use_run=False)
    assert np.array_equal(a, b) and np.array_equal(da, db)


# --------------------------------------------------------- workload parity --
def test_riemann_1d_512_100_steps():
    """1-D 512 cells, seeded two-state Riemann problem, 100 steps."""
    for seed in (0, 1, 2):
        cells, dx, p = ic.riemann_1d(n=512, seed=seed)
        ref, dts_ref = oracle_run(p, cells, dx, 100)
        got, dts = _gpu_steps(p, cells, dx, 100, use_run=True)
        assert_bitwise(got, dts, ref, dts_ref)
        assert_fp64_parity(got, ref, 1, dts, dts_ref)


def test_slab_2d_256_500_steps():
    """2-D 256x256 periodic shear slab, minmod, 500 steps: bit-identical to
    the oracle with the C library's pow (the Kelvin-Helmholtz layer amplifies
    any one-ulp difference, so nothing weaker would meet 1e-12 here)."""
    cells, dx, p = ic.slab_2d(n=256, seed=0)
    ref, dts_ref = oracle_run(p, cells, dx, 500)
    got, dts = _gpu_steps(p, cells, dx, 500, use_run=True)
    assert_bitwise(got, dts, ref, dts_ref)
    assert_fp64_parity(got, ref, 2, dts, dts_ref)
