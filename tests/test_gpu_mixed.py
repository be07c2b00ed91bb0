"""Mixed-precision path (FP32 reconstruction / Riemann / flux, FP64 state
accumulation, FP64 Riemann fallback) against the plain FP64 GPU path.

Tolerance: relative L1 of the density <= 1e-6 after the stated steps (the
bar the mixed form is quoted at); total energy <= 1e-5; momentum components
(which can be near zero everywhere) <= 1e-5 of the density's L1 norm times
the box's maximum signal speed; dt within 1e-5 (an FP32 maximum over a
state that differs from the FP64 one by the accumulated mixed rounding).
These workloads do not amplify rounding differences (the 2-D shear slab
does, and is quoted in FP64 only).
"""
import numpy as np
import pytest

from parity import field_errors

from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import FP64, MINMOD, MIXED, OUTFLOW, PERIODIC, VAN_LEER, hydro_params

pytestmark = pytest.mark.gpu

MIXED_L1_RHO = 1e-6
MIXED_L1_OTHER = 1e-5
MIXED_DT = 1e-5


def run(p, cells, dx, nsteps, precision):
    c = cells.copy()
    with gpu.Context(dict(p, precision=precision)) as ctx:
        box = ctx.register_box(c)
        dts = ctx.run(box, dx, nsteps)
        fb = ctx.fallback_count(box)
        ctx.sync_to_host(box)
    return c, dts, fb


def check(p, cells, dx, nsteps, rho_tol=MIXED_L1_RHO, other_tol=MIXED_L1_OTHER):
    a, da, _ = run(p, cells, dx, nsteps, FP64)
    b, db, fb = run(p, cells, dx, nsteps, MIXED)
    assert np.isfinite(b).all()
    nd = p["ndim"]
    errs = field_errors(b, a, nd)
    assert errs[0][0] <= rho_tol, errs
    assert errs[nd + 1][0] <= other_tol, errs
    inner = (slice(None),) + (slice(2, -2),) * nd
    ai, bi = a[inner], b[inner]
    rho_norm = np.abs(ai[0]).sum()
    vmax = max(np.abs(ai[1 + k] / ai[0]).max() for k in range(nd)) + np.sqrt(p["gamma"] * 10.0)
    for k in range(nd):
        assert np.abs(bi[1 + k] - ai[1 + k]).sum() <= other_tol * rho_norm * vmax, errs
    assert np.max(np.abs(db - da) / da) <= MIXED_DT
    return errs, fb


def test_mixed_riemann_1d():
    for seed in (0, 1):
        cells, dx, p = ic.riemann_1d(n=512, seed=seed)
        errs, _ = check(p, cells, dx, 100)
        print("1-D riemann seed", seed, errs)


def test_mixed_acoustic_pulse_2d():
    """A smooth 2-D pressure pulse (no shear layer), periodic, van Leer.

    A smooth, small-amplitude flow is the hard case for FP32 fluxes: the
    flux difference of a cell is small against the fluxes themselves, so
    their FP32 rounding sets the error (relative L1 of the density 6.5e-7
    with the FP32 flux formed from the sampled primitive state; 1.1e-6
    when it was formed from the conserved state, whose E - |m|^2/(2 rho)
    cancels), against 8e-8 on the 256^3 sphere configuration."""
    n = 96
    g = 5.0 / 3.0
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    r2 = (X - 0.5) ** 2 + (Y - 0.5) ** 2
    rho = 1.0 + 0.2 * np.exp(-r2 / 0.01)
    pr = 1.0 + 0.5 * np.exp(-r2 / 0.01)
    cells = ic.empty_box(2, [n, n])
    cells[:, 2:-2, 2:-2] = ic.prim_to_cons(rho, [np.zeros_like(rho)] * 2, pr, g)
    p = hydro_params(2, limiter=VAN_LEER, bc=[PERIODIC] * 4, courant=0.5)
    errs, _ = check(p, cells, [1.0 / n] * 2, 150)
    print("2-D pulse", errs)


def test_mixed_spheres_3d():
    cells, dx, p = ic.spheres_3d(n=64, nspheres=32, seed=0)
    errs, _ = check(p, cells, dx, 100)
    print("3-D spheres 64^3", errs)


def test_mixed_fallback_near_vacuum():
    """Two receding states beyond the vacuum-generation limit (du = 1.22
    du_crit) open a near-vacuum gap: those interfaces go to the FP64 solver
    and the result stays finite and close to FP64. The reference scheme
    itself keeps this case positive only at small Courant numbers (at 0.5,
    or with u = -+3 and p = 0.05, the plain FP64 run, like the CPU oracle,
    reaches negative densities within a few tens of steps), so the FP64 run
    is checked first."""
    n = 256
    g = 5.0 / 3.0
    cells = ic.empty_box(1, [n])
    x = np.arange(n)
    rho = np.ones(n)
    u = np.where(x < n // 2, -3.0, 3.0)
    pr = np.full(n, 0.4)
    cells[:, 2:-2] = ic.prim_to_cons(rho, [u], pr, g)
    p = hydro_params(1, limiter=MINMOD, bc=[OUTFLOW] * 2, vac_rho=1e-8, vac_p=1e-10, courant=0.3)
    a, da, _ = run(p, cells, [1.0 / n], 40, FP64)
    assert np.isfinite(a).all() and a[0, 2:-2].min() > 0
    b, db, fb = run(p, cells, [1.0 / n], 40, MIXED)
    assert fb > 0
    assert np.isfinite(b).all()
    errs = field_errors(b, a, 1)
    assert errs[0][0] <= 1e-4, errs
    print("near-vacuum 1-D: FP64 interfaces", fb, "errors", errs)


def test_mixed_stepwise_api_matches_run():
    cells, dx, p = ic.spheres_3d(n=32, nspheres=4, seed=2)
    q = dict(p, precision=MIXED)
    a = cells.copy()
    b = cells.copy()
    with gpu.Context(q) as ctx:
        box = ctx.register_box(a)
        ctx.run(box, dx, 5)
        ctx.sync_to_host(box)
    with gpu.Context(q) as ctx:
        box = ctx.register_box(b)
        for _ in range(5):
            dt = ctx.cfl_time_step(box, dx)
            ctx.set_boundaries(box)
            ctx.muscl_hancock_solve(box, dx, dt)
        ctx.sync_to_host(box)
    errs = field_errors(b, a, 3)
    assert max(e[0] for e in errs) <= 1e-12, errs
