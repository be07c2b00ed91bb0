"""Seeded synthetic initial conditions for the benchmark workloads.

The reference's own IC painter (rhyme_drawing) cannot express the seeded
phases and velocity fields these workloads need, so they are generated here
with numpy. Each generator returns conserved hydro fields in the reference
layout (NDIM+2, [N3+4,] [N2+4,] N1+4) with zeroed ghosts, as
rhyme_samr_bc_init.f90:61-87 leaves them, plus dx and the run parameters.
"""
import numpy as np

from .params import (GAMMA, MINMOD, OUTFLOW, PERIODIC, REFLECTIVE, SUPERBEE,
                     VAN_ALBADA, VAN_LEER, hydro_params)


# Courant number of the 3-D workloads. The reference's unsplit step (no
# corner-transport terms) is stable only well below its default 0.8 in 3-D;
# 0.3 keeps the sphere and Riemann workloads positive for hundreds of steps.
COURANT_3D = 0.3


def empty_box(ndim, dims):
    shape = (ndim + 2,) + tuple(int(d) + 4 for d in list(dims)[::-1])
    return np.zeros(shape, dtype=np.float64)


def interior(ndim, dims):
    return (slice(None),) + tuple(slice(2, int(d) + 2) for d in list(dims)[::-1])


def prim_to_cons(rho, vel, p, gamma):
    """U = (rho, rho v, .5 rho |v|^2 + p/(gamma-1)) (ideal gas)."""
    ndim = len(vel)
    out = np.empty((ndim + 2,) + np.shape(rho))
    out[0] = rho
    s = np.zeros(np.shape(rho))
    for a in range(ndim):
        out[1 + a] = rho * vel[a]
        s = s + vel[a] * vel[a]
    out[ndim + 1] = 0.5 * rho * s + p / (gamma - 1.0)
    return out


def riemann_states(rng):
    """Two states: rho, p log-uniform in [0.1, 10], u uniform in [-1, 1]."""
    rho = 10.0 ** rng.uniform(-1.0, 1.0, 2)
    p = 10.0 ** rng.uniform(-1.0, 1.0, 2)
    u = rng.uniform(-1.0, 1.0, 2)
    return rho, u, p


def riemann_1d(n=512, seed=0):
    """1-D two-state Riemann problem, discontinuity between cells n/2 and
    n/2+1; outflow, van Leer (omega 0), courant 0.8, tol 1e-6, 100 iterations,
    gamma 5/3, box length 1."""
    rng = np.random.default_rng(seed)
    rho, u, p = riemann_states(rng)
    g = GAMMA["monatomic"]
    cells = empty_box(1, [n])
    side = np.arange(n) < n // 2
    R = np.where(side, rho[0], rho[1])
    U = np.where(side, u[0], u[1])
    P = np.where(side, p[0], p[1])
    cells[:, 2:n + 2] = prim_to_cons(R, [U], P, g)
    params = hydro_params(1, limiter=VAN_LEER, bc=[OUTFLOW] * 6, gamma=g)
    return cells, [1.0 / n], params


def slab_2d(n=256, seed=0):
    """2-D periodic shear slab: rho 1 | 2, u -0.5 | +0.5 with tanh ramps of
    width 2 cells at rows n/4 and 3n/4 (the smoothed-slab profile of
    rhyme_drawing_smoothed_slab_2d.f90:76-83), p = 2.5, and
    v = 0.01 cos(2 pi x / (n/4) + phase) with a seeded phase. Minmod,
    courant 0.8, gamma 5/3, box length 1 per axis."""
    rng = np.random.default_rng(seed)
    phase = rng.uniform(0.0, 2.0 * np.pi)
    g = GAMMA["monatomic"]
    y = (np.arange(n) + 0.5)[:, None] * np.ones((1, n))
    x = np.ones((n, 1)) * (np.arange(n) + 0.5)[None, :]
    yc, rs, sigma = n / 2.0, n / 4.0, 2.0 * n / 256.0
    ramp = 0.25 * (1.0 + np.tanh((rs - (y - yc)) / sigma)) * (1.0 + np.tanh((rs + (y - yc)) / sigma))
    rho = 1.0 + (2.0 - 1.0) * ramp
    u = -0.5 + (0.5 - (-0.5)) * ramp
    v = 0.01 * np.cos(2.0 * np.pi * x / (n / 4.0) + phase)
    p = np.full((n, n), 2.5)
    cells = empty_box(2, [n, n])
    cells[:, 2:n + 2, 2:n + 2] = prim_to_cons(rho, [u, v], p, g)
    params = hydro_params(2, limiter=MINMOD, bc=[PERIODIC] * 4 + [OUTFLOW] * 2, gamma=g)
    return cells, [1.0 / n, 1.0 / n], params


def spheres_3d(n=256, nspheres=32, seed=0):
    """3-D periodic box: canvas rho 1, p 1, v 0; nspheres sharp spheres with
    centres uniform in the box (periodic images), radii uniform in [4, 16]
    cells (scaled by n/256), density log-uniform in [1, 100], p 1, bulk
    velocity uniform in [-0.5, 0.5] per axis; then rho += 0.05 cos(2 pi x/32)
    (scaled) on the conserved density only. Superbee, gamma 5/3, courant
    COURANT_3D (the reference's default 0.8 is beyond the stability limit of
    its unsplit scheme in 3-D: this workload blows up within 30 steps)."""
    rng = np.random.default_rng(seed)
    g = GAMMA["monatomic"]
    scale = n / 256.0
    rho = np.ones((n, n, n))
    vel = [np.zeros((n, n, n)) for _ in range(3)]
    p = np.ones((n, n, n))
    c = (np.arange(n) + 0.5)
    for _ in range(nspheres):
        ctr = rng.uniform(0.0, n, 3)
        r = rng.uniform(4.0, 16.0) * scale
        dens = 10.0 ** rng.uniform(0.0, 2.0)
        bulk = rng.uniform(-0.5, 0.5, 3)
        d = [np.minimum(np.abs(c - ctr[a]), n - np.abs(c - ctr[a])) for a in range(3)]
        r2 = d[2][:, None, None] ** 2 + d[1][None, :, None] ** 2 + d[0][None, None, :] ** 2
        m = r2 < r * r
        rho[m] = dens
        for a in range(3):
            vel[a][m] = bulk[a]
    cells = empty_box(3, [n, n, n])
    U = prim_to_cons(rho, vel, p, g)
    x = c[None, None, :] * np.ones((n, n, 1))
    U[0] = U[0] + 0.05 * np.cos(2.0 * np.pi * x / (32.0 * scale))
    cells[:, 2:n + 2, 2:n + 2, 2:n + 2] = U
    params = hydro_params(3, limiter=SUPERBEE, bc=[PERIODIC] * 6, gamma=g, courant=COURANT_3D)
    return cells, [1.0 / n] * 3, params


def batch_box(rng, edges=(8, 16, 24, 32, 40, 48, 56, 64)):
    """One box of the many-box workload: edges drawn per axis; either a
    two-state Riemann problem split at the mid-plane of a random axis
    (states as in riemann_1d) or a canvas (rho 1, p 1, v 0) holding a sharp
    centred sphere of radius U[0.1, 0.4] x the shortest edge and density
    log-uniform in [1, 100]. Faces reflective or outflow at random.
    Cell size 1/64 on every axis; van Albada, courant COURANT_3D, gamma 5/3."""
    g = GAMMA["monatomic"]
    dims = [int(rng.choice(edges)) for _ in range(3)]
    cells = empty_box(3, dims)
    n1, n2, n3 = dims
    kind = int(rng.integers(0, 2))
    if kind == 0:
        axis = int(rng.integers(0, 3))
        rho, u, p = riemann_states(rng)
        idx = np.indices((n3, n2, n1))[2 - axis]
        left = idx < dims[axis] // 2
        R = np.where(left, rho[0], rho[1])
        P = np.where(left, p[0], p[1])
        vel = [np.zeros((n3, n2, n1)) for _ in range(3)]
        vel[axis] = np.where(left, u[0], u[1])
        U = prim_to_cons(R, vel, P, g)
    else:
        r = rng.uniform(0.1, 0.4) * min(dims)
        dens = 10.0 ** rng.uniform(0.0, 2.0)
        z, y, x = np.indices((n3, n2, n1)) + 0.5
        r2 = (x - n1 / 2.0) ** 2 + (y - n2 / 2.0) ** 2 + (z - n3 / 2.0) ** 2
        R = np.where(r2 < r * r, dens, 1.0)
        U = prim_to_cons(R, [np.zeros_like(R)] * 3, np.ones_like(R), g)
    cells[:, 2:n3 + 2, 2:n2 + 2, 2:n1 + 2] = U
    bc = [REFLECTIVE if rng.integers(0, 2) == 0 else OUTFLOW for _ in range(6)]
    params = hydro_params(3, limiter=VAN_ALBADA, bc=bc, gamma=g, courant=COURANT_3D)
    return cells, [1.0 / 64] * 3, params


def batch_boxes(nboxes=4096, seed=0):
    rng = np.random.default_rng(seed)
    return [batch_box(rng) for _ in range(nboxes)]
