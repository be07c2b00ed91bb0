"""Seeded stream of hydro-solve requests and its replay against the server.

The stream: Poisson arrivals at `rate` per second; each request is 1-, 2- or
3-D with equal probability, its total cell count log-uniform in
[256, 128^3] split near-cubically, 50-500 steps, initial conditions drawn as
in the 1-D Riemann and 3-D sphere workloads (a two-state Riemann problem
along a random axis, or a canvas holding spheres with a harmonic density
ripple), limiter and boundary types drawn per request. Each request holds
its initial state both as an array and as the equivalent shape list for
painting on the device.

replay() feeds the stream to rhyme_gb300.gpu.Server at the arrival times
(wall clock) and returns per-request latencies (done - submitted, on the
server's clock) and the throughput in cell-updates/s over the makespan.
"""
import time

import numpy as np

from . import gpu, ic
from .params import GAMMA, OUTFLOW, PERIODIC, REFLECTIVE

COURANT = (0.8, 0.5, 0.3)


def _split(total, nd, rng):
    """Near-cubic dims with product ~ total."""
    if nd == 1:
        return [max(4, int(round(total)))]
    base = total ** (1.0 / nd)
    dims = [max(4, int(round(base * f))) for f in rng.uniform(0.8, 1.25, nd)]
    return dims


def _state(nd, dims, rng):
    """The initial state as an array and as the equivalent device shape list
    (rhyme_gb300.drawing) drawn from the same random numbers."""
    from . import drawing
    g = GAMMA["monatomic"]
    shp = tuple(dims[::-1])
    if rng.uniform() < 0.5:
        rho, u, p = ic.riemann_states(rng)
        axis = int(rng.integers(0, nd))
        idx = np.indices(shp)[nd - 1 - axis]
        left = idx < dims[axis] // 2
        R = np.where(left, rho[0], rho[1])
        P = np.where(left, p[0], p[1])
        vel = [np.zeros(shp) for _ in range(nd)]
        vel[axis] = np.where(left, u[0], u[1])
        U = ic.prim_to_cons(R, vel, P, g)
        wl = [rho[0], 0.0, 0.0, 0.0, p[0]]
        wr = [rho[1], 0.0, 0.0, 0.0, p[1]]
        wl[1 + axis], wr[1 + axis] = u[0], u[1]
        lengths = [dims[a] if a != axis else dims[axis] // 2 for a in range(nd)]
        shapes = [drawing.canvas(wr), drawing.sharp_cuboid([1] * nd, lengths, wl)]
    else:
        R = np.ones(shp)
        vel = [np.zeros(shp) for _ in range(nd)]
        grids = np.indices(shp)[::-1] + 0.5
        shapes = [drawing.canvas([1.0, 0.0, 0.0, 0.0, 1.0])]
        for _ in range(int(rng.integers(1, 5))):
            ctr = [rng.uniform(0, d) for d in dims]
            r = rng.uniform(0.1, 0.3) * min(dims)
            d2 = sum((grids[a] - ctr[a]) ** 2 for a in range(nd))
            m = d2 < r * r
            dens = 10.0 ** rng.uniform(0.0, 2.0)
            R[m] = dens
            bulk = rng.uniform(-0.5, 0.5, nd)
            for a in range(nd):
                vel[a][m] = bulk[a]
            inside = [dens, 0.0, 0.0, 0.0, 1.0]
            for a in range(nd):
                inside[1 + a] = bulk[a]
            shapes.append(drawing.sphere(list(ctr), r, inside, keep_outside=True))
        U = ic.prim_to_cons(R, vel, np.ones(shp), g)
        wavelength = max(8.0, dims[0] / 8.0)
        U[0] = U[0] + 0.05 * np.cos(2.0 * np.pi * grids[0] / wavelength)
        shapes.append(drawing.harmonic(0, 0.05, wavelength, [1.0, 0.0, 0.0, 0.0, 0.0]))
    cells = ic.empty_box(nd, dims)
    cells[ic.interior(nd, dims)] = U
    return cells, shapes


def make_stream(n=64, rate=10.0, seed=0, max_cells=128 ** 3):
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(n):
        t += rng.exponential(1.0 / rate)
        nd = int(rng.integers(1, 4))
        total = float(np.exp(rng.uniform(np.log(256.0), np.log(float(max_cells)))))
        dims = _split(total, nd, rng)
        cells, shapes = _state(nd, dims, rng)
        bc = [int(rng.choice([REFLECTIVE, OUTFLOW, PERIODIC])) for _ in range(2 * nd)] + [OUTFLOW] * (6 - 2 * nd)
        out.append(dict(arrival=t, ndim=nd, dims=dims, cells=cells, shapes=shapes, nsteps=int(rng.integers(50, 501)),
                        dx=[1.0 / max(dims)] * nd, limiter=int(rng.integers(1, 5)), bc=bc))
    return out


def replay(stream, base_params, courant=COURANT, hbm_budget=150 << 30, max_active=256, timeout_s=3600.0,
           paint=False):
    """Serve `stream` with submissions at the arrival times; returns a dict
    with latencies (s), makespan (s), cell_updates and the results. With
    paint, each request's initial state is painted on the device from its
    shape list instead of uploaded."""
    outs = [np.zeros_like(r["cells"]) if paint else r["cells"].copy() for r in stream]
    ids = [None] * len(stream)
    with gpu.Server(base_params, courant, hbm_budget, max_active) as srv:
        t0 = time.perf_counter()
        nxt = 0
        peak = 0
        while True:
            now = time.perf_counter() - t0
            while nxt < len(stream) and stream[nxt]["arrival"] <= now:
                r = stream[nxt]
                ids[nxt] = srv.submit(outs[nxt], r["nsteps"], r["dx"], r["limiter"], r["bc"],
                                      shapes=r["shapes"] if paint else None)
                nxt += 1
            a, p, d = srv.tick()
            peak = max(peak, a)
            if nxt == len(stream) and a == 0 and p == 0 and d == 0:
                break
            if a == 0 and p == 0 and d == 0 and nxt < len(stream):
                time.sleep(max(0.0, min(0.01, stream[nxt]["arrival"] - now)))
            if now > timeout_s:
                raise TimeoutError("serving replay exceeded %.0f s" % timeout_s)
        makespan = time.perf_counter() - t0
        lat = []
        for i in ids:
            st, tt, _ = srv.request(i)
            lat.append(tt[2] - tt[0])
        cu, _ = srv.stats()
    return dict(latencies=np.asarray(lat), makespan=makespan, cell_updates=cu, results=outs,
                peak_active=peak)


def run_alone(req, base_params, precision, courant=COURANT):
    """The request stepped on its own (no server) in the given precision:
    its final state array."""
    from .params import hydro_params
    nd = req["ndim"]
    p = hydro_params(nd, limiter=req["limiter"], bc=req["bc"], courant=courant[nd - 1], precision=precision,
                     gamma=base_params.get("gamma", GAMMA["monatomic"]))
    c = req["cells"].copy()
    with gpu.Context(p) as ctx:
        b = ctx.register_box(c)
        ctx.run(b, req["dx"], req["nsteps"], trace=False)
        ctx.sync_to_host(b)
    return c
