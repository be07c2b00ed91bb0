"""Continuous-batching server: every request's result is the same alone and
in the mix (FP64 bit for bit; mixed precision within 1e-12, its FP64
fix-up adds with atomics), requests of all dimensionalities overlap, and
admission respects the HBM budget and the active cap."""
import numpy as np
import pytest

from parity import field_errors

from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import FP64, MIXED, OUTFLOW, PERIODIC, REFLECTIVE, hydro_params

pytestmark = pytest.mark.gpu

COURANT = (0.8, 0.5, 0.3)


def _requests(seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nd = int(rng.integers(1, 4))
        dims = [int(x) for x in rng.integers(6, {1: 200, 2: 40, 3: 16}[nd], nd)]
        cells = ic.empty_box(nd, dims)
        shp = tuple(dims[::-1])
        rho = 1.0 + 0.5 * rng.uniform(size=shp)
        vel = [0.3 * rng.uniform(-1, 1, shp) for _ in range(nd)]
        pr = 1.0 + 0.5 * rng.uniform(size=shp)
        cells[ic.interior(nd, dims)] = ic.prim_to_cons(rho, vel, pr, 5.0 / 3.0)
        bc = [int(rng.choice([REFLECTIVE, OUTFLOW, PERIODIC])) for _ in range(2 * nd)]
        out.append(dict(cells=cells, nsteps=int(rng.integers(3, 12)), dx=[1.0 / max(dims)] * nd,
                        limiter=int(rng.integers(1, 5)), bc=bc + [OUTFLOW] * (6 - 2 * nd)))
    return out


def _alone(req, precision):
    nd = req["cells"].ndim - 1
    p = hydro_params(nd, limiter=req["limiter"], bc=req["bc"], courant=COURANT[nd - 1], precision=precision)
    c = req["cells"].copy()
    with gpu.Context(p) as ctx:
        b = ctx.register_box(c)
        ctx.run(b, req["dx"], req["nsteps"])
        ctx.sync_to_host(b)
    return c


def _serve(reqs, precision, max_active=64, budget=150 << 30):
    base = hydro_params(3, precision=precision)
    outs = [r["cells"].copy() for r in reqs]
    with gpu.Server(base, COURANT, budget, max_active) as srv:
        ids = [srv.submit(o, r["nsteps"], r["dx"], r["limiter"], r["bc"]) for o, r in zip(outs, reqs)]
        peak = 0
        for _ in range(10000):
            a, p, d = srv.tick()
            peak = max(peak, a)
            if a == 0 and p == 0 and d == 0:
                break
        states = [srv.request(i)[0] for i in ids]
    assert all(s == gpu.REQ_DONE for s in states)
    return outs, peak


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_served_equals_alone(precision):
    reqs = _requests(5, 12)
    outs, peak = _serve(reqs, precision)
    assert peak > 1  # requests were in flight together
    for r, o in zip(reqs, outs):
        ref = _alone(r, precision)
        nd = o.ndim - 1
        if precision == FP64:
            assert np.array_equal(o[(slice(None),) + (slice(2, -2),) * nd], ref[(slice(None),) + (slice(2, -2),) * nd])
        else:
            assert max(e[0] for e in field_errors(o, ref, nd)) <= 1e-12


def test_admission_cap():
    reqs = _requests(7, 6)
    outs, peak = _serve(reqs, MIXED, max_active=2)
    assert peak <= 2
    for r, o in zip(reqs, outs):
        ref = _alone(r, MIXED)
        assert max(e[0] for e in field_errors(o, ref, o.ndim - 1)) <= 1e-12


def test_served_output_drain():
    """Requests that ask for it also receive their result in the Chombo
    level-data layout (FP32), equal to packing the FP64 result."""
    from oracle import chombo_pack
    reqs = _requests(9, 6)
    base = hydro_params(3, precision=MIXED)
    outs = [r["cells"].copy() for r in reqs]
    levels = []
    with gpu.Server(base, COURANT, 150 << 30, 64) as srv:
        ids = []
        for o, r in zip(outs, reqs):
            nd = o.ndim - 1
            lv = np.zeros((nd + 2) * int(np.prod([s - 4 for s in o.shape[1:]])), dtype=np.float32)
            levels.append(lv)
            ids.append(srv.submit(o, r["nsteps"], r["dx"], r["limiter"], r["bc"], output=lv))
        for _ in range(10000):
            a, p, d = srv.tick()
            if a == 0 and p == 0 and d == 0:
                break
        assert all(srv.request(i)[0] == gpu.REQ_DONE for i in ids)
    for o, lv in zip(outs, levels):
        assert np.array_equal(lv, chombo_pack.pack_level([o]))
