"""Device sanity checks and conservation totals against the oracle's loop
restatement of rhyme_sanity_check_fill/perform and
rhyme_samr_calc_total_mass/energy."""
import math

import numpy as np
import pytest

from oracle import sanity as osan
from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import KB_AMU_SI, hydro_params

pytestmark = pytest.mark.gpu


def _box(nd, dims, seed, nans=0):
    rng = np.random.default_rng(seed)
    c = ic.empty_box(nd, dims)
    shp = tuple(dims[::-1])
    rho = np.exp(rng.normal(0, 1, shp))
    vel = [rng.normal(0, 1, shp) for _ in range(nd)]
    p = np.exp(rng.normal(0, 1, shp))
    c[ic.interior(nd, dims)] = ic.prim_to_cons(rho, vel, p, 5.0 / 3.0)
    # a few negative densities / energies, repeated (tied) extremes
    sl = ic.interior(nd, dims)
    r = c[0][sl[1:]]
    r.reshape(-1)[rng.integers(0, r.size, 3)] = -0.5
    e = c[nd + 1][sl[1:]]
    e.reshape(-1)[rng.integers(0, e.size, 2)] = -2.0
    c[0][sl[1:]] = r
    c[nd + 1][sl[1:]] = e
    for _ in range(nans):
        idx = tuple(int(rng.integers(2, s - 2)) for s in c.shape[1:])
        c[(1,) + idx] = np.nan
    # ghosts: arbitrary signed values (the totals include them)
    g = rng.normal(0, 1, c.shape)
    mask = np.ones(c.shape, dtype=bool)
    mask[sl] = False
    c[mask] = g[mask]
    return c


RANGES = {"rho": (0.2, 3.0), "vx": (-1.0, 1.5), "vy": (-2.0, 2.0), "vz": (-1.5, 1.0), "e_tot": (0.0, 8.0),
          "abs_v": (0.0, 2.0), "mach": (0.0, 1.5)}


@pytest.mark.parametrize("nd,dims", [(1, [1000]), (2, [37, 61]), (3, [20, 13, 31])])
def test_sanity_matches_loop(nd, dims):
    c = _box(nd, dims, seed=nd, nans=1)
    ranges = {k: v for k, v in RANGES.items() if not (k == "vy" and nd < 2) and not (k == "vz" and nd < 3)}
    p = hydro_params(nd)
    with gpu.Context(p) as ctx:
        b = ctx.register_box(c)
        props, general = ctx.sanity_check(b, ranges)
        tot = ctx.box_totals(b)
    ref, gref = osan.sanity(c, ranges, kb_amu=KB_AMU_SI)
    for name in ranges:
        a, r = props[name], ref[name]
        if name == "mach":  # cs through the reference's EOS chain; same operations
            for key in ("nbelow", "nabove", "cbelow", "cabove"):
                assert a[key] == r[key], (name, key, a[key], r[key])
            for key in ("vbelow", "vbelow_prev", "vabove", "vabove_prev"):
                assert a[key] == pytest.approx(r[key], rel=1e-14), (name, key)
        else:
            assert a == r, (name, a, r)
    assert general["nan"] == gref["nan"]
    assert general["rho_min"] == gref["rho_min"] and general["rho_min_at"] == gref["rho_min_at"]
    assert general["e_tot_min"] == gref["e_tot_min"] and general["e_tot_min_at"] == gref["e_tot_min_at"]
    seq, exact = osan.totals(c)
    for t, s_, x in zip(tot, seq, exact):
        assert t == x or abs(t - x) <= 2 * math.ulp(x), (t, x)  # the exact sum, rounded
        assert abs(t - s_) <= 1e-12 * abs(x)                       # the reference's sequential sum


def test_totals_after_steps():
    """Totals of a stepped 3-D box (many blocks, ghosts included) equal the
    exact sums of the same state downloaded."""
    cells, dx, p = ic.spheres_3d(n=64, nspheres=8, seed=1)
    with gpu.Context(p) as ctx:
        b = ctx.register_box(cells)
        ctx.run(b, dx, 10)
        m, e = ctx.box_totals(b)
        ctx.sync_to_host(b)
    _, exact = osan.totals(cells)
    assert m == exact[0] or abs(m - exact[0]) <= 2 * math.ulp(exact[0])
    assert e == exact[1] or abs(e - exact[1]) <= 2 * math.ulp(exact[1])


def test_sanity_unknown_box():
    with gpu.Context(hydro_params(2)) as ctx:
        b = ctx.register_box(ic.empty_box(2, [4, 4]))
        ctx.unregister_box(b)
        with pytest.raises(gpu.RhymeGpuError) as e:
            ctx.box_totals(b)
        assert e.value.code == gpu.ENOTFOUND
