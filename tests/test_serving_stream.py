"""The seeded request stream of the serving workload (rhyme_gb300.serving)
on CPU: deterministic for a seed, within its stated ranges, and each
request's shape list (what the server paints on the device) paints, through
the oracle's painter, the same initial state as the request's array; plus
the parity metric of rhyme_gb300.metrics on known answers."""
import numpy as np
import pytest

from oracle import drawing as od
from rhyme_gb300 import ic, metrics, serving


def _as_dicts(shapes):
    return [dict(type=s.type, axis=s.axis, periodic=s.periodic, keep_outside=s.keep_outside,
                 left_corner=list(s.left_corner), lengths=list(s.lengths),
                 colors=[list(s.prim[0]), list(s.prim[1])], origin=list(s.origin), r=s.r, sigma=s.sigma,
                 pos=list(s.pos), slab_sigma=list(s.slab_sigma), amplitude=s.amplitude,
                 wavelength=s.wavelength, phase=s.phase, base=list(s.base)) for s in shapes]


def test_stream_is_deterministic_and_in_range():
    a = serving.make_stream(n=16, rate=8.0, seed=3, max_cells=24 ** 3)
    b = serving.make_stream(n=16, rate=8.0, seed=3, max_cells=24 ** 3)
    arrivals = [r["arrival"] for r in a]
    assert all(x < y for x, y in zip(arrivals, arrivals[1:]))
    for r, s in zip(a, b):
        assert r["arrival"] == s["arrival"] and r["dims"] == s["dims"] and r["nsteps"] == s["nsteps"]
        assert np.array_equal(r["cells"], s["cells"])
        assert r["ndim"] in (1, 2, 3) and len(r["dims"]) == r["ndim"] and min(r["dims"]) >= 4
        assert 50 <= r["nsteps"] <= 500 and 1 <= r["limiter"] <= 4
        assert all(x in (1, 2, 3) for x in r["bc"][:2 * r["ndim"]])
        assert r["cells"].shape == ic.empty_box(r["ndim"], r["dims"]).shape
    assert serving.make_stream(n=16, rate=8.0, seed=4, max_cells=24 ** 3)[0]["arrival"] != a[0]["arrival"]


@pytest.mark.parametrize("seed", [0, 1])
def test_shape_lists_paint_the_arrays(seed):
    for r in serving.make_stream(n=10, rate=8.0, seed=seed, max_cells=20 ** 3):
        nd = r["ndim"]
        painted = od.paint(ic.empty_box(nd, r["dims"]), _as_dicts(r["shapes"]))
        inner = ic.interior(nd, r["dims"])
        a, b = painted[inner], r["cells"][inner]
        scale = np.maximum(np.abs(b), 1.0)
        assert np.max(np.abs(a - b) / scale) <= 1e-13, (nd, r["dims"])


def test_field_errors_known_answers():
    ref = ic.empty_box(2, [4, 3])
    ref[:, 2:-2, 2:-2] = 2.0
    got = ref.copy()
    got[0, 2, 2] += 0.5            # one interior cell of rho
    got[1, 0, 0] = 99.0            # a ghost cell: not counted
    errs = metrics.field_errors(got, ref, 2)
    assert errs[0][0] == pytest.approx(0.5 / 24.0) and errs[0][1] == pytest.approx(0.25)
    assert errs[1] == (0.0, 0.0)
