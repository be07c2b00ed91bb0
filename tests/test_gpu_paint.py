"""Device initial-condition painting (rhyme_gpu_paint) against the oracle's
restatement of the reference's painter. Memberships (cuboid bounds, sharp
spheres) and the algebra are the same operations; tanh, cos and exp may
differ from the C library's by an ulp, hence a 1e-14 relative bar."""
import numpy as np
import pytest

from oracle import drawing as od
from rhyme_gb300 import drawing, gpu, ic
from rhyme_gb300.params import FP64, MIXED, OUTFLOW, PERIODIC, hydro_params

pytestmark = pytest.mark.gpu


def _as_dicts(shapes):
    out = []
    for s in shapes:
        out.append(dict(type=s.type, axis=s.axis, periodic=s.periodic, keep_outside=s.keep_outside,
                        left_corner=list(s.left_corner), lengths=list(s.lengths),
                        colors=[list(s.prim[0]), list(s.prim[1])], origin=list(s.origin), r=s.r, sigma=s.sigma,
                        pos=list(s.pos), slab_sigma=list(s.slab_sigma), amplitude=s.amplitude,
                        wavelength=s.wavelength, phase=s.phase, base=list(s.base)))
    return out


def _paint_both(nd, dims, shapes, left_edge=(1, 1, 1), precision=FP64):
    dev = ic.empty_box(nd, dims)
    with gpu.Context(hydro_params(nd, precision=precision)) as ctx:
        b = ctx.register_box(dev)
        ctx.paint(b, shapes, left_edge)
        ctx.sync_to_host(b)
    ref = od.paint(ic.empty_box(nd, dims), _as_dicts(shapes), left_edge=left_edge)
    return dev, ref


def _close(a, b, rtol=1e-14):
    scale = np.maximum(np.abs(b), 1.0)
    return np.max(np.abs(a - b) / scale) <= rtol


def test_paint_3d_spheres_cuboid_harmonic():
    shapes = [drawing.canvas([1.0, 0, 0, 0, 1.0]),
              drawing.sharp_cuboid([3, 2, 1], [4, 5, 3], [2.0, 0.1, -0.2, 0.3, 1.5]),
              drawing.sphere([5.0, 6.0, 4.0], 3.3, [10.0, 0.5, 0, 0, 1.0], periodic=True, keep_outside=True),
              drawing.sphere([22.0, 1.0, 15.0], 4.0, [30.0, 0, 0.2, 0, 1.0], periodic=True, keep_outside=True),
              drawing.harmonic(0, 0.05, 8.0, [1.0, 0, 0, 0, 0])]
    dev, ref = _paint_both(3, [24, 20, 16], shapes)
    assert _close(dev, ref)
    # the sharp parts are exact: only the harmonic ripple goes through cos
    dev2, ref2 = _paint_both(3, [24, 20, 16], shapes[:-1])
    assert np.array_equal(dev2, ref2)


def test_paint_smooth_sphere_repaints_outside():
    """A smooth sphere blends its colours over every cell, as the reference
    does (a second sphere repaints the first one's outside)."""
    shapes = [drawing.sphere([6.0, 6.0], 3.0, [5.0, 0, 0, 0, 2.0], [1.0, 0, 0, 0, 1.0], sigma=1.0),
              drawing.sphere([14.0, 9.0], 2.5, [3.0, 0.1, 0.1, 0, 1.0], [0.5, 0, 0, 0, 0.7], sigma=0.5)]
    dev, ref = _paint_both(2, [20, 12], shapes)
    assert _close(dev, ref)


def test_paint_2d_slab_and_perturbations():
    shapes = [drawing.smoothed_slab(1, [16.0, 48.0], [2.0, 2.0], [1.0, -0.5, 0, 0, 2.5], [2.0, 0.5, 0, 0, 2.5]),
              drawing.harmonic(0, 0.01, 64.0, [0, 0, 1.0, 0, 0], phase=0.7),
              drawing.harmonic(1, 0.02, 32.0, [0, 0, 0.5, 0, 0]),
              drawing.symmetric_decaying(1, 0.5, 32.0, 40.0, [1.0, 0, 0, 0, 1.0])]
    dev, ref = _paint_both(2, [64, 64], shapes, left_edge=(1, 1))
    assert _close(dev, ref, 1e-13)


def test_paint_1d_riemann_offset_box():
    shapes = [drawing.canvas([0.125, 0, 0, 0, 0.1]),
              drawing.sharp_cuboid([1], [260], [1.0, 0.3, 0, 0, 1.0])]
    dev, ref = _paint_both(1, [200], shapes, left_edge=(101,))
    assert np.array_equal(dev, ref)


def test_paint_mixed_mirror_steps_like_upload():
    """In a mixed-precision context the painted state and its FP32 mirror
    step exactly like the same state uploaded from the host."""
    shapes = drawing.spheres_3d(n=32, nspheres=6, seed=4)
    p = hydro_params(3, bc=[PERIODIC] * 6, courant=0.3, precision=MIXED)
    a = ic.empty_box(3, [32, 32, 32])
    with gpu.Context(p) as ctx:
        b = ctx.register_box(a)
        ctx.paint(b, shapes)
        ctx.sync_to_host(b)
        init = a.copy()
        ctx.run(b, [1 / 32.0] * 3, 4)
        ctx.sync_to_host(b)
    c = init.copy()
    with gpu.Context(p) as ctx:
        b = ctx.register_box(c)
        ctx.run(b, [1 / 32.0] * 3, 4)
        ctx.sync_to_host(b)
    assert np.array_equal(a, c)


def test_server_painted_requests():
    """Requests whose initial state is painted on the device give the same
    result as the painted state uploaded."""
    courant = (0.8, 0.5, 0.3)
    base = hydro_params(3, precision=MIXED)
    reqs = []
    for k in range(4):
        shapes = [drawing.canvas([1.0, 0, 0, 0, 1.0]),
                  drawing.sphere([8.0 + k, 8.0, 8.0], 4.0, [5.0 + k, 0.2, 0, 0, 1.0], periodic=True,
                                 keep_outside=True)]
        reqs.append((shapes, [16, 16, 16], 5 + k))
    painted, uploaded = [], []
    with gpu.Server(base, courant, 150 << 30, 8) as srv:
        ids = []
        for shapes, dims, n in reqs:
            c = ic.empty_box(3, dims)
            painted.append(c)
            ids.append(srv.submit(c, n, [1 / 16.0] * 3, 3, [OUTFLOW] * 6, shapes=shapes))
        for _ in range(1000):
            a, p, d = srv.tick()
            if a == 0 and p == 0 and d == 0:
                break
    with gpu.Server(base, courant, 150 << 30, 8) as srv:
        for shapes, dims, n in reqs:
            c = od.paint(ic.empty_box(3, dims), _as_dicts(shapes))
            uploaded.append(c)
            srv.submit(c, n, [1 / 16.0] * 3, 3, [OUTFLOW] * 6)
        for _ in range(1000):
            a, p, d = srv.tick()
            if a == 0 and p == 0 and d == 0:
                break
    for x, y in zip(painted, uploaded):
        assert np.array_equal(x[:, 2:-2, 2:-2, 2:-2], y[:, 2:-2, 2:-2, 2:-2])


def test_paint_errors():
    with gpu.Context(hydro_params(1)) as ctx:
        b = ctx.register_box(ic.empty_box(1, [16]))
        bad_axis = drawing.harmonic(1, 0.1, 8.0, [1.0, 0, 0, 0, 0])
        with pytest.raises(gpu.RhymeGpuError) as e:
            ctx.paint(b, [bad_axis])
        assert e.value.code == gpu.EINVAL
        slab = drawing.smoothed_slab(0, [2.0, 8.0], [1.0, 1.0], [1.0, 0, 0, 0, 1.0], [2.0, 0, 0, 0, 1.0])
        with pytest.raises(gpu.RhymeGpuError) as e:
            ctx.paint(b, [slab])  # a slab needs NDIM > 1
        assert e.value.code == gpu.EINVAL
        ctx.paint(b, [])  # nothing to paint
