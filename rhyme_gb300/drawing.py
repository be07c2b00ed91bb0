"""Shape lists for rhyme_gpu_paint (device initial conditions), and the
seeded workloads of rhyme_gb300.ic expressed as shape lists.

Primitive colours are (rho, u, v, w, p); positions and lengths are in cells
of level 0.
"""
import numpy as np

from . import gpu

CANVAS, SHARP_CUBOID, SPHERE, SMOOTHED_SLAB, HARMONIC, SYMMETRIC_DECAYING = range(6)


def _prim(w):
    w = list(w) + [0.0] * (5 - len(w))
    return [float(x) for x in w]


def _shape(kind, **kw):
    s = gpu.Shape()
    s.type = kind
    s.axis = int(kw.get("axis", 0))
    s.periodic = int(kw.get("periodic", 0))
    s.keep_outside = int(kw.get("keep_outside", 0))
    for i, w in enumerate(kw.get("colors", [])):
        for c, x in enumerate(_prim(w)):
            s.prim[i][c] = x
    for a, x in enumerate(kw.get("left_corner", [])):
        s.left_corner[a] = int(x)
    for a, x in enumerate(kw.get("lengths", [])):
        s.lengths[a] = int(x)
    for a, x in enumerate(kw.get("origin", [])):
        s.origin[a] = float(x)
    s.r = float(kw.get("r", 0.0))
    s.sigma = float(kw.get("sigma", 0.0))
    for a, x in enumerate(kw.get("pos", [])):
        s.pos[a] = float(x)
    for a, x in enumerate(kw.get("slab_sigma", [])):
        s.slab_sigma[a] = float(x)
    s.amplitude = float(kw.get("amplitude", 0.0))
    s.wavelength = float(kw.get("wavelength", 0.0))
    s.phase = float(kw.get("phase", 0.0))
    for c, x in enumerate(_prim(kw.get("base", []))):
        s.base[c] = x
    return s


def canvas(prim):
    return _shape(CANVAS, colors=[prim])


def sharp_cuboid(left_corner, lengths, prim):
    return _shape(SHARP_CUBOID, left_corner=left_corner, lengths=lengths, colors=[prim])


def sphere(origin, r, inside, outside=None, sigma=0.0, periodic=False, keep_outside=False):
    return _shape(SPHERE, origin=origin, r=r, sigma=sigma, colors=[inside, outside or inside], periodic=periodic,
                  keep_outside=keep_outside)


def smoothed_slab(axis, pos, sigma, outside, inside):
    return _shape(SMOOTHED_SLAB, axis=axis, pos=pos, slab_sigma=sigma, colors=[outside, inside])


def harmonic(axis, amplitude, wavelength, base, phase=0.0):
    return _shape(HARMONIC, axis=axis, amplitude=amplitude, wavelength=wavelength, base=base, phase=phase)


def symmetric_decaying(axis, amplitude, pos, sigma, base):
    return _shape(SYMMETRIC_DECAYING, axis=axis, amplitude=amplitude, pos=[pos], sigma=sigma, base=base)


def spheres_3d(n=256, nspheres=32, seed=0):
    """The shapes of rhyme_gb300.ic.spheres_3d (same seeded draws): canvas
    rho 1, p 1; sharp periodic spheres with bulk velocity; harmonic density
    ripple of amplitude 0.05 and wavelength 32 cells (scaled) along x."""
    rng = np.random.default_rng(seed)
    scale = n / 256.0
    out = [canvas([1.0, 0, 0, 0, 1.0])]
    for _ in range(nspheres):
        ctr = rng.uniform(0.0, n, 3)
        r = rng.uniform(4.0, 16.0) * scale
        dens = 10.0 ** rng.uniform(0.0, 2.0)
        bulk = rng.uniform(-0.5, 0.5, 3)
        out.append(sphere(ctr, r, [dens, bulk[0], bulk[1], bulk[2], 1.0], periodic=True, keep_outside=True))
    out.append(harmonic(0, 0.05, 32.0 * scale, [1.0, 0, 0, 0, 0]))
    return out
