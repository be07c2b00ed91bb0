"""Test infrastructure (the checker, never the product): numpy restatement
of the hydro part of the reference's initial-condition painter, cell by cell
in its evaluation order.

rhyme_drawing_init.f90:20-78 (canvas, shapes in order, then the
perturbations); rhyme_drawing_uniform_canvas.f90; rhyme_drawing_sharp_cuboid
.f90:44-60 (bounds lb = left_corner - left_edge, ub = left_corner + lengths
- left_edge, clamped); rhyme_drawing_sphere.f90:96 and smoothing_factor
:189-209 (x = cell - 0.5, f = (1 + tanh((r - dist)/sigma))/2, colours
blended in primitive form); rhyme_drawing_smoothed_slab_2d.f90:63-85;
rhyme_drawing_apply_perturbations.f90 (harmonic A cos(2 pi/lambda x) base,
symmetric decaying A exp(-x^2/sigma) base, product when both, added as a
conserved vector). The extensions of the device painter (periodic images,
sharp spheres that keep the outside, harmonic phase) are restated too.
Shapes are dicts with the fields of rhyme_gpu_shape.
"""
import math

import numpy as np


def prim_to_cons(w, nd, gamma):
    """(rho, v_1..v_nd, p) -> (rho, rho v, 0.5 rho |v|^2 + p/(gamma-1)),
    as rhyme_ideal_gas_primitive_vars_to_conserved."""
    rho = w[0]
    u = [rho]
    s = 0.0
    for a in range(nd):
        u.append(rho * w[1 + a])
        s = s + w[1 + a] * w[1 + a]
    u.append(0.5 * rho * s + w[nd + 1] / (gamma - 1.0))
    return u


def _pack(w5, nd):
    w5 = list(w5) + [0.0] * (5 - len(w5))
    return [float(w5[0])] + [float(w5[1 + a]) for a in range(nd)] + [float(w5[4])]


def paint(cells, shapes, gamma=5.0 / 3.0, left_edge=(1, 1, 1)):
    """Paints the interior of `cells` (reference layout) in place."""
    nd = cells.ndim - 1
    K = nd + 2
    dims = [s - 4 for s in cells.shape[1:]][::-1] + [1] * (3 - nd)
    le = list(left_edge) + [1] * (3 - len(left_edge))
    pi = 4.0 * math.atan(1.0)
    bounds = []
    for s in shapes:
        lb, ub = [], []
        for a in range(3):
            lc = s.get("left_corner", [0, 0, 0])[a] if a < len(s.get("left_corner", [])) else 0
            ln = s.get("lengths", [0, 0, 0])[a] if a < len(s.get("lengths", [])) else 0
            x = lc - le[a]
            x = 1 if x < 1 else x
            x = dims[a] + 1 if x > dims[a] else x
            y = lc + ln - le[a]
            y = 0 if y < 1 else y
            y = dims[a] if y > dims[a] else y
            lb.append(x)
            ub.append(y)
        bounds.append((lb, ub))
    for k in range(1, dims[2] + 1):
        for j in range(1, dims[1] + 1):
            for i in range(1, dims[0] + 1):
                idx = [i, j, k]
                pos = tuple(v + 1 for v in ([k, j][: nd - 1] if nd == 3 else ([j] if nd == 2 else []))) + (i + 1,)
                u = [float(cells[(c,) + pos]) for c in range(K)]
                xl = [idx[a] - 0.5 for a in range(3)]
                xg = [idx[a] - 0.5 + le[a] - 1.0 for a in range(3)]
                h = [0.0] * K
                d = [0.0] * K
                has_h = has_d = False
                for s, (lb, ub) in zip(shapes, bounds):
                    t = s["type"]
                    if t == 0:
                        u = prim_to_cons(_pack(s["colors"][0], nd), nd, gamma)
                    elif t == 1:
                        if all(lb[a] <= idx[a] <= ub[a] for a in range(nd)):
                            u = prim_to_cons(_pack(s["colors"][0], nd), nd, gamma)
                    elif t == 2:
                        ss = 0.0
                        for a in range(nd):
                            dd = xl[a] - s["origin"][a]
                            if s.get("periodic"):
                                dd = abs(dd)
                                e = dims[a] - dd
                                if e < dd:
                                    dd = e
                            ss = ss + dd * dd
                        dist = math.sqrt(ss)
                        sigma = s.get("sigma", 0.0)
                        if sigma > 0.0:
                            f = (1.0 + math.tanh((s["r"] - dist) / sigma)) / 2.0
                        else:
                            f = 1.0 if dist < s["r"] else 0.0
                            if f == 0.0 and s.get("keep_outside"):
                                continue
                        w1 = _pack(s["colors"][0], nd)
                        w2 = _pack(s["colors"][1], nd)
                        u = prim_to_cons([f * a + (1.0 - f) * b for a, b in zip(w1, w2)], nd, gamma)
                    elif t == 3:
                        x = xg[s["axis"]]
                        centre = (s["pos"][0] + s["pos"][1]) / 2.0
                        rs = abs(centre - s["pos"][0])
                        fac = (1.0 + math.tanh((rs - (x - centre)) / s["slab_sigma"][0])) * \
                              (1.0 + math.tanh((rs + (x - centre)) / s["slab_sigma"][1]))
                        w1 = _pack(s["colors"][0], nd)
                        w2 = _pack(s["colors"][1], nd)
                        u = prim_to_cons([a + 0.25 * (b - a) * fac for a, b in zip(w1, w2)], nd, gamma)
                    elif t == 4:
                        kx = 2.0 * pi / s["wavelength"] * xg[s["axis"]] + s.get("phase", 0.0)
                        ak = s["amplitude"] * math.cos(kx)
                        base = _pack(s["base"], nd)
                        h = [h[c] + ak * base[c] for c in range(K)]
                        has_h = True
                    elif t == 5:
                        xr = xg[s["axis"]] - s["pos"][0]
                        ad = s["amplitude"] * math.exp(-(xr * xr) / s["sigma"])
                        base = _pack(s["base"], nd)
                        d = [d[c] + ad * base[c] for c in range(K)]
                        has_d = True
                if has_h or has_d:
                    w = [(h[c] * d[c] if has_d else h[c]) if has_h else d[c] for c in range(K)]
                    du = prim_to_cons(w, nd, gamma)
                    u = [u[c] + du[c] for c in range(K)]
                for c in range(K):
                    cells[(c,) + pos] = u[c]
    return cells
