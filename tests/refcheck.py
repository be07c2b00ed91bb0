"""Tolerance helpers restating the reference's assertion DSL.

rhyme_assertion_to_be.f90:192      `.toBe.` on doubles:
    |v - e| < max(epsilon(0d0)*v, tiny(0d0))
rhyme_assertion_within.f90:16-23    `.within. n` (integer n, significant
    figures): power = int(log10(|v|)) (truncated toward zero), pass when
    |v - e| <= 10**(power - n + 1), v being the computed value.
"""
import math

import numpy as np

EPS = np.finfo(np.float64).eps
TINY = np.finfo(np.float64).tiny

# kB / amu in SI from the reference's single-precision literals
# (rhyme_units.f90:25,29; rhyme_hydro_base_factory.f90:16-18).
KB_AMU_SI = float(np.float64(np.float32(1.38064852e-23)) / np.float64(np.float32(1.6605e-27)))

GAMMA = {"monatomic": 5.0 / 3.0, "diatomic": 7.0 / 5.0, "polyatomic": 4.0 / 3.0}


def to_be(v, e):
    v = np.asarray(v, dtype=np.float64)
    e = np.asarray(e, dtype=np.float64)
    return np.all(np.abs(v - e) < np.maximum(EPS * v, TINY))


def within(v, e, n):
    v = np.atleast_1d(np.asarray(v, dtype=np.float64))
    e = np.atleast_1d(np.asarray(e, dtype=np.float64))
    ok = True
    for vi, ei in zip(v.ravel(), e.ravel()):
        av = abs(vi)
        power = int(math.log10(av)) if av > 0 else -400
        tol = 10.0 ** (power - n + 1) if power > -300 else 0.0
        if not abs(vi - ei) <= tol:
            ok = False
    return ok
