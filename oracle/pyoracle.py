"""ctypes wrapper over oracle/_build/liboracle.so (test infrastructure only).

Arrays follow the reference's memory layout: a box is the hydro part of the
Fortran array cells(-1:N1+2, -1:N2+2, -1:N3+2, 1:NDIM+2), i.e. a C-ordered
numpy array of shape (NDIM+2, [N3+4,] [N2+4,] N1+4). State vectors are rows
(rho, m_1..m_NDIM, E).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

__all__ = ["set_pow_mode", "pow_mode", "pow_pair", "OracleParams", "params_struct", "lib", "run", "cfl_time_step",
           "set_boundaries", "mh_solve", "riemann_solve", "irs_exec",
           "guess_p_star", "nonlinear_wave", "star_and_sample",
           "slope_limiter", "half_step", "eos"]


class OracleParams(C.Structure):
    _fields_ = [("ndim", C.c_int), ("limiter", C.c_int), ("n_iter", C.c_int),
                ("solver_type", C.c_int), ("bc", C.c_int * 6),
                ("gamma", C.c_double), ("kb_amu", C.c_double),
                ("courant", C.c_double), ("omega", C.c_double),
                ("vac_rho", C.c_double), ("vac_p", C.c_double),
                ("tol", C.c_double), ("inflow", (C.c_double * 5) * 6)]


def params_struct(p):
    """Build OracleParams from a mapping with the hot-path parameters."""
    s = OracleParams()
    s.ndim = int(p["ndim"])
    s.limiter = int(p["limiter"])
    s.n_iter = int(p["n_iter"])
    s.solver_type = int(p.get("solver_type", 2))
    for i, b in enumerate(p["bc"]):
        s.bc[i] = int(b)
    s.gamma = float(p["gamma"])
    s.kb_amu = float(p["kb_amu"])
    s.courant = float(p["courant"])
    s.omega = float(p.get("omega", 0.0))
    s.vac_rho = float(p.get("vac_rho", 0.0))
    s.vac_p = float(p.get("vac_p", 0.0))
    s.tol = float(p["tol"])
    inflow = p.get("inflow")
    if inflow is not None:
        for i in range(6):
            for c in range(min(5, len(inflow[i]))):
                s.inflow[i][c] = float(inflow[i][c])
    return s


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        pp = C.POINTER(OracleParams)
        L.oracle_run.argtypes = [pp, dp, ip, dp, C.c_int, dp, C.c_int, C.POINTER(C.c_longlong)]
        L.oracle_cfl_time_step.argtypes = [pp, dp, ip, dp]
        L.oracle_cfl_time_step.restype = C.c_double
        L.oracle_set_boundaries.argtypes = [pp, dp, ip]
        L.oracle_mh_solve.argtypes = [pp, dp, ip, dp, C.c_double, C.c_int]
        L.oracle_riemann_solve.argtypes = [pp, dp, dp, C.c_longlong, C.c_double, C.c_double, C.c_int, dp]
        L.oracle_irs_exec.argtypes = [C.c_double, C.c_double, C.c_int, dp, C.c_longlong, dp]
        L.oracle_guess_p_star.argtypes = [C.c_double, dp, C.c_longlong, dp]
        L.oracle_nonlinear_wave.argtypes = [C.c_double, dp, C.c_longlong, dp]
        L.oracle_star_and_sample.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                             dp, dp, dp, C.c_double, C.c_longlong, dp]
        L.oracle_slope_limiter.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp, dp, C.c_longlong, dp]
        L.oracle_half_step.argtypes = [C.c_int, C.c_double, dp, dp, C.c_longlong, C.c_int, C.c_double, C.c_double, dp, dp]
        L.oracle_eos.argtypes = [C.c_int, C.c_double, C.c_double, dp, C.c_longlong, C.c_int, dp, dp, dp]
        L.oracle_set_pow_mode.argtypes = [C.c_int]
        L.oracle_pow_pair.argtypes = [dp, dp, C.c_longlong, dp, dp]
        _lib = L
    return _lib


def set_pow_mode(mode):
    """0: C library pow (as the compiled reference); 1: libm_pow::pow, its
    restatement that the CUDA library runs. Returns the previous mode."""
    global _pow_mode
    prev = _pow_mode
    if lib().oracle_set_pow_mode(int(mode)) != 0:
        raise ValueError(mode)
    _pow_mode = int(mode)
    return prev


_pow_mode = 0


class pow_mode:
    """Context manager selecting the oracle's power function."""

    def __init__(self, mode):
        self.mode = mode

    def __enter__(self):
        self.prev = set_pow_mode(self.mode)

    def __exit__(self, *a):
        set_pow_mode(self.prev)


def pow_pair(x, y):
    """(restated pow, C library pow) of the same arguments."""
    x, y = _f64(x), _f64(y)
    mine = np.zeros_like(x)
    libv = np.zeros_like(x)
    lib().oracle_pow_pair(_d(x), _d(y), x.size, _d(mine), _d(libv))
    return mine, libv


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _dims(ndim, cells):
    shp = cells.shape[1:][::-1]  # (ext1, ext2, ext3)
    dims = np.ones(3, dtype=np.int32)
    for a in range(ndim):
        dims[a] = shp[a] - 4
    return dims


def _dx3(dx):
    d = np.ones(3)
    d[:len(dx)] = dx
    return d


def run(p, cells, dx, nsteps, nthreads=0, stats=False):
    """oracle_run: nsteps of (dt -> ghost fill -> solve), in place.

    Returns the dt trace (and [solves, iterations, extra_guesses] if
    stats=True).
    """
    assert cells.dtype == np.float64 and cells.flags.c_contiguous
    P = params_struct(p)
    dims = _dims(P.ndim, cells)
    dts = np.zeros(max(nsteps, 1))
    st = (C.c_longlong * 3)() if stats else None
    rc = lib().oracle_run(C.byref(P), _d(cells), dims.ctypes.data_as(C.POINTER(C.c_int)),
                          _d(_dx3(dx)), int(nsteps), _d(dts), int(nthreads), st)
    if rc != 0:
        raise RuntimeError("oracle_run failed: %d" % rc)
    if stats:
        return dts[:nsteps], [st[0], st[1], st[2]]
    return dts[:nsteps]


def cfl_time_step(p, cells, dx):
    P = params_struct(p)
    cells = _f64(cells)
    dims = _dims(P.ndim, cells)
    return lib().oracle_cfl_time_step(C.byref(P), _d(cells), dims.ctypes.data_as(C.POINTER(C.c_int)), _d(_dx3(dx)))


def set_boundaries(p, cells):
    assert cells.dtype == np.float64 and cells.flags.c_contiguous
    P = params_struct(p)
    dims = _dims(P.ndim, cells)
    rc = lib().oracle_set_boundaries(C.byref(P), _d(cells), dims.ctypes.data_as(C.POINTER(C.c_int)))
    if rc != 0:
        raise RuntimeError("oracle_set_boundaries failed")


def mh_solve(p, cells, dx, dt, nthreads=0):
    assert cells.dtype == np.float64 and cells.flags.c_contiguous
    P = params_struct(p)
    dims = _dims(P.ndim, cells)
    rc = lib().oracle_mh_solve(C.byref(P), _d(cells), dims.ctypes.data_as(C.POINTER(C.c_int)),
                               _d(_dx3(dx)), float(dt), int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle_mh_solve failed")


def riemann_solve(p, l, r, dx, dt, axis):
    """rhyme_riemann_problem_solve for rows of l, r (axis is 0-based)."""
    P = params_struct(p)
    l = _f64(l)
    r = _f64(r)
    u = np.zeros_like(l)
    n = l.shape[0]
    lib().oracle_riemann_solve(C.byref(P), _d(l), _d(r), n, float(dx), float(dt), int(axis), _d(u))
    return u


def irs_exec(gamma, tol, n_iter, states):
    """rhyme_irs_exec; states[n, 8] -> [n, 3] (p*, l_f, r_f)."""
    states = _f64(states)
    out = np.zeros((states.shape[0], 3))
    lib().oracle_irs_exec(float(gamma), float(tol), int(n_iter), _d(states), states.shape[0], _d(out))
    return out


def guess_p_star(gamma, states):
    states = _f64(states)
    out = np.zeros((states.shape[0], 6))
    lib().oracle_guess_p_star(float(gamma), _d(states), states.shape[0], _d(out))
    return out


def nonlinear_wave(gamma, rows):
    rows = _f64(rows)
    out = np.zeros((rows.shape[0], 2))
    lib().oracle_nonlinear_wave(float(gamma), _d(rows), rows.shape[0], _d(out))
    return out


def star_and_sample(gamma, kb_amu, vac_p, tol, n_iter, sides, sample_dx=None, sample_dt=1.0):
    sides = _f64(sides)
    star = np.zeros(10)
    if sample_dx is None:
        sample_dx = np.zeros(0)
    sample_dx = _f64(sample_dx)
    u = np.zeros((len(sample_dx), 3))
    lib().oracle_star_and_sample(float(gamma), float(kb_amu), float(vac_p), float(tol), int(n_iter),
                                 _d(sides), _d(star), _d(sample_dx), float(sample_dt), len(sample_dx), _d(u))
    return star, u


def slope_limiter(ndim, type_, omega, ul, u, ur):
    ul, u, ur = _f64(ul), _f64(u), _f64(ur)
    d = np.zeros_like(u)
    lib().oracle_slope_limiter(int(ndim), int(type_), float(omega), _d(ul), _d(u), _d(ur), u.shape[0], _d(d))
    return d


def half_step(ndim, gamma, u, delta, axis, dx, dt):
    u, delta = _f64(u), _f64(delta)
    l = np.zeros_like(u)
    r = np.zeros_like(u)
    lib().oracle_half_step(int(ndim), float(gamma), _d(u), _d(delta), u.shape[0], int(axis), float(dx), float(dt), _d(l), _d(r))
    return l, r


def eos(ndim, gamma, kb_amu, u, axis):
    """(flux[n, D+2], p[n], cs[n]) for conserved rows u."""
    u = _f64(u)
    f = np.zeros_like(u)
    p = np.zeros(u.shape[0])
    cs = np.zeros(u.shape[0])
    lib().oracle_eos(int(ndim), float(gamma), float(kb_amu), _d(u), u.shape[0], int(axis), _d(f), _d(p), _d(cs))
    return f, p, cs
