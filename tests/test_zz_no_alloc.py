"""The allocation-free solve entry point (rhyme_gpu_mh_solve_noalloc).

It serves callers that cannot allocate device memory (their device arrays
come from their own pool or a Fortran runtime, or they run under a fixed
device-memory budget): they pass device pointers in and out, and the solver's
scratch is a fixed array inside the library. This file is collected last so
that a failure here stops a run only after every other test has run; it
passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import hydro_params


def _reference_step(p, cells, dx, dt):
    """One step through the existing entry point (rhyme_gpu_mh_solve)."""
    host = cells.copy()
    with gpu.Context(p) as ctx:
        box = ctx.register_box(host)
        ctx.muscl_hancock_solve(box, dx, dt)
        ctx.sync_to_host(box)
    return host


def _noalloc_step(p, cells, dx, dt, stream_ptr):
    import torch
    lib = gpu.load()
    d_in = torch.from_numpy(cells.copy()).cuda()
    d_out = d_in.clone()
    dims = np.ones(3, dtype=np.int32)
    ext = cells.shape[1:][::-1]
    for a in range(p["ndim"]):
        dims[a] = ext[a] - 4
    dx3 = np.ones(3)
    dx3[:len(dx)] = dx
    s = gpu.params_struct(p)
    torch.cuda.synchronize()
    rc = lib.rhyme_gpu_mh_solve_noalloc(C.byref(s), C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                        dims.ctypes.data_as(C.POINTER(C.c_int)),
                                        dx3.ctypes.data_as(C.POINTER(C.c_double)), float(dt),
                                        C.c_void_p(stream_ptr))
    assert rc == gpu.OK
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


def _interior(c, ndim):
    return c[(slice(None),) + (slice(2, -2),) * ndim]


@pytest.mark.gpu
@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_noalloc_matches_existing_entry_point_twice(ndim):
    torch = pytest.importorskip("torch")
    if ndim == 1:
        cells, dx, p = ic.riemann_1d(n=256, seed=4)
    elif ndim == 2:
        cells, dx, p = ic.slab_2d(n=64, seed=4)
    else:
        cells, dx, p = ic.spheres_3d(n=24, nspheres=3, seed=4)
    oracle.set_boundaries(p, cells)  # the caller fills the ghosts
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row on different states, sharing the fixed scratch
    second = cells.copy()
    second[0] *= 1.1
    for state in (cells, second):
        dt = oracle.cfl_time_step(p, state, dx)
        ref = _reference_step(p, state, dx, dt)
        got = _noalloc_step(p, state, dx, dt, stream)
        # same kernels, same arithmetic: identical interiors (the FP64 tests'
        # tolerance is bit-identity with the oracle)
        assert np.array_equal(_interior(got, ndim), _interior(ref, ndim))


def _call(lib, p, d_in, d_out, dims, dt=1e-3, stream=None):
    s = gpu.params_struct(p)
    dims = np.array(list(dims) + [1] * (3 - len(dims)), dtype=np.int32)
    dx3 = np.full(3, 1.0 / 64)
    return lib.rhyme_gpu_mh_solve_noalloc(C.byref(s), C.c_void_p(d_in), C.c_void_p(d_out),
                                          dims.ctypes.data_as(C.POINTER(C.c_int)),
                                          dx3.ctypes.data_as(C.POINTER(C.c_double)), dt,
                                          C.c_void_p(stream))


# The scratch holds 2 Mi doubles and a box needs 32 + 3*D*(D+2)*prod(N+4):
# 291^2 and 31^3 fit, 292^2 and 32^3 do not.
@pytest.mark.parametrize("ndim,dims", [(2, (292, 292)), (3, (32, 32, 32)), (3, (64, 64, 64))])
def test_noalloc_rejects_boxes_beyond_the_scratch(ndim, dims):
    # rejected before any CUDA call, so the dummy pointers are never used
    lib = gpu.load()
    assert _call(lib, hydro_params(ndim), 1 << 20, 1 << 30, dims) == gpu.EINVAL


def test_noalloc_rejects_overlapping_state_arrays():
    lib = gpu.load()
    p = hydro_params(1)
    assert _call(lib, p, 1 << 20, 1 << 20, (64,)) == gpu.EINVAL
    assert _call(lib, p, 1 << 20, (1 << 20) + 8, (64,)) == gpu.EINVAL


@pytest.mark.gpu
@pytest.mark.parametrize("ndim,n", [(2, 291), (3, 31)])
def test_noalloc_accepts_boxes_at_the_limit(ndim, n):
    torch = pytest.importorskip("torch")
    if ndim == 2:
        cells, dx, p = ic.slab_2d(n=n, seed=6)
    else:
        cells, dx, p = ic.spheres_3d(n=n, nspheres=2, seed=6)
    oracle.set_boundaries(p, cells)
    dt = oracle.cfl_time_step(p, cells, dx)
    stream = torch.cuda.current_stream().cuda_stream
    got = _noalloc_step(p, cells, dx, dt, stream)
    ref = _reference_step(p, cells, dx, dt)
    assert np.array_equal(_interior(got, ndim), _interior(ref, ndim))
