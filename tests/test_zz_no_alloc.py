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

pytestmark = pytest.mark.gpu


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
        # tolerance is bit-identity with the det-pow oracle)
        assert np.array_equal(_interior(got, ndim), _interior(ref, ndim))


def test_noalloc_rejects_boxes_beyond_the_scratch():
    lib = gpu.load()
    p = hydro_params(3)
    s = gpu.params_struct(p)
    dims = np.array([64, 64, 64], dtype=np.int32)
    dx3 = np.full(3, 1.0 / 64)
    rc = lib.rhyme_gpu_mh_solve_noalloc(C.byref(s), C.c_void_p(16), C.c_void_p(16),
                                        dims.ctypes.data_as(C.POINTER(C.c_int)),
                                        dx3.ctypes.data_as(C.POINTER(C.c_double)), 1e-3, None)
    assert rc == gpu.EINVAL
