"""ctypes binding of librhyme_gpu.so, mirroring Rhyme's module interfaces.

    ctx = Context(hydro_params(...))             # rhyme_*_init
    box = ctx.register_box(cells)                # samr%levels(0)%boxes(1)
    dt  = ctx.cfl_time_step(box, dx)             # rhyme_cfl_time_step
    ctx.set_boundaries(box)                      # rhyme_samr_bc_set_boundaries
    ctx.muscl_hancock_solve(box, dx, dt)         # rhyme_muscl_hancock_solve
    ctx.sync_to_host(box)                        # cells now hold the new state

`cells` is a C-ordered float64 numpy array of shape
(NCMP, [N3+4,] [N2+4,] N1+4): the memory of the Fortran array
cells(-1:N1+2, ..., 1:NCMP). There is no CPU fallback: if the library is
missing or no GPU is present, calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "librhyme_gpu.so")

OK, EINVAL, ENOMEM, ECUDA, ETIMEDOUT, ENANSTATE, ENOTFOUND = 0, -1, -2, -3, -4, -5, -6
_NAMES = {EINVAL: "EINVAL", ENOMEM: "ENOMEM", ECUDA: "ECUDA", ETIMEDOUT: "ETIMEDOUT",
          ENANSTATE: "ENANSTATE", ENOTFOUND: "ENOTFOUND"}

# Every symbol include/rhyme_gpu.h declares.
EXPORTS = ["rhyme_gpu_abi_version", "rhyme_gpu_create", "rhyme_gpu_destroy", "rhyme_gpu_last_error",
           "rhyme_gpu_get_stream", "rhyme_gpu_register_box", "rhyme_gpu_unregister_box",
           "rhyme_gpu_sync_to_device", "rhyme_gpu_sync_to_host", "rhyme_gpu_set_host_writeback",
           "rhyme_gpu_get_rows", "rhyme_gpu_set_rows",
           "rhyme_gpu_cfl_time_step", "rhyme_gpu_cfl_dt",
           "rhyme_gpu_set_boundaries", "rhyme_gpu_mh_solve", "rhyme_gpu_run", "rhyme_gpu_synchronize",
           "rhyme_gpu_riemann_solve", "rhyme_gpu_irs_exec", "rhyme_gpu_slope_limiter",
           "rhyme_gpu_half_step", "rhyme_gpu_profile_steps", "rhyme_gpu_box_status",
           "rhyme_gpu_fallback_count", "rhyme_gpu_mh_solve_noalloc", "rhyme_gpu_set_box_params",
           "rhyme_gpu_tma_launches", "rhyme_gpu_rate_probe", "rhyme_gpu_check_conversions",
           "rhyme_gpu_batch_create", "rhyme_gpu_batch_run", "rhyme_gpu_batch_dt", "rhyme_gpu_batch_destroy",
           "rhyme_gpu_server_create", "rhyme_gpu_server_submit", "rhyme_gpu_server_tick",
           "rhyme_gpu_server_request", "rhyme_gpu_server_stats", "rhyme_gpu_server_last_error",
           "rhyme_gpu_server_destroy", "rhyme_gpu_sweep_plan",
           "rhyme_gpu_output_level", "rhyme_gpu_output_wait", "rhyme_gpu_box_totals",
           "rhyme_gpu_sanity_check", "rhyme_gpu_paint"]
REQ_PENDING, REQ_ACTIVE, REQ_DRAINING, REQ_DONE = 0, 1, 2, 3


class Shape(C.Structure):
    """struct rhyme_gpu_shape (include/rhyme_gpu.h); see rhyme_gb300.drawing."""
    _fields_ = [("type", C.c_int), ("axis", C.c_int), ("periodic", C.c_int), ("keep_outside", C.c_int),
                ("left_corner", C.c_int * 3), ("lengths", C.c_int * 3), ("prim", (C.c_double * 5) * 2),
                ("origin", C.c_double * 3), ("r", C.c_double), ("sigma", C.c_double), ("pos", C.c_double * 2),
                ("slab_sigma", C.c_double * 2), ("amplitude", C.c_double), ("wavelength", C.c_double),
                ("phase", C.c_double), ("base", C.c_double * 5)]


class Request(C.Structure):
    """struct rhyme_gpu_request (include/rhyme_gpu.h)."""
    _fields_ = [("ndim", C.c_int), ("dims", C.c_int * 3), ("nsteps", C.c_int), ("limiter", C.c_int),
                ("bc", C.c_int * 6), ("omega", C.c_double), ("dx", C.c_double * 3),
                ("cells", C.POINTER(C.c_double)), ("output", C.POINTER(C.c_float)),
                ("shapes", C.POINTER(Shape)), ("nshapes", C.c_int), ("reserved", C.c_int)]
SANITY_PROPERTIES = ["rho", "vx", "vy", "vz", "e_tot", "abs_v", "mach"]


class SanityProperty(C.Structure):
    """struct rhyme_gpu_sanity_property (include/rhyme_gpu.h)."""
    _fields_ = [("range", C.c_double * 2), ("enabled", C.c_int), ("reserved", C.c_int),
                ("nbelow", C.c_longlong), ("nabove", C.c_longlong), ("vbelow", C.c_double),
                ("vbelow_prev", C.c_double), ("vabove", C.c_double), ("vabove_prev", C.c_double),
                ("cbelow", C.c_int * 3), ("cabove", C.c_int * 3)]


class SanityReport(C.Structure):
    """struct rhyme_gpu_sanity_report (include/rhyme_gpu.h)."""
    _fields_ = [("prop", SanityProperty * 7), ("nan", C.c_int * 5), ("reserved", C.c_int),
                ("rho_min", C.c_double), ("e_tot_min", C.c_double), ("rho_min_at", C.c_int * 3),
                ("e_tot_min_at", C.c_int * 3)]


PHASES = ["cfl", "ghost_fill", "faces", "fluxes", "update"]
PHASES_MIXED = ["cfl", "ghost_fill", "sweep_x", "sweep_y", "sweep_z"]


class RhymeGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_NAMES.get(code, "?"), code, msg))
        self.code = code


class Params(C.Structure):
    """struct rhyme_gpu_params (include/rhyme_gpu.h)."""
    _fields_ = [("ndim", C.c_int), ("limiter", C.c_int), ("n_iteration", C.c_int),
                ("solver_type", C.c_int), ("bc", C.c_int * 6), ("precision", C.c_int),
                ("sweep_tuning", C.c_int), ("gamma", C.c_double), ("kb_amu", C.c_double),
                ("courant", C.c_double), ("omega", C.c_double), ("vacuum_density", C.c_double),
                ("vacuum_pressure", C.c_double), ("tolerance", C.c_double),
                ("inflow", (C.c_double * 5) * 6)]


def params_struct(p):
    s = Params()
    s.ndim = p["ndim"]
    s.limiter = p["limiter"]
    s.n_iteration = p["n_iter"]
    s.solver_type = p.get("solver_type", 2)
    for i, b in enumerate(p["bc"]):
        s.bc[i] = b
    s.precision = p.get("precision", 0)
    s.sweep_tuning = p.get("sweep_tuning", 0)
    s.gamma = p["gamma"]
    s.kb_amu = p["kb_amu"]
    s.courant = p["courant"]
    s.omega = p.get("omega", 0.0)
    s.vacuum_density = p.get("vac_rho", 0.0)
    s.vacuum_pressure = p.get("vac_p", 0.0)
    s.tolerance = p["tol"]
    inflow = p.get("inflow")
    if inflow is not None:
        for i in range(6):
            for c in range(min(5, len(inflow[i]))):
                s.inflow[i][c] = inflow[i][c]
    return s


_lib = None


def load():
    """Load librhyme_gpu.so (built by rhyme_gb300.build / __graft_entry__.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("librhyme_gpu.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    dp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p
    L.rhyme_gpu_abi_version.restype = C.c_int
    L.rhyme_gpu_create.argtypes = [C.POINTER(vp), C.POINTER(Params)]
    L.rhyme_gpu_destroy.argtypes = [vp]
    L.rhyme_gpu_last_error.argtypes = [vp]
    L.rhyme_gpu_last_error.restype = C.c_char_p
    L.rhyme_gpu_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.rhyme_gpu_register_box.argtypes = [vp, C.c_int, C.c_int, dp, ip, C.c_int, C.c_int, ip]
    L.rhyme_gpu_unregister_box.argtypes = [vp, C.c_int]
    L.rhyme_gpu_sync_to_device.argtypes = [vp, C.c_int]
    L.rhyme_gpu_sync_to_host.argtypes = [vp, C.c_int]
    L.rhyme_gpu_set_host_writeback.argtypes = [vp, C.c_int, C.c_int]
    L.rhyme_gpu_get_rows.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
    L.rhyme_gpu_set_rows.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
    L.rhyme_gpu_cfl_time_step.argtypes = [vp, C.c_int, dp, dp]
    L.rhyme_gpu_set_boundaries.argtypes = [vp, C.c_int]
    L.rhyme_gpu_cfl_dt.argtypes = [vp, C.c_int, dp]
    L.rhyme_gpu_cfl_dt.restype = C.c_double
    L.rhyme_gpu_mh_solve.argtypes = [vp, C.c_int, dp, C.c_double]
    L.rhyme_gpu_run.argtypes = [vp, C.c_int, dp, C.c_int, dp]
    L.rhyme_gpu_synchronize.argtypes = [vp]
    L.rhyme_gpu_riemann_solve.argtypes = [vp, dp, dp, C.c_longlong, C.c_double, C.c_double, C.c_int, dp]
    L.rhyme_gpu_irs_exec.argtypes = [vp, dp, C.c_longlong, dp]
    L.rhyme_gpu_slope_limiter.argtypes = [vp, dp, dp, dp, C.c_longlong, dp]
    L.rhyme_gpu_half_step.argtypes = [vp, dp, dp, C.c_longlong, C.c_int, C.c_double, C.c_double, dp, dp]
    L.rhyme_gpu_profile_steps.argtypes = [vp, C.c_int, dp, C.c_int, dp]
    L.rhyme_gpu_box_status.argtypes = [vp, C.c_int, ip]
    L.rhyme_gpu_fallback_count.argtypes = [vp, C.c_int, C.POINTER(C.c_longlong)]
    L.rhyme_gpu_tma_launches.argtypes = [C.POINTER(C.c_longlong)]
    L.rhyme_gpu_rate_probe.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.rhyme_gpu_check_conversions.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_ulonglong)]
    L.rhyme_gpu_sweep_plan.argtypes = [vp, C.c_int, dp, ip, ip]
    L.rhyme_gpu_output_level.argtypes = [vp, ip, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_longlong]
    L.rhyme_gpu_output_wait.argtypes = [vp]
    L.rhyme_gpu_box_totals.argtypes = [vp, C.c_int, dp]
    L.rhyme_gpu_sanity_check.argtypes = [vp, C.c_int, C.POINTER(SanityReport)]
    L.rhyme_gpu_paint.argtypes = [vp, C.c_int, ip, C.POINTER(Shape), C.c_int]
    L.rhyme_gpu_mh_solve_noalloc.argtypes = [C.POINTER(Params), vp, vp, ip, dp, C.c_double, vp]
    L.rhyme_gpu_set_box_params.argtypes = [vp, C.c_int, ip, C.c_int, C.c_double]
    L.rhyme_gpu_batch_create.argtypes = [vp, ip, dp, C.c_int, C.POINTER(vp)]
    L.rhyme_gpu_batch_run.argtypes = [vp, C.c_int]
    L.rhyme_gpu_batch_dt.argtypes = [vp, dp]
    L.rhyme_gpu_batch_destroy.argtypes = [vp]
    L.rhyme_gpu_server_create.argtypes = [C.POINTER(Params), dp, C.c_longlong, C.c_int, C.POINTER(vp)]
    L.rhyme_gpu_server_submit.argtypes = [vp, C.POINTER(Request), ip]
    L.rhyme_gpu_server_tick.argtypes = [vp, ip, ip, ip]
    L.rhyme_gpu_server_request.argtypes = [vp, C.c_int, ip, dp, ip]
    L.rhyme_gpu_server_stats.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.rhyme_gpu_server_last_error.argtypes = [vp]
    L.rhyme_gpu_server_last_error.restype = C.c_char_p
    L.rhyme_gpu_server_destroy.argtypes = [vp]
    _lib = L
    return L


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _dx3(dx):
    d = np.ones(3)
    d[:len(dx)] = dx
    return d


class Box:
    def __init__(self, ctx, handle, cells, dims):
        self.ctx, self.handle, self.cells, self.dims = ctx, handle, cells, dims


class Batch:
    """rhyme_gpu_batch: independent boxes stepped together (own dt each)."""

    def __init__(self, ctx, boxes, dxs):
        self.ctx = ctx
        self.boxes = list(boxes)
        n = len(self.boxes)
        handles = np.array([b.handle for b in self.boxes], dtype=np.int32)
        dx = np.ones((n, 3))
        for i, d in enumerate(dxs):
            dx[i, :len(d)] = d
        h = C.c_void_p()
        ctx._check(ctx.lib.rhyme_gpu_batch_create(ctx.h, handles.ctypes.data_as(C.POINTER(C.c_int)),
                                                   _d(dx), n, C.byref(h)))
        self.h = h

    def run(self, nsteps):
        self.ctx._check(self.ctx.lib.rhyme_gpu_batch_run(self.h, int(nsteps)))

    def dts(self):
        out = np.zeros(len(self.boxes))
        self.ctx._check(self.ctx.lib.rhyme_gpu_batch_dt(self.h, _d(out)))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.rhyme_gpu_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Context:
    """One rhyme_gpu_ctx: run parameters, a CUDA stream, registered boxes."""

    def __init__(self, params):
        self.lib = load()
        self.params = dict(params)
        self.ndim = int(params["ndim"])
        self._p = params_struct(params)
        h = C.c_void_p()
        rc = self.lib.rhyme_gpu_create(C.byref(h), C.byref(self._p))
        if rc != OK:
            raise RhymeGpuError(rc, "rhyme_gpu_create failed (see stderr)")
        self.h = h
        self.boxes = []

    def _check(self, rc):
        if rc != OK:
            raise RhymeGpuError(rc, self.lib.rhyme_gpu_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.rhyme_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        s = C.c_void_p()
        self._check(self.lib.rhyme_gpu_get_stream(self.h, C.byref(s)))
        return s.value or 0

    # ---- boxes ---------------------------------------------------------
    def register_box(self, cells, level=0, number=1):
        assert cells.dtype == np.float64 and cells.flags.c_contiguous
        D = self.ndim
        ext = cells.shape[1:][::-1]
        assert len(ext) == D, "cells must have NDIM spatial axes"
        dims = np.ones(3, dtype=np.int32)
        for a in range(D):
            dims[a] = ext[a] - 4
        handle = C.c_int()
        self._check(self.lib.rhyme_gpu_register_box(self.h, level, number, _d(cells),
                                                    dims.ctypes.data_as(C.POINTER(C.c_int)), 2,
                                                    cells.shape[0], C.byref(handle)))
        b = Box(self, handle.value, cells, dims)
        self.boxes.append(b)
        return b

    def unregister_box(self, box):
        self._check(self.lib.rhyme_gpu_unregister_box(self.h, box.handle))

    def sync_to_device(self, box):
        self._check(self.lib.rhyme_gpu_sync_to_device(self.h, box.handle))

    def sync_to_host(self, box):
        self._check(self.lib.rhyme_gpu_sync_to_host(self.h, box.handle))

    def rows_shape(self, box, nrows):
        return (self.ndim + 2, int(nrows)) + box.cells.shape[2:]

    def get_rows(self, box, row0, nrows, out=None):
        """Rows [row0, row0 + nrows) of the outermost axis of the box's
        ghosted block, shape (NDIM+2, nrows, ...): into a new host array, or
        into `out`, a contiguous float64 torch CUDA tensor of that shape
        (the rows then stay on the device)."""
        if out is None:
            out = np.empty(self.rows_shape(box, nrows), dtype=np.float64)
            ptr = _d(out)
        else:
            assert out.is_cuda and out.is_contiguous() and tuple(out.shape) == self.rows_shape(box, nrows)
            ptr = C.c_void_p(out.data_ptr())
        self._check(self.lib.rhyme_gpu_get_rows(self.h, box.handle, int(row0), int(nrows), ptr))
        return out

    def set_rows(self, box, row0, rows):
        """Writes rows (as from get_rows: a host array, or a contiguous
        float64 torch CUDA tensor) at row0 into both state buffers."""
        if hasattr(rows, "is_cuda") and rows.is_cuda:
            assert rows.is_contiguous() and rows.dtype.is_floating_point and rows.element_size() == 8
            ptr, n = C.c_void_p(rows.data_ptr()), int(rows.shape[1])
        else:
            rows = np.ascontiguousarray(rows, dtype=np.float64)
            ptr, n = _d(rows), int(rows.shape[1])
        self._check(self.lib.rhyme_gpu_set_rows(self.h, box.handle, int(row0), n, ptr))

    def set_host_writeback(self, box, on=True):
        """Each solve of the box also copies the new state into its cells
        array (overlapped with the solve for large 2-/3-D mixed boxes);
        sync_to_host then only waits for those copies."""
        self._check(self.lib.rhyme_gpu_set_host_writeback(self.h, box.handle, 1 if on else 0))

    def box_status(self, box):
        """Status bits of the box since the last query (0 = clean)."""
        f = C.c_int()
        rc = self.lib.rhyme_gpu_box_status(self.h, box.handle, C.byref(f))
        if rc not in (OK, ENANSTATE):
            self._check(rc)
        return f.value

    def fallback_count(self, box):
        """Interfaces redone in FP64 by the mixed solver since the last query."""
        n = C.c_longlong()
        self._check(self.lib.rhyme_gpu_fallback_count(self.h, box.handle, C.byref(n)))
        return n.value

    def sweep_plan(self, box, dx):
        """[(cells along the axis, pencils)] per axis of the box's mixed
        sweeps (empty in FP64 mode)."""
        s = np.zeros(3, dtype=np.int32)
        p = np.zeros(3, dtype=np.int32)
        self._check(self.lib.rhyme_gpu_sweep_plan(self.h, box.handle, _d(_dx3(dx)),
                                                  s.ctypes.data_as(C.POINTER(C.c_int)),
                                                  p.ctypes.data_as(C.POINTER(C.c_int))))
        return [(int(a), int(b)) for a, b in zip(s, p) if a]

    def output_level(self, boxes, ncmp=None, out=None):
        """Start the level output of `boxes` (the Chombo "data:datatype=0"
        layout, FP32, hydro components); returns the float32 array that
        receives it once output_wait() returns."""
        ncmp = self.ndim + 2 if ncmp is None else int(ncmp)
        n = sum(int(np.prod(b.dims[:self.ndim])) for b in boxes) * ncmp
        if out is None:
            out = np.zeros(n, dtype=np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous
        handles = np.array([b.handle for b in boxes], dtype=np.int32)
        self._keep_out = (out, handles)
        self._check(self.lib.rhyme_gpu_output_level(self.h, handles.ctypes.data_as(C.POINTER(C.c_int)),
                                                    len(boxes), ncmp, out.ctypes.data_as(C.POINTER(C.c_float)),
                                                    out.size))
        return out

    def box_totals(self, box):
        """(sum of rho > 0, sum of e_tot > 0) over all cells, ghosts included."""
        t = np.zeros(2)
        self._check(self.lib.rhyme_gpu_box_totals(self.h, box.handle, _d(t)))
        return float(t[0]), float(t[1])

    def sanity_check(self, box, ranges):
        """ranges: {property: (lo, hi)} for the enabled properties (names in
        SANITY_PROPERTIES). Returns (report dict per property, general
        checks dict)."""
        rep = SanityReport()
        for i, name in enumerate(SANITY_PROPERTIES):
            if name in ranges:
                rep.prop[i].enabled = 1
                rep.prop[i].range[0], rep.prop[i].range[1] = ranges[name]
        self._check(self.lib.rhyme_gpu_sanity_check(self.h, box.handle, C.byref(rep)))
        props = {}
        for i, name in enumerate(SANITY_PROPERTIES):
            if name in ranges:
                q = rep.prop[i]
                props[name] = dict(nbelow=q.nbelow, nabove=q.nabove, vbelow=q.vbelow, vbelow_prev=q.vbelow_prev,
                                   vabove=q.vabove, vabove_prev=q.vabove_prev, cbelow=tuple(q.cbelow),
                                   cabove=tuple(q.cabove))
        general = dict(nan=[bool(x) for x in rep.nan[:self.ndim + 2]], rho_min=rep.rho_min,
                       e_tot_min=rep.e_tot_min, rho_min_at=tuple(rep.rho_min_at),
                       e_tot_min_at=tuple(rep.e_tot_min_at))
        return props, general

    def paint(self, box, shapes, left_edge=(1, 1, 1)):
        """Paint the box's initial state on the device from a list of Shape
        (rhyme_gb300.drawing builds them)."""
        arr = (Shape * max(1, len(shapes)))(*shapes)
        le = np.asarray(list(left_edge) + [1] * (3 - len(left_edge)), dtype=np.int32)
        self._check(self.lib.rhyme_gpu_paint(self.h, box.handle, le.ctypes.data_as(C.POINTER(C.c_int)), arr,
                                             len(shapes)))

    def output_wait(self):
        self._check(self.lib.rhyme_gpu_output_wait(self.h))

    def synchronize(self):
        self._check(self.lib.rhyme_gpu_synchronize(self.h))

    def set_box_params(self, box, bc=None, limiter=None, omega=None):
        """Per-box boundary types / limiter / omega (defaults: the context's)."""
        limiter = self.params["limiter"] if limiter is None else limiter
        omega = self.params.get("omega", 0.0) if omega is None else omega
        bcs = None
        if bc is not None:
            bcs = np.zeros(6, dtype=np.int32)
            bcs[:len(bc)] = bc
        self._check(self.lib.rhyme_gpu_set_box_params(
            self.h, box.handle, bcs.ctypes.data_as(C.POINTER(C.c_int)) if bcs is not None else None,
            int(limiter), float(omega)))

    def batch(self, boxes, dxs):
        """A Batch stepping `boxes` together (dxs: one cell size per box)."""
        return Batch(self, boxes, dxs)

    # ---- the driver's step ---------------------------------------------
    def cfl_time_step(self, box, dx):
        dt = C.c_double()
        self._check(self.lib.rhyme_gpu_cfl_time_step(self.h, box.handle, _d(_dx3(dx)), C.byref(dt)))
        return dt.value

    def set_boundaries(self, box):
        self._check(self.lib.rhyme_gpu_set_boundaries(self.h, box.handle))

    def muscl_hancock_solve(self, box, dx, dt):
        self._check(self.lib.rhyme_gpu_mh_solve(self.h, box.handle, _d(_dx3(dx)), float(dt)))

    def run(self, box, dx, nsteps, trace=True):
        """nsteps driver iterations on the device; returns the dt trace."""
        dts = np.zeros(max(int(nsteps), 1)) if trace else None
        self._check(self.lib.rhyme_gpu_run(self.h, box.handle, _d(_dx3(dx)), int(nsteps),
                                           _d(dts) if trace else None))
        return dts[:nsteps] if trace else None

    def profile_steps(self, box, dx, nsteps):
        """Mean ms per step of each phase (PHASES, or PHASES_MIXED in mixed
        precision, with sweep_xy for sweep_x and sweep_y where one kernel ran
        both) over nsteps steps."""
        ms = np.zeros(5)
        self._check(self.lib.rhyme_gpu_profile_steps(self.h, box.handle, _d(_dx3(dx)), int(nsteps), _d(ms)))
        names = PHASES_MIXED if self._p.precision == 1 else PHASES
        out = dict(zip(names, ms.tolist()))
        if self._p.precision == 1 and out["sweep_y"] < 0:
            # the x and y sweeps ran as one kernel
            out = {"cfl": out["cfl"], "ghost_fill": out["ghost_fill"], "sweep_xy": out["sweep_x"],
                   "sweep_z": out["sweep_z"]}
        return out

    # ---- element-level interfaces --------------------------------------
    def riemann_problem_solve(self, l, r, dx, dt, axis):
        l, r = _f64(l), _f64(r)
        u = np.zeros_like(l)
        self._check(self.lib.rhyme_gpu_riemann_solve(self.h, _d(l), _d(r), l.shape[0], float(dx),
                                                     float(dt), int(axis), _d(u)))
        return u

    def irs_exec(self, states):
        states = _f64(states)
        out = np.zeros((states.shape[0], 3))
        self._check(self.lib.rhyme_gpu_irs_exec(self.h, _d(states), states.shape[0], _d(out)))
        return out

    def slope_limiter_run(self, ul, u, ur):
        ul, u, ur = _f64(ul), _f64(u), _f64(ur)
        d = np.zeros_like(u)
        self._check(self.lib.rhyme_gpu_slope_limiter(self.h, _d(ul), _d(u), _d(ur), u.shape[0], _d(d)))
        return d

    def half_step_extrapolation(self, u, delta, axis, dx, dt):
        u, delta = _f64(u), _f64(delta)
        l = np.zeros_like(u)
        r = np.zeros_like(u)
        self._check(self.lib.rhyme_gpu_half_step(self.h, _d(u), _d(delta), u.shape[0], int(axis),
                                                 float(dx), float(dt), _d(l), _d(r)))
        return l, r


class Server:
    """rhyme_gpu_server: continuous batching of hydro solves.

    base: gas / Riemann / precision parameters (hydro_params mapping);
    courant: Courant number per dimensionality (1-D, 2-D, 3-D).
    """

    def __init__(self, base, courant=(0.8, 0.5, 0.3), hbm_budget=150 << 30, max_active=256):
        self.lib = load()
        self._p = params_struct(base)
        cr = np.asarray(courant, dtype=np.float64)
        h = C.c_void_p()
        rc = self.lib.rhyme_gpu_server_create(C.byref(self._p), _d(cr), int(hbm_budget), int(max_active),
                                              C.byref(h))
        if rc != OK:
            raise RhymeGpuError(rc, "rhyme_gpu_server_create failed")
        self.h = h
        self._keep = {}

    def _check(self, rc):
        if rc != OK:
            raise RhymeGpuError(rc, self.lib.rhyme_gpu_server_last_error(self.h).decode())

    def submit(self, cells, nsteps, dx, limiter, bc, omega=0.0, output=None, shapes=None):
        """Queue one solve; `cells` (NDIM+2, ...) receives the result and, if
        given, `output` (float32, (NDIM+2) x interior cells) the result in the
        Chombo level-data layout; with `shapes` (rhyme_gb300.drawing) the
        initial state is painted on the device instead of uploaded."""
        assert cells.dtype == np.float64 and cells.flags.c_contiguous
        r = Request()
        nd = cells.ndim - 1
        r.ndim = nd
        ext = cells.shape[1:][::-1]
        for a in range(3):
            r.dims[a] = ext[a] - 4 if a < nd else 1
            r.dx[a] = dx[a] if a < len(dx) else 1.0
        r.nsteps = int(nsteps)
        r.limiter = int(limiter)
        for i in range(6):
            r.bc[i] = int(bc[i]) if i < len(bc) else 2
        r.omega = float(omega)
        r.cells = _d(cells)
        if output is not None:
            assert output.dtype == np.float32 and output.flags.c_contiguous
            assert output.size == (nd + 2) * int(np.prod([r.dims[a] for a in range(nd)]))
            r.output = output.ctypes.data_as(C.POINTER(C.c_float))
        arr = None
        if shapes:
            arr = (Shape * len(shapes))(*shapes)
            r.shapes = C.cast(arr, C.POINTER(Shape))
            r.nshapes = len(shapes)
        rid = C.c_int()
        self._check(self.lib.rhyme_gpu_server_submit(self.h, C.byref(r), C.byref(rid)))
        self._keep[rid.value] = (cells, output)
        return rid.value

    def tick(self):
        a, p, d = C.c_int(), C.c_int(), C.c_int()
        self._check(self.lib.rhyme_gpu_server_tick(self.h, C.byref(a), C.byref(p), C.byref(d)))
        return a.value, p.value, d.value

    def request(self, rid):
        st = C.c_int()
        t = np.zeros(3)
        n = C.c_int()
        self._check(self.lib.rhyme_gpu_server_request(self.h, int(rid), C.byref(st), _d(t), C.byref(n)))
        return st.value, t, n.value

    def stats(self):
        cu, used = C.c_longlong(), C.c_longlong()
        self._check(self.lib.rhyme_gpu_server_stats(self.h, C.byref(cu), C.byref(used)))
        return cu.value, used.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.rhyme_gpu_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def tma_launches():
    """Single-box sweep launches of this process that staged with TMA."""
    n = C.c_longlong()
    rc = load().rhyme_gpu_tma_launches(C.byref(n))
    if rc != OK:
        raise RhymeGpuError(rc, "rhyme_gpu_tma_launches")
    return n.value


RATE_KINDS = ["fp64_fma_flops", "fp64_div", "fp64_sqrt", "fp64_pow", "fp32_fma_flops", "fp32_div_approx",
              "fp32_pow_exp2_log2", "fp64_add", "fp64_fp32_conversions"]


def check_conversions(n, seed=0):
    """Mismatches of the integer FP64 <-> FP32 conversions of the mixed state
    update against the hardware conversions over n values
    (rhyme_gpu_check_conversions)."""
    bad = C.c_ulonglong()
    rc = load().rhyme_gpu_check_conversions(int(n), int(seed), C.byref(bad))
    if rc != OK:
        raise RhymeGpuError(rc, "rhyme_gpu_check_conversions")
    return bad.value


def rate_probe(kind, iters=2000):
    """(operations per second, ms) of one probe kind (rhyme_gpu_rate_probe)."""
    r, ms = C.c_double(), C.c_double()
    rc = load().rhyme_gpu_rate_probe(int(kind), int(iters), C.byref(r), C.byref(ms))
    if rc != OK:
        raise RhymeGpuError(rc, "rhyme_gpu_rate_probe")
    return r.value, ms.value
