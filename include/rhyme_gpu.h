/*
 * rhyme_gpu.h -- C-ABI of the GB300 (sm_103a) MUSCL-Hancock hydro step for
 * Rhyme SAMR boxes.
 *
 * The Fortran driver (src/main.f90) reaches these entry points through a thin
 * ISO_C_BINDING shim that keeps Rhyme's module interfaces; each declaration
 * names the reference interface it replaces (paths relative to Rhyme's src/).
 *
 * Conventions
 *  - Every function returns 0 (RHYME_GPU_OK) or a negative RHYME_GPU_E* code;
 *    rhyme_gpu_last_error() gives the message of the last failure on a
 *    context. The reference has no error returns (it calls logger%err and
 *    goes on, rhyme_muscl_hancock_solve.f90:24-26); the shim maps a non-zero
 *    code to logger%err.
 *  - A box's `cells` is the caller's Fortran array
 *    cells(-1:N1+2, -1:N2+2, -1:N3+2, 1:NCMP) (rhyme_samr_init_box.f90:29-33),
 *    column-major and contiguous, ghost width 2 on every active axis
 *    (rhyme_initial_condition_init_simple.f90:31). The library mirrors the
 *    hydro components 1..NDIM+2 (rho, rho*u[, rho*v[, rho*w]], e_tot;
 *    rhyme_units.f90:32-36) on the device and never frees the host array.
 *    Axes beyond NDIM have dims 1 and no ghosts.
 *  - Between rhyme_gpu_sync_to_device and rhyme_gpu_sync_to_host the device
 *    copy is authoritative.
 *  - Axis arguments are 0-based (x = 0); the Fortran shim subtracts one.
 *  - One context is used by one host thread at a time; it owns one CUDA
 *    stream, on which every call below is ordered.
 */
#ifndef RHYME_GPU_H
#define RHYME_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RHYME_GPU_ABI_VERSION 1

enum {
  RHYME_GPU_OK = 0,
  RHYME_GPU_EINVAL = -1,     /* bad argument or unsupported parameter */
  RHYME_GPU_ENOMEM = -2,     /* device or pinned allocation failed */
  RHYME_GPU_ECUDA = -3,      /* a CUDA runtime call failed */
  RHYME_GPU_ETIMEDOUT = -4,  /* a bounded host wait ran out */
  RHYME_GPU_ENANSTATE = -5,  /* the state holds NaN/Inf or non-positive rho */
  RHYME_GPU_ENOTFOUND = -6   /* unknown box handle */
};

/* Slope limiter ids: slid, rhyme_slope_limiter.f90:6-10. */
enum { RHYME_GPU_VAN_LEER = 1, RHYME_GPU_MINMOD = 2, RHYME_GPU_VAN_ALBADA = 3,
       RHYME_GPU_SUPERBEE = 4 };
/* Boundary ids: bcid, rhyme_samr_bc.f90:9-12. RHYME_GPU_HALO (no reference
 * counterpart) leaves the face to the caller: the face of a slab of a box
 * decomposed along its outermost axis, whose two ghost rows the caller
 * copies from the neighbouring slab (rhyme_gpu_get_rows / _set_rows). */
enum { RHYME_GPU_REFLECTIVE = 1, RHYME_GPU_OUTFLOW = 2, RHYME_GPU_PERIODIC = 3,
       RHYME_GPU_INFLOW = 4, RHYME_GPU_HALO = 5 };
/* Solver ids: mhid, rhyme_muscl_hancock.f90:10-15. */
enum { RHYME_GPU_CPU_INTENSIVE = 1, RHYME_GPU_MEMORY_INTENSIVE = 2 };
/* Arithmetic of the step (this library): FP64 throughout, or FP32
 * reconstruction / Riemann / flux with FP64 state accumulation and an FP64
 * Riemann fallback near vacuum or where the FP32 Newton iteration fails. */
enum { RHYME_GPU_FP64 = 0, RHYME_GPU_MIXED = 1 };

/*
 * Tile shapes of the mixed-precision sweeps (no reference counterpart):
 * TUNE_AUTO times the candidate shapes (cells along the sweep axis x
 * pencils: 8x32, 16x16, 32x8, 64x4; 64..512 cells in 1-D) on the first box
 * of each box-size class a context meets and keeps the fastest per class;
 * TUNE_FIXED uses a size rule without timing launches. Results do not
 * depend on the shape. Ignored in FP64 mode.
 */
enum { RHYME_GPU_TUNE_AUTO = 0, RHYME_GPU_TUNE_FIXED = 1 };

/*
 * Run parameters: the values Rhyme's modules hold after load_params
 * (rhyme_param_parser_load_params.f90: BCs :259-293, courant :307, gas :314,
 * Riemann :493-499, limiter :512-513, solver :523) and rhyme_*_init.
 */
typedef struct rhyme_gpu_params {
  int ndim;          /* NDIM (1, 2 or 3) */
  int limiter;       /* sl%type */
  int n_iteration;   /* rp%irs%n_iteration */
  int solver_type;   /* mh%solver_type */
  int bc[6];         /* bc%types(left, right, bottom, top, back, front) */
  int precision;     /* RHYME_GPU_FP64 or RHYME_GPU_MIXED */
  int sweep_tuning;  /* RHYME_GPU_TUNE_AUTO (0) or RHYME_GPU_TUNE_FIXED (1) */
  double gamma;      /* get_gamma(), rhyme_thermo_base_get_gamma.f90:8-19 */
  double kb_amu;     /* units%kb%v / units%amu%v, rhyme_thermo_base.f90:130 */
  double courant;    /* cfl%courant_number */
  double omega;      /* sl%w */
  double vacuum_density;   /* rp%w_vacuum(cid%rho) */
  double vacuum_pressure;  /* rp%w_vacuum(cid%p) */
  double tolerance;        /* rp%irs%tolerance */
  double inflow[6][5];     /* bc%cons_inflows(rho:e_tot, side) for inflow faces */
} rhyme_gpu_params;

typedef struct rhyme_gpu_ctx rhyme_gpu_ctx;

/* ABI version of the loaded library (RHYME_GPU_ABI_VERSION). */
int rhyme_gpu_abi_version(void);

/*
 * Creates a context on the current CUDA device with the run parameters.
 * Replaces the module set-up of rhyme_riemann_problem_init
 * (rhyme_riemann_problem.f90:64-69, rhyme_riemann_problem_init.f90:20-27),
 * rhyme_irs_init (rhyme_irs_init.f90:21-27), rhyme_muscl_hancock_init
 * (rhyme_muscl_hancock.f90:22-27), rhyme_cfl_init (rhyme_cfl.f90:12-17) and
 * rhyme_samr_bc_init (rhyme_samr_bc.f90:31-36).
 */
int rhyme_gpu_create(rhyme_gpu_ctx** ctx, const rhyme_gpu_params* params);
int rhyme_gpu_destroy(rhyme_gpu_ctx* ctx);

/* Message of the last failure on ctx ("" if none). */
const char* rhyme_gpu_last_error(const rhyme_gpu_ctx* ctx);

/* The cudaStream_t (as void*) every call on ctx is ordered on. */
int rhyme_gpu_get_stream(rhyme_gpu_ctx* ctx, void** stream);

/*
 * Registers one SAMR box (samr%levels(level)%boxes(number)); allocates its
 * device mirror and uploads the hydro components. ghost must be 2, ncmp >= NDIM+2.
 * Replaces the lazy per-box workspace of rhyme_mh_workspace_check
 * (rhyme_mh_workspace_check.f90:36-77); the device holds two state buffers
 * and no per-box workspace beyond the solver's scratch.
 */
int rhyme_gpu_register_box(rhyme_gpu_ctx* ctx, int level, int number,
                           double* cells, const int dims[3], int ghost,
                           int ncmp, int* handle);
int rhyme_gpu_unregister_box(rhyme_gpu_ctx* ctx, int handle);

/* Host -> device copy of the hydro components (and ghosts) of a box.
 * Asynchronous: the array the library page-locked at registration must
 * not be written until a later call waits on the context stream (every
 * call that returns a value does). For a 2-D or 3-D box in mixed precision
 * of 16 MiB or more the copy runs in slabs of rows of the outermost axis,
 * each slab's share of the CFL maximum taken while the next one is in
 * flight, and the next rhyme_gpu_cfl_time_step only forms dt from it. */
int rhyme_gpu_sync_to_device(rhyme_gpu_ctx* ctx, int handle);
/* Device -> host copy into the registered cells array; waits for the stream
 * (bounded wait, RHYME_GPU_ETIMEDOUT). With host write-back on, the last
 * solve's copies are already in flight and this only waits for them. */
int rhyme_gpu_sync_to_host(rhyme_gpu_ctx* ctx, int handle);

/*
 * Host write-back (default off). With on != 0 every rhyme_gpu_mh_solve of
 * the box also copies the new state into the registered cells array: the
 * drop-in mode, in which the shim's rhyme_muscl_hancock_solve returns with
 * box%cells current (the reference updates box%cells in place,
 * rhyme_muscl_hancock_solve_memory_intensive.f90:148-179), for the host
 * readers of src/main.f90:122-155. For a box whose upload runs in slabs
 * (rhyme_gpu_sync_to_device) the solve runs in slabs of rows as well and
 * each slab's finished rows are copied while the next slab is solved;
 * otherwise one copy follows the solve. The array is being written until
 * rhyme_gpu_sync_to_host or rhyme_gpu_synchronize returns.
 */
int rhyme_gpu_set_host_writeback(rhyme_gpu_ctx* ctx, int handle, int on);

/*
 * Rows [row0, row0 + nrows) of the box's outermost axis (rows of the
 * ghosted block: 0 and 1 are the left ghosts, 2 .. N+1 the interior) of the
 * hydro components, copied into out: NDIM+2 component blocks of nrows rows
 * each, a row being the ghosted extent of the other axes. out may be host
 * memory or device memory (this GPU's, or a peer's with peer access), so a
 * multi-GPU exchange can keep the rows on the devices. Waits.
 * With rhyme_gpu_set_rows, the halo exchange of a box decomposed into slabs
 * along its outermost axis (one slab per GPU): each slab sends its first and
 * last two interior rows to the neighbours' ghost rows, whose faces have the
 * RHYME_GPU_HALO boundary type, after the ghost fill and before the solve;
 * dt is the minimum of the slabs' dt, which equals the whole box's dt since
 * dt = RN(courant minval(dx) / max) is monotone in the maximum. No reference
 * counterpart (the reference steps one box per process).
 */
int rhyme_gpu_get_rows(rhyme_gpu_ctx* ctx, int handle, int row0, int nrows, double* out);
/* The same rows from `in` (host or device memory), into both state buffers
 * of the box. */
int rhyme_gpu_set_rows(rhyme_gpu_ctx* ctx, int handle, int row0, int nrows, const double* in);

/*
 * Reads and clears the box's status word (no reference counterpart: the
 * reference only logs, rhyme_sanity_check_perform.f90:34-63). Bit 0 is set
 * when a CFL pass met a cell with non-positive density or a non-finite
 * signal speed; such cells are skipped by the dt maximum exactly as the
 * reference's `if (u > max_u)` skips them, and the run goes on. Returns
 * RHYME_GPU_ENANSTATE when a bit is set, RHYME_GPU_OK otherwise.
 */
int rhyme_gpu_box_status(rhyme_gpu_ctx* ctx, int handle, int* flags);

/*
 * dt = courant * minval(dx) / max(|v| + cs) over the box interior.
 * Replaces pure function rhyme_cfl_time_step(c, samr)
 * (rhyme_cfl.f90:19-23, rhyme_cfl_time_step.f90:63-84). Waits for the result.
 */
int rhyme_gpu_cfl_time_step(rhyme_gpu_ctx* ctx, int handle, const double dx[3],
                            double* dt);

/*
 * The same time step returned as the function value (a negative value on
 * error, message in rhyme_gpu_last_error), for Fortran callers that must
 * call it from the pure rhyme_cfl_time_step (rhyme_cfl.f90:19-23): a pure
 * Fortran function cannot take an intent(out) argument.
 */
double rhyme_gpu_cfl_dt(rhyme_gpu_ctx* ctx, int handle, const double dx[3]);

/*
 * Ghost fill of the 2-cell face slabs (corners untouched) with the context's
 * boundary types. Replaces pure subroutine rhyme_samr_bc_set_boundaries
 * (rhyme_samr_bc.f90:38-41, rhyme_samr_bc_set_boundaries.f90:9-20).
 */
int rhyme_gpu_set_boundaries(rhyme_gpu_ctx* ctx, int handle);

/*
 * One unsplit MUSCL-Hancock update of the box interior with time step dt.
 * Replaces rhyme_muscl_hancock_solve (rhyme_muscl_hancock.f90:47-56,
 * rhyme_muscl_hancock_solve.f90:3-30) and, by solver_type, its
 * memory-intensive (rhyme_muscl_hancock_solve_memory_intensive.f90:3-181)
 * and cpu-intensive (rhyme_muscl_hancock_solve_cpu_intensive.f90:3-159)
 * forms. Asynchronous on the context stream.
 */
int rhyme_gpu_mh_solve(rhyme_gpu_ctx* ctx, int handle, const double dx[3],
                       double dt);

/*
 * nsteps iterations of the driver's loop body (src/main.f90:109-136):
 * dt from the state, ghost fill, solve, with dt kept on the device. The
 * step is captured once in a CUDA graph and replayed. dt_trace (optional,
 * host, nsteps entries) receives each dt. Leaves the state on the device.
 */
int rhyme_gpu_run(rhyme_gpu_ctx* ctx, int handle, const double dx[3],
                  int nsteps, double* dt_trace);

/*
 * Instrumentation (no reference counterpart): runs nsteps driver steps with
 * direct launches and CUDA events between the library's kernels on the
 * context stream; ms[5] receives the mean milliseconds per launch of the
 * phases cfl, ghost_fill, faces, fluxes, update (RHYME_GPU_FP64) or cfl,
 * ghost_fill, sweep_x, sweep_y, sweep_z (RHYME_GPU_MIXED; the last one that
 * runs includes the FP64 fix-up, absent axes read 0; in a 3-D box whose x
 * and y sweeps ran as one kernel, ms[2] is that kernel and ms[3] is -1).
 * The state advances nsteps steps exactly as rhyme_gpu_run would advance
 * it.
 */
int rhyme_gpu_profile_steps(rhyme_gpu_ctx* ctx, int handle, const double dx[3],
                            int nsteps, double ms[5]);

/*
 * Instrumentation (no reference counterpart): number of interfaces of the
 * box that the mixed-precision solver redid with the FP64 Riemann solver
 * since the last query (0 in FP64 mode); clears the counter.
 */
int rhyme_gpu_fallback_count(rhyme_gpu_ctx* ctx, int handle, long long* count);

/*
 * Chombo output drain: replaces the packing loop of
 * rhyme_chombo_write_level_data.f90:36-70 for the hydro components. Packs
 * the interior cells of the listed boxes (their current state), box after
 * box and component after component, in Fortran order and converted to
 * FP32, into `data` in the layout of the level's "data:datatype=0" dataset:
 * box b starts at sum over the boxes before it of prod(dims) * ncmp, its
 * component c at + c * prod(dims). Only components 1..NDIM+2 are written;
 * the blocks of the other ncmp - NDIM - 2 components (temperature, species
 * fractions, which stay on the host) are left untouched. Asynchronous: the
 * pack runs after the work already queued on the context's stream and the
 * copy on a copy stream; `data` (capacity in floats) must stay valid until
 * rhyme_gpu_output_wait returns (page-locked memory keeps the copy off the
 * host's critical path). A second output waits for the first.
 */
int rhyme_gpu_output_level(rhyme_gpu_ctx* ctx, const int* handles, int n, int ncmp, float* data,
                           long long capacity);
int rhyme_gpu_output_wait(rhyme_gpu_ctx* ctx);

/*
 * Conservation totals, rhyme_samr_calc_total_mass.f90 and
 * rhyme_samr_calc_total_energy.f90 on the device: totals[0] = sum of rho
 * where rho > 0 and totals[1] = sum of e_tot where e_tot > 0 over every
 * cell of the box, ghosts included (the reference then multiplies by
 * product(box_lengths)). Summed in double-double and rounded once.
 */
int rhyme_gpu_box_totals(rhyme_gpu_ctx* ctx, int handle, double totals[2]);

/*
 * Sanity checks on the device: the general checks of
 * rhyme_sanity_check_perform.f90:34-90 and the property statistics of
 * rhyme_sanity_check_fill.f90:75-185 for the properties that live on the
 * device (rho, vx, vy, vz, e_tot, |v|, Mach), over the interior cells.
 * Per property: in range[2] and enabled (sc%<p>_range, sc%properties);
 * out the counts below / above the range, the lowest value below it and
 * the highest above it with their first 1-based cells in Fortran loop
 * order, and the running extreme the loop held just before reaching them
 * (the reference's vbelow(1) / vabove(1) within this call; +-DBL_MAX when
 * none). The reference keeps vbelow/vabove across calls; a caller merges
 * with its kept values (a new extreme replaces them only if beyond them).
 * Mach is |v| / cs of the cell's own state (the reference passes the slice
 * rho_u:e_tot to calc_cs, which reads one component past it).
 */
enum { RHYME_GPU_SC_RHO = 0, RHYME_GPU_SC_VX, RHYME_GPU_SC_VY, RHYME_GPU_SC_VZ, RHYME_GPU_SC_E_TOT,
       RHYME_GPU_SC_ABS_V, RHYME_GPU_SC_MACH, RHYME_GPU_SC_COUNT };

typedef struct rhyme_gpu_sanity_property {
  double range[2];
  int enabled;
  int reserved;
  long long nbelow, nabove;
  double vbelow, vbelow_prev;
  double vabove, vabove_prev;
  int cbelow[3], cabove[3];
} rhyme_gpu_sanity_property;

typedef struct rhyme_gpu_sanity_report {
  rhyme_gpu_sanity_property prop[RHYME_GPU_SC_COUNT];
  int nan[5];          /* a NaN in component c (rho, rho_u, [rho_v, [rho_w,]] e_tot) */
  int reserved;
  double rho_min, e_tot_min;           /* minval over the interior (negative: the warnings) */
  int rho_min_at[3], e_tot_min_at[3];  /* minloc, 1-based */
} rhyme_gpu_sanity_report;

int rhyme_gpu_sanity_check(rhyme_gpu_ctx* ctx, int handle, rhyme_gpu_sanity_report* report);

/*
 * Initial conditions painted on the device: the hydro part of
 * rhyme_drawing_init.f90:20-78. The shapes are applied in order (a canvas
 * or shape overwrites the cells it covers; without a canvas the cells keep
 * their values, the reference's transparent canvas), then every perturbation
 * is summed per cell and added once as a conserved vector
 * (rhyme_drawing_apply_perturbations.f90). Colours and bases are primitive
 * (rho, u, v, w, p); lengths are in level-0 cells. A sphere blends its two
 * colours over every cell of the box, as the reference does, so a second
 * sphere repaints the first one's outside. Extensions, off when 0:
 * `periodic` (a sphere also covers the box's periodic images), sigma = 0 for
 * a sphere (sharp edge, dist < r), `keep_outside` (a sharp sphere leaves the
 * cells outside it alone, so several spheres can be drawn), `phase` (of a
 * harmonic). Not painted on
 * the device: the power-law canvas, smooth cuboids, prisms and white noise
 * (the reference draws it from the Fortran generator).
 */
enum { RHYME_GPU_DRAW_CANVAS = 0, RHYME_GPU_DRAW_SHARP_CUBOID = 1, RHYME_GPU_DRAW_SPHERE = 2,
       RHYME_GPU_DRAW_SMOOTHED_SLAB = 3, RHYME_GPU_DRAW_HARMONIC = 4, RHYME_GPU_DRAW_SYMMETRIC_DECAYING = 5 };

typedef struct rhyme_gpu_shape {
  int type;            /* RHYME_GPU_DRAW_* */
  int axis;            /* slab / perturbation axis (0 = x) */
  int periodic;        /* sphere: nearest periodic image */
  int keep_outside;    /* sharp sphere: cells outside keep their values */
  int left_corner[3];  /* sharp cuboid: shape%cuboid%left_corner, lengths */
  int lengths[3];
  double prim[2][5];   /* colours: [0] canvas, cuboid, sphere inside, slab outside;
                          [1] sphere outside, slab inside */
  double origin[3];    /* sphere centre (cells) */
  double r, sigma;     /* sphere radius and tanh width; symmetric decaying: sigma */
  double pos[2];       /* slab edges; symmetric decaying: pos[0] */
  double slab_sigma[2];
  double amplitude, wavelength, phase;  /* perturbation A, lambda (cells), phase */
  double base[5];      /* perturbation base */
} rhyme_gpu_shape;

/* left_edge: the box's left edge in level-0 cells (1 for a single box). */
int rhyme_gpu_paint(rhyme_gpu_ctx* ctx, int handle, const int left_edge[3], const rhyme_gpu_shape* shapes,
                    int n);

/*
 * Instrumentation (no reference counterpart): the tile shape of each axis of
 * the box's mixed-precision sweeps (cells along the axis, pencils), as the
 * autotuner or the size rule chose it; tunes the box's size classes first
 * if needed (dx: cell size used for the timing launches). Zeros for absent
 * axes and in FP64 mode.
 */
int rhyme_gpu_sweep_plan(rhyme_gpu_ctx* ctx, int handle, const double dx[3], int tile_cells[3],
                         int tile_pencils[3]);

/*
 * Instrumentation (no reference counterpart): how many single-box sweep
 * launches of this process staged their slabs with TMA tensor copies
 * (2-/3-D boxes whose x extent plus ghosts is a multiple of 4 cells; the
 * others, and every launch with RHYME_GPU_TMA=0 in the environment, stage
 * with coalesced loads and give the same results).
 */
int rhyme_gpu_tma_launches(long long* n);

/*
 * Instrumentation (no reference counterpart): arithmetic rate of the current
 * GPU for the operations this path is bound by, from `iters` iterations of 8
 * independent chains per thread on 8 CTAs of 256 threads per SM (the fastest
 * of three timed launches after one warm-up; CUDA events). kind: 0 FP64 FMA
 * (2 flops each), 1 FP64 division, 2 FP64 square root, 3 FP64 power (the
 * restated C-library pow), 4 FP32 FMA (2 flops), 5 FP32 approximate
 * division, 6 FP32 power as exp2f(y log2f(x)), 7 FP64 add, 8 FP64 -> FP32
 * -> FP64 conversions (2 each). *ops_per_second: operations per second;
 * *ms (optional): the timed launch.
 */
int rhyme_gpu_rate_probe(int kind, int iters, double* ops_per_second, double* ms);

/*
 * Instrumentation (no reference counterpart): checks the integer forms of
 * the FP64 <-> FP32 conversions of the mixed state update against the
 * hardware conversions on n pseudo-random values from `seed` (doubles of
 * every exponent, FP32 rounding ties and range limits, FP32 values).
 * *mismatches: the number that differ (0 expected).
 */
int rhyme_gpu_check_conversions(long long n, unsigned long long seed, unsigned long long* mismatches);

/*
 * No counterpart in the reference: one plain-FP64 MUSCL-Hancock update
 * (the same kernels as rhyme_gpu_mh_solve) that allocates nothing, for
 * callers that cannot allocate device memory: hosts whose device arrays come
 * from their own pool or from a Fortran runtime (CUDA Fortran, OpenACC) and
 * that keep all device allocations under their own control, or runs under a
 * fixed device-memory budget where an allocation in the middle of a step
 * could fail or synchronize the device.
 *
 *  - d_cells_in / d_cells_out: device pointers to the NDIM+2 hydro component
 *    blocks of the box in the layout of rhyme_gpu_register_box, ghosts of
 *    d_cells_in already filled. The interior of d_cells_out receives U^{n+1};
 *    its ghosts are not written. The two arrays must not overlap (an
 *    in-place call is rejected with RHYME_GPU_EINVAL).
 *  - params->precision must be RHYME_GPU_FP64.
 *  - Scratch: a fixed device array of RHYME_GPU_NOALLOC_SCRATCH_DOUBLES
 *    doubles (16 MiB) inside this library, which every GPU that loads the
 *    library holds until the process exits. A box needs
 *    32 + 3*NDIM*(NDIM+2)*prod(N_a + 4) doubles (at most a 2-D 291^2 box
 *    or a 3-D 31^3 box); larger boxes are rejected with RHYME_GPU_EINVAL and a
 *    message on stderr.
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current; make that first call
 *    before any stream capture.
 *  - All calls on a device share the array: calls whose work overlaps on the
 *    GPU (different streams, no ordering between them) race. Nothing in the
 *    array needs clearing between calls.
 *  - stream: the cudaStream_t to launch on (NULL: the default stream).
 *    Asynchronous; errors of the launch are returned, not of the kernels.
 */
#define RHYME_GPU_NOALLOC_SCRATCH_DOUBLES (2LL * 1024 * 1024)
int rhyme_gpu_mh_solve_noalloc(const rhyme_gpu_params* params,
                               const double* d_cells_in, double* d_cells_out,
                               const int dims[3], const double dx[3], double dt,
                               void* stream);

/* ---- batches of independent boxes -------------------------------------
 * Steps many boxes of uneven sizes together, each with its own dt, boundary
 * types, limiter and cell size, through one persistent kernel per pass fed
 * by a work queue, one CUDA graph per step. Rhyme's driver steps only box 1
 * of level 0 (rhyme_cfl_time_step.f90:42-49, rhyme_samr_bc_set_boundaries.f90:
 * 9-20) and calls rhyme_muscl_hancock_solve once per box
 * (src/main.f90:130-136); a batch runs that loop body for every box at once.
 * A box stepped in a batch gives the same state and dt as stepped alone.
 */
typedef struct rhyme_gpu_batch rhyme_gpu_batch;

/* Per-box boundary types (bc may be NULL to keep the context's), limiter id
 * and omega, overriding the context's for this box in every call. */
int rhyme_gpu_set_box_params(rhyme_gpu_ctx* ctx, int handle, const int bc[6],
                             int limiter, double omega);

/* A batch of n registered boxes; dx[3*i .. 3*i+2] is box i's cell size. */
int rhyme_gpu_batch_create(rhyme_gpu_ctx* ctx, const int* handles,
                           const double* dx, int n, rhyme_gpu_batch** batch);
/* nsteps driver steps of every box of the batch (asynchronous). */
int rhyme_gpu_batch_run(rhyme_gpu_batch* batch, int nsteps);
/* dts[i] = the dt of box i's last step (waits for the stream). */
int rhyme_gpu_batch_dt(rhyme_gpu_batch* batch, double* dts);
int rhyme_gpu_batch_destroy(rhyme_gpu_batch* batch);

/* ---- serving: continuous batching of hydro solves (no reference
 * counterpart; the reference runs one solve per process) ------------------
 * Requests of any dimensionality and size are submitted as they arrive;
 * each tick admits pending requests first come first served while the HBM
 * budget and the active-request cap allow, advances every active request by
 * one step (one batch per dimensionality, each on its own stream, so their
 * work overlaps on the device) and retires finished ones: their state is
 * downloaded asynchronously on a copy stream through page-locked staging and
 * copied into the request's cells array when the copy completes.
 */
enum { RHYME_GPU_REQ_PENDING = 0, RHYME_GPU_REQ_ACTIVE = 1,
       RHYME_GPU_REQ_DRAINING = 2, RHYME_GPU_REQ_DONE = 3 };

typedef struct rhyme_gpu_request {
  int ndim;
  int dims[3];
  int nsteps;
  int limiter;
  int bc[6];
  double omega;
  double dx[3];
  double* cells;  /* host, NDIM+2 ghosted blocks: initial state in, result out */
  float* output;  /* optional (NULL): the result as a one-box level output in the
                     Chombo "data:datatype=0" layout (FP32, NDIM+2 components,
                     interior cells), drained like rhyme_gpu_output_level */
  const struct rhyme_gpu_shape* shapes;  /* optional: paint the initial state on the
                                            device (rhyme_gpu_paint, from zero cells)
                                            instead of uploading `cells` */
  int nshapes;
  int reserved;
} rhyme_gpu_request;

typedef struct rhyme_gpu_server rhyme_gpu_server;

/* base: gas, Riemann, precision (ndim, limiter, bc ignored); courant[k] is
 * the Courant number of (k+1)-D requests. */
int rhyme_gpu_server_create(const rhyme_gpu_params* base, const double courant[3],
                            long long hbm_budget_bytes, int max_active,
                            rhyme_gpu_server** server);
int rhyme_gpu_server_submit(rhyme_gpu_server* server, const rhyme_gpu_request* req, int* id);
/* One tick: finished downloads land in the callers' arrays, pending requests
 * are admitted in arrival order against the budget and the active cap, then
 * every active request advances by the same number of steps (as many as the
 * request nearest to completion still needs, 1 to 8; a batch whose
 * membership has not changed since its last tick replays CUDA graphs), and
 * finished requests start their download. */
int rhyme_gpu_server_tick(rhyme_gpu_server* server, int* n_active, int* n_pending,
                          int* n_draining);
/* state (RHYME_GPU_REQ_*), times = (submitted, admitted, done) in seconds
 * since the server started, steps taken. */
int rhyme_gpu_server_request(rhyme_gpu_server* server, int id, int* state, double times[3],
                             int* steps_done);
int rhyme_gpu_server_stats(rhyme_gpu_server* server, long long* cell_updates,
                           long long* hbm_used);
const char* rhyme_gpu_server_last_error(const rhyme_gpu_server* server);
int rhyme_gpu_server_destroy(rhyme_gpu_server* server);

/* Waits (bounded) for all work on the context stream. */
int rhyme_gpu_synchronize(rhyme_gpu_ctx* ctx);

/* ---- element-level entry points (host arrays in and out) ----------------
 * These run the same device functions as the box solver over n independent
 * inputs, for the Fortran interfaces Rhyme's unit tests call directly.
 * State rows are (rho, rho*u.., e_tot), NDIM+2 doubles each.
 */

/* rhyme_riemann_problem_solve(rp, l, r, dx, dt, axis, u) for n pairs
 * (rhyme_riemann_problem.f90:71-77, rhyme_riemann_problem_solve.f90:3-104). */
int rhyme_gpu_riemann_solve(rhyme_gpu_ctx* ctx, const double* l,
                            const double* r, long long n, double dx,
                            double dt, int axis, double* u);

/* p* = rhyme_irs_exec(irs, l_rho, l_v, l_p, l_cs, l_f, r_rho, r_v, r_p, r_cs,
 * r_f, axis) (rhyme_irs.f90:22-30, rhyme_irs_exec.f90:3-45) for n rows
 * states[n][8] = (l_rho, l_v, l_p, l_cs, r_rho, r_v, r_p, r_cs), v being the
 * normal velocity; out[n][3] = (p*, l_f, r_f). */
int rhyme_gpu_irs_exec(rhyme_gpu_ctx* ctx, const double* states, long long n,
                       double* out);

/* rhyme_slope_limiter_run(sl, ul, u, ur, delta) for n rows
 * (rhyme_slope_limiter.f90:18-22, rhyme_slope_limiter_run.f90:3-20). */
int rhyme_gpu_slope_limiter(rhyme_gpu_ctx* ctx, const double* ul,
                            const double* u, const double* ur, long long n,
                            double* delta);

/* rhyme_muscl_hancock_half_step_extrapolation(u, delta, axis, dx, dt, l, r)
 * for n rows (rhyme_muscl_hancock.f90:58-64,
 * rhyme_muscl_hancock_half_step_extrapolation.f90:3-24). */
int rhyme_gpu_half_step(rhyme_gpu_ctx* ctx, const double* u,
                        const double* delta, long long n, int axis, double dx,
                        double dt, double* l, double* r);

#ifdef __cplusplus
}
#endif

#endif /* RHYME_GPU_H */
