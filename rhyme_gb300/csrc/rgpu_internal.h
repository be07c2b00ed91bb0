// rgpu_internal.h -- types shared by the kernels and the C-ABI layer.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "hydro.cuh"

namespace rgpu {

// Per-run parameters passed by value to every kernel.
struct DevParams {
  Gas<double> G;
  Rp<double> rp;
  int ndim;
  int limiter;
  double omega;
  int solver_type;
  int bc[6];
  double inflow[6][5];
  double courant;
};

// Parameters of the mixed-precision kernels: FP32 copies of the gas and
// Riemann constants (rounded from their FP64 values) plus the FP64 set for
// the fallback solver.
struct MixedParams {
  Gas<float> G;
  Rp<float> rp;
  Gas<double> G64;
  Rp<double> rp64;
  int ndim;
  int limiter;
  float omega;
  double omega64;
};

// One interface queued for the FP64 solver by a mixed sweep: its axis, the
// index along that axis of its left cell (0..N) and the offset of that cell.
// The fix-up redoes the whole interface (slopes, half step, Riemann problem)
// in FP64 from the FP64 state at the start of the step.
struct FallbackEntry {
  int axis;
  int ga;
  int box;  // index in the batch's box table (0 for a single box)
  int pad;
  long long o;
};

struct FallbackQueue {
  FallbackEntry* e;
  int* n;       // entries this step (reset before each step)
  int cap;
  int* status;  // bit 1: queue overflow
  int* total;   // running count of FP64 interfaces (statistics)
  // A sweep over a slab of a box sees the box from the slab's first row
  // (shifted pointers): its entries are shifted back by these.
  long long o_base = 0;
  int ga_base = 0;
};

// Tile shapes of the mixed sweeps, the autotuner's candidate set: S cells
// along the sweep axis x P pencils, S * P = 256 for 2-/3-D boxes; 1-D boxes
// have a single pencil.
constexpr int kSweepShapes = 4;

__host__ __device__ inline void sweep_shape(int ndim, int shape, int* S, int* P) {
  if (ndim == 1) {
    *S = 64 << shape;  // 64, 128, 256, 512
    *P = 1;
  } else {
    *S = 8 << shape;  // 8x32, 16x16, 32x8, 64x4
    *P = 256 / *S;
  }
}

// Shape used without tuning: the smallest tile S that covers the box along
// the axis, up to 32 along x (pencils stay 8 cells wide) and 16 along y and
// z (pencils along x stay 16 cells wide, for coalescing); 256 cells in 1-D.
inline int default_sweep_shape(int ndim, int axis, int nA) {
  if (ndim == 1) return 2;
  const int cap = (axis == 0) ? 2 : 1;
  int k = 0;
  while (k < cap && (8 << k) < nA) ++k;
  return k;
}

// Tile shape per axis of one box's mixed sweeps.
struct SweepPlan {
  int shape[3];
  int fuse_xy = 0;  // 3-D: the x and y sweeps as one kernel (sweep_xy_kernel) where it can run
};

// Geometry of one box in the reference layout: component blocks of
// `field` doubles, cell (i,j,k) (1-based interior, ghosts -1..N+2) at
// (i+1)*s0 + (j+1)*s1 + (k+1)*s2 for the active axes.
struct Geom {
  int n[3];          // interior cells per axis (1 beyond NDIM)
  long long s[3];    // element strides per axis
  long long field;   // elements per component block
  __host__ __device__ long long at(int D, int i, int j, int k) const {
    long long o = (long long)(i + 1) * s[0];
    if (D > 1) o += (long long)(j + 1) * s[1];
    if (D > 2) o += (long long)(k + 1) * s[2];
    return o;
  }
};

inline Geom make_geom(int D, const int* dims) {
  Geom g;
  int ext[3];
  for (int a = 0; a < 3; ++a) {
    g.n[a] = (a < D) ? dims[a] : 1;
    ext[a] = (a < D) ? dims[a] + 4 : 1;
  }
  g.s[0] = 1;
  g.s[1] = ext[0];
  g.s[2] = (long long)ext[0] * ext[1];
  g.field = g.s[2] * ext[2];
  return g;
}

// Device scratch of one box for the plain FP64 solver.
struct StepScratch {
  double* faces = nullptr;   // [D][2][D+2][field]: ul, ur per axis
  double* fluxes = nullptr;  // [D][D+2][field]
  double* dt = nullptr;      // current dt (device scalar)
  unsigned long long* max_bits = nullptr;  // CFL max, as bits (self-resetting)
  unsigned int* counter = nullptr;         // CFL finished-block counter (self-resetting)
  int* status = nullptr;                   // sticky status bits (1: NaN/Inf or rho <= 0)
  double* dt_trace = nullptr;              // optional device dt trace
  int* trace_pos = nullptr;                // next trace slot
  int trace_cap = 0;
};

struct Dx {
  double v[3];
  double min;    // minval(dx(1:NDIM))
  float inv_f[3];  // 1/dx in FP32 (the mixed sweeps' dt/dx = FP32(dt) * inv_f)
};

}  // namespace rgpu
struct rhyme_gpu_params;
namespace rgpu {
// The kernels' parameters from the C-ABI's (gas constants, Riemann and
// limiter settings, boundary types), in rhyme_gpu.cu.
void make_dev_params(const rhyme_gpu_params* p, DevParams* d);

// Launchers (kernels_box.cu). All asynchronous on `st`.
// *dst = v in stream order (a scalar from the host without a staging buffer).
cudaError_t launch_set_double(double* dst, double v, cudaStream_t st);
// Ghost fill of U, its values also written to U_mirror (the other state
// buffer) and, as FP32, to Uf (the mixed form's mirror) when given.
cudaError_t launch_ghost_fill(const DevParams& P, double* U, double* U_mirror, const Geom& g,
                              cudaStream_t st, float* Uf = nullptr);
cudaError_t launch_cfl(const DevParams& P, const double* U, const Geom& g, const Dx& dx,
                       const StepScratch& s, cudaStream_t st);
// ev (optional, 4 events): recorded before the face pass and after the face,
// flux and update passes, for phase timing.
cudaError_t launch_mh_solve(const DevParams& P, const double* U, double* Unew, const Geom& g,
                            const Dx& dx, const StepScratch& s, cudaStream_t st,
                            cudaEvent_t* ev = nullptr);
int max_cfl_blocks();

// A 4-D tensor map (x, y, z, component) of a box's FP32 mirror Uf whose
// copy box is the staged slab of a sweep along axis A with tiles of S cells
// by P pencils (kernels_mixed.cu). False where a tensor copy cannot be used:
// 1-D boxes, rows of the mirror not a multiple of 16 bytes, a slab larger
// than the array, the driver's encoder unavailable, or RHYME_GPU_TMA=0 in
// the environment. The sweeps then stage with coalesced loads (same
// results).
bool encode_mirror_map(CUtensorMap* out, const float* Uf, const Geom& g, int D, int A, int S, int P);

// The FP32 mirror of an FP64 state value: rounded to nearest, an FP32
// subnormal flushed to zero of the same sign. The FP32 units of the mixed
// form run with denormals flushed (-ftz=true) and the others do not; the
// explicit flush gives every unit that writes a mirror (CFL pass, carried
// pass, ghost fill, ingest, painting) the same bits.
__device__ __forceinline__ float mirror_of(double x) {
  const float f = __double2float_rn(x);
  return (fabsf(f) < FLT_MIN) ? copysignf(0.f, f) : f;
}

// FP32 <-> FP64 conversions of the state update by integer operations. The
// FP64 pipe of GB300 converts at the rate of its FP64 adds, about 1/70 of
// the FP32 rate; the last sweep converts each component twice per cell.
// widen_f32: exact; an FP32 zero or subnormal (never formed: -ftz) gives a
// zero of the same sign, an infinity an infinity, a NaN a quiet NaN with the
// payload moved up. No path through the FP64 pipe.
__device__ __forceinline__ double widen_f32(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned mag = b & 0x7fffffffu;
  const unsigned sign = b & 0x80000000u;
  unsigned hi, lo;
  if (mag >= 0x7f800000u) {  // infinity, NaN
    hi = sign | 0x7ff00000u | ((mag & 0x007fffffu) >> 3) | (mag != 0x7f800000u ? 0x00080000u : 0u);
    lo = b << 29;
  } else if (mag >= 0x00800000u) {  // normal: exponent rebiased by 1023 - 127 = 896
    hi = sign | ((mag >> 3) + 0x38000000u);
    lo = b << 29;
  } else {
    hi = sign;
    lo = 0u;
  }
  return __hiloint2double((int)hi, (int)lo);
}

// narrow_mirror: mirror_of(x) (round to nearest even, an FP32 subnormal
// flushed to a zero of the same sign) by integer operations only; an
// overflow gives an infinity, a NaN a quiet NaN.
__device__ __forceinline__ float narrow_mirror(double x) {
  const unsigned long long t = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(t >> 32) & 0x80000000u;
  const unsigned long long mag = t & 0x7fffffffffffffffull;
  const int e = (int)(mag >> 52) - 896;  // the FP32 biased exponent
  unsigned r;
  if (e >= 1 && e <= 254) {
    const unsigned rem = (unsigned)(mag & 0x1fffffffull);  // the 29 bits rounded off
    r = (unsigned)((mag >> 29) - (896ull << 23));         // FP32 exponent and mantissa
    r += (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;  // ties to even; a carry
  } else if (e <= 0) {                                                       // moves into the exponent
    // below FLT_MIN: flushed, unless it rounds up to FLT_MIN
    // (x >= 2^-126 (1 - 2^-24), ties included)
    r = (e == 0 && (mag & 0x000fffffffffffffull) >= 0x000fffffe0000000ull) ? 0x00800000u : 0u;
  } else if (mag > 0x7ff0000000000000ull) {  // NaN
    r = 0x7fc00000u | (unsigned)((mag & 0x000fffffffffffffull) >> 29);
  } else {  // overflow, infinity
    r = 0x7f800000u;
  }
  return __uint_as_float(sign | r);
}

// Signal speed |v| + cs of a cell's FP32 state (the mixed CFL's); bad is set
// for a non-positive density or a non-finite speed, which the maximum skips.
template <int D>
__device__ __forceinline__ float speed_f32(const MixedParams& M, const float* u, int& bad) {
  float ss = 0.f;
#pragma unroll
  for (int a = 0; a < D; ++a) ss = ss + u[1 + a] * u[1 + a];
  const float v = sqrtf(ss) / u[0] + sound_speed<D>(M.G, u);
  if (!(u[0] > 0.f) || !isfinite(v)) bad = 1;
  return v;
}

// The CFL pass carried by the last sweep of the mixed step: besides U^{n+1}
// it writes the interior of U^{n+1}'s FP32 mirror (Uf_next) and folds the
// FP32 signal speeds of U^{n+1} into *bits, so the next step's CFL pass
// only forms dt (launch_cfl_carry). Null members: no carry.
struct SweepCarry {
  float* Uf_next = nullptr;
  unsigned long long* bits = nullptr;
  int* status = nullptr;
};

// Mixed-precision launchers (kernels_mixed.cu).
cudaError_t launch_to_f32(const double* U, float* Uf, long long n, cudaStream_t st);
// The CFL of a step whose previous step carried the pass: when *carry_ok and
// that step queued no FP64 fix-up (*prev_fix == 0; the fix-up would have
// changed cells after the carry), dt from *carry_bits; otherwise the whole
// launch_cfl_mixed pass. Either way *carry_bits is cleared and *carry_ok set
// for the step's own carrying sweep.
cudaError_t launch_cfl_carry(const MixedParams& M, const double* U, float* Uf, const Geom& g, double courant,
                             const Dx& dx, const StepScratch& s, unsigned long long* carry_bits, int* carry_ok,
                             const int* prev_fix, cudaStream_t st);
// FP32 CFL of the mixed form: also writes the interior of the FP32 mirror Uf
// from U (the sweeps read the mirror; the step that wrote U left it stale).
cudaError_t launch_cfl_mixed(const MixedParams& M, const double* U, float* Uf, const Geom& g, double courant,
                             const Dx& dx, const StepScratch& s, cudaStream_t st);
cudaError_t launch_mh_solve_mixed(const MixedParams& M, const double* U, const float* Uf,
                                  double* Unew, float* acc, const Geom& g,
                                  const Dx& dx, const StepScratch& s, const FallbackQueue& q,
                                  const SweepPlan& plan, cudaStream_t st, cudaEvent_t* ev = nullptr,
                                  const SweepCarry& carry = SweepCarry(), int* fused = nullptr);
// The x and y sweeps of a 3-D box as one kernel (sweeps.cu, sweep_xy_kernel):
// cudaErrorNotSupported where its tensor copy cannot be used (rows of the
// mirror not a multiple of 16 bytes, the encoder unavailable, too many tiles);
// the caller then runs the two sweeps.
cudaError_t launch_sweep_xy_3(const MixedParams& M, const float* Uf, const Geom& g, const Dx& dx,
                              const double* dtp, float* acc, const FallbackQueue& q, cudaStream_t st);
// The tensor map of sweep_xy_kernel's plane copies (kernels_mixed.cu).
bool encode_xy_map(CUtensorMap* out, const float* Uf, const Geom& g, int TX, int TY);
cudaError_t launch_ghost_fill_f32(const DevParams& P, float* Uf, const Geom& g, cudaStream_t st);
// The mixed solve of the slab of interior cells [lo, hi] of the outermost
// axis: its sweeps, then the FP64 fix-up of the queue entries from *done on,
// after which *done is the queue's length. Solving every slab in order, with
// *q.n and *done zeroed before the first, gives launch_mh_solve_mixed's
// result. A slab's cells are final after its call except its last row: the
// interface between it and the next slab's first row is queued for the FP64
// fix-up (if at all) by the next slab.
cudaError_t launch_mh_solve_mixed_slab(const MixedParams& M, const double* U, const float* Uf, double* Unew,
                                       float* acc, const Geom& g, const Dx& dx, const StepScratch& s,
                                       const FallbackQueue& q, int* done, const SweepPlan& plan, int lo, int hi,
                                       cudaStream_t st);
// Elements [e0, e1) of a box's component blocks just copied into U: their
// FP32 mirror written to Uf, ghost cells copied into V, FP32 CFL maximum of
// the interior folded into *bits (launch_cfl_finish turns it into dt as
// launch_cfl_mixed would).
cudaError_t launch_ingest_mixed(const MixedParams& M, const double* U, double* V, float* Uf, const Geom& g,
                                long long e0, long long e1, unsigned long long* bits, int* status,
                                cudaStream_t st);
cudaError_t launch_cfl_finish(const unsigned long long* bits, double courant, const Dx& dx, const StepScratch& s,
                              cudaStream_t st);

// ---- batches of boxes (kernels_batch.cu) ---------------------------------
// One entry of a batch's device box table, for one step parity: U is read,
// V written (and in mixed precision the FP32 mirror Uf of U, which the
// step's CFL pass writes).
struct BoxDesc {
  double* U;
  double* V;
  float* Uf;
  float* acc;
  double* faces;
  double* fluxes;
  double* ctl;  // control block: dt, CFL max bits, counter, status, ...
  Geom g;
  Dx dx;
  double omega;
  float omega_f;
  int limiter;
  int solver_type;
  int bc[6];
  double inflow[6][5];
  int cfl_items;  // CFL work items of this box (last one finishes dt)
};

// A work item: `chunk` of pass `axis` of box `box` (or a sweep tile).
struct WorkItem {
  int box;
  int axis;
  long long chunk;
};

// Device views of a batch's per-pass item lists and queue heads.
struct BatchLists {
  const WorkItem* cfl;
  const WorkItem* ghost;
  const WorkItem* faces;
  const WorkItem* flux;
  const WorkItem* update;
  const WorkItem* sweep[3][kSweepShapes];  // tiles of each axis, grouped by shape
  int n_cfl, n_ghost, n_faces, n_flux, n_update, n_sweep[3][kSweepShapes];
  int* heads;  // one queue head per pass (kBatchHeads, reset before each step)
};

// Tile count of a sweep of a box of dims n along `axis` with tile shape
// `shape` (the work items of a batch enumerate these).
long long sweep_tile_count(int ndim, int axis, int shape, const int* n);

// One mixed sweep along `axis` with tile shape `shape` of the slab of a box
// holding interior cells [lo, hi] of its outermost axis (sweeps.cu, compiled
// once per dimensionality).
#define RGPU_SWEEP_DECL(D)                                                                              \
  cudaError_t launch_sweep_axis_##D(int axis, int shape, const MixedParams& M, const float* Uf,         \
                                    const double* U, const Geom& g, const Dx& dx, const double* dtp,    \
                                    float* acc, double* Unew, const FallbackQueue& q, int lo, int hi,   \
                                    cudaStream_t st, const SweepCarry& carry);                          \
  cudaError_t launch_batch_sweep_axis_##D(int axis, int shape, const MixedParams& M, const BoxDesc* TB, \
                                          const WorkItem* items, int n, int* head, const FallbackQueue& q, \
                                          cudaStream_t st);
RGPU_SWEEP_DECL(1)
RGPU_SWEEP_DECL(2)
RGPU_SWEEP_DECL(3)
#undef RGPU_SWEEP_DECL

inline cudaError_t launch_sweep_slab(int ndim, int axis, int shape, const MixedParams& M, const float* Uf,
                                     const double* U, const Geom& g, const Dx& dx, const double* dtp,
                                     float* acc, double* Unew, const FallbackQueue& q, int lo, int hi,
                                     cudaStream_t st, const SweepCarry& carry = SweepCarry()) {
  switch (ndim) {
    case 1: return launch_sweep_axis_1(axis, shape, M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
    case 2: return launch_sweep_axis_2(axis, shape, M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
    case 3: return launch_sweep_axis_3(axis, shape, M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
    default: return cudaErrorInvalidValue;
  }
}

// The sweep over the whole box (carry: given to the last axis only).
inline cudaError_t launch_sweep_axis(int ndim, int axis, int shape, const MixedParams& M, const float* Uf,
                                     const double* U, const Geom& g, const Dx& dx, const double* dtp,
                                     float* acc, double* Unew, const FallbackQueue& q, cudaStream_t st,
                                     const SweepCarry& carry = SweepCarry()) {
  if (ndim < 1 || ndim > 3) return cudaErrorInvalidValue;
  return launch_sweep_slab(ndim, axis, shape, M, Uf, U, g, dx, dtp, acc, Unew, q, 1, g.n[ndim - 1], st, carry);
}

inline cudaError_t launch_batch_sweep_axis(int ndim, int axis, int shape, const MixedParams& M,
                                           const BoxDesc* TB, const WorkItem* items, int n, int* head,
                                           const FallbackQueue& q, cudaStream_t st) {
  switch (ndim) {
    case 1: return launch_batch_sweep_axis_1(axis, shape, M, TB, items, n, head, q, st);
    case 2: return launch_batch_sweep_axis_2(axis, shape, M, TB, items, n, head, q, st);
    case 3: return launch_batch_sweep_axis_3(axis, shape, M, TB, items, n, head, q, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_batch_cfl_mixed(const MixedParams& M, double courant, const BoxDesc* TB,
                                   const BatchLists& L, cudaStream_t st);
cudaError_t launch_batch_sweeps(const MixedParams& M, const BoxDesc* TB, const BatchLists& L,
                                const FallbackQueue& q, cudaStream_t st);
cudaError_t launch_batch_step(const DevParams& P, const MixedParams& M, bool mixed, int ndim,
                              const BoxDesc* table, const BatchLists& L, FallbackQueue q,
                              cudaStream_t st);

// Queue heads of a batch step: 0 cfl, 1 ghost, 2 faces, 3 flux, 4 update,
// 5 ghost (FP32 mirror), 6 + kSweepShapes * axis + shape the sweeps.
constexpr int kBatchHeads = 32;
constexpr int kHeadGhostF32 = 5;
constexpr int kHeadSweep0 = 6;

// Chunk sizes of the batched passes (elements per work item).
constexpr int kBatchChunk = 256;
constexpr int kBatchFluxChunk = 128;

// One box of a level output (kernels_output.cu): its current state, its
// interior cell count, the start of its hydro elements in the flattened
// list of all boxes' hydro elements, and its offset in the output dataset
// (sum over the boxes before it of cells x NCMP).
struct PackDesc {
  const double* U;
  Geom g;
  long long cells;
  long long hydro_off;
  long long out_off;
};

cudaError_t launch_pack_level(const PackDesc* desc, int n, long long total, int ndim, float* out,
                              cudaStream_t st);

// Sanity checks (kernels_sanity.cu): the properties of
// rhyme_sanity_check_fill.f90 that live on the device, their ranges, and
// the partial result of a run of cells in loop order.
enum { SC_RHO = 0, SC_VX, SC_VY, SC_VZ, SC_E_TOT, SC_ABS_V, SC_MACH, SC_COUNT };

struct SanityRanges {
  double range[SC_COUNT][2];
  int enabled[SC_COUNT];
};

struct SanityPartial {
  long long nbelow[SC_COUNT], nabove[SC_COUNT];
  double vbelow[SC_COUNT], pbelow[SC_COUNT];  // extreme below the range, running extreme before it
  double vabove[SC_COUNT], pabove[SC_COUNT];
  long long ibelow[SC_COUNT], iabove[SC_COUNT];  // loop-order cell index of the extremes (-1: none)
  int nan[5];                                    // a NaN in component c
  double rho_min, e_min;                         // minima of rho and e_tot
  long long irho_min, ie_min;                    // their first cells
};

__host__ __device__ void merge_partial(SanityPartial& a, const SanityPartial& b);
cudaError_t launch_sanity(int ndim, const double* U, const Geom& g, const Gas<double>& G, const SanityRanges& R,
                          SanityPartial* parts, int nblocks, SanityPartial* out, cudaStream_t st);
// parts: 2 * nblocks double-double pairs (32 bytes each)
cudaError_t launch_totals(int ndim, const double* U, long long field, void* parts, int nblocks, double* out,
                          cudaStream_t st);

// Initial-condition painting (kernels_paint.cu). Colours and perturbation
// bases are primitive vectors packed as (rho, v_1..v_NDIM, p).
enum { PAINT_CANVAS = 0, PAINT_SHARP_CUBOID, PAINT_SPHERE, PAINT_SMOOTHED_SLAB, PAINT_HARMONIC,
       PAINT_SYMMETRIC_DECAYING };

struct PaintShape {
  int type, axis, periodic, keep_outside;
  int lb[3], ub[3];  // sharp cuboid: cell bounds in this box (1-based, inclusive)
  double prim[2][5];
  double origin[3];
  double r, sigma;
  double pos[2], slab_sigma[2];
  double amplitude, wavelength, phase;
  double base[5];
};

cudaError_t launch_paint(int ndim, const PaintShape* shapes, int n, const Gas<double>& G, const Geom& g,
                         const int* left_edge, double* U, float* Uf, cudaStream_t st);

// Element-level launchers (kernels_elem.cu): device arrays in and out.
cudaError_t launch_riemann_solve(const DevParams& P, const double* l, const double* r, long long n,
                                 double dxdt, int axis, double* u, cudaStream_t st);
cudaError_t launch_irs_exec(const DevParams& P, const double* states, long long n, double* out,
                            cudaStream_t st);
cudaError_t launch_slope_limiter(const DevParams& P, const double* ul, const double* u,
                                 const double* ur, long long n, double* delta, cudaStream_t st);
cudaError_t launch_half_step(const DevParams& P, const double* u, const double* delta, long long n,
                             int axis, double hdtdx, double* l, double* r, cudaStream_t st);

}  // namespace rgpu
