// kernels_mixed.cu -- mixed-precision MUSCL-Hancock step.
//
// The conserved state stays FP64 in HBM (U) and is mirrored once per step as
// FP32 (Uf) by the step's first pass, the FP32 CFL, which reads U anyway.
// Each axis is one fused sweep kernel: a CTA stages a slab of Uf (S cells
// along the sweep axis plus the 2-cell ghost/halo layer, for P pencils) in
// shared memory with coalesced loads, computes FP32 limited slopes and
// half-step face states for S+2 cells, solves the S+1 exact Riemann problems
// of the slab in FP32 and forms the flux difference of its S cells. The flux
// differences of the axes are summed in FP32 in the reference's association
// ((X + Y) + Z), and the last sweep adds the sum to U in FP64 and writes
// U^{n+1}: one FP64 add per conserved component and cell, since on GB300 even
// FP64 adds are scarce (the next step's CFL makes the new mirror, where the
// conversions cost nothing but bandwidth).
//
// Interfaces that near vacuum, or whose FP32 Newton iteration misses the
// tolerance on its first guess, or whose FP32 face states or flux are not
// finite, get a zero flux in the sweep and are appended (once, by the tile
// that owns them) to a device queue. After the last sweep one kernel redoes
// each queued interface in FP64 from U^n, which the step leaves intact
// (limited slopes and half-step face states of its two cells, exact Riemann
// problem, flux: the device code of the plain path instantiated for double),
// and applies -+ dt/dx * F to the two adjacent interior cells of U^{n+1}.
// Keeping the FP64 code out of the sweeps keeps them at 50-52 registers (it
// tripled their register count inline).
//
// The CFL maximum of the mixed path is taken in FP32 over the mirror; dt
// itself is formed in FP64.
//
// For the drop-in loop with the state in host memory, ingest_kernel takes
// each slab of an upload as it arrives (the mirror, the ghost cells of the
// other buffer, the slab's share of the CFL maximum), cfl_finish_kernel
// forms dt from that maximum, and launch_mh_solve_mixed_slab solves the box
// in slabs of rows, each with the FP64 fix-up of the entries queued so far,
// so that finished rows can be copied back while the next slab is solved.
#include <math_constants.h>

#include <atomic>
#include <cstdint>
#include <cstdlib>

#include "../../include/rhyme_gpu.h"
#include "rgpu_internal.h"

namespace rgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 152 * 32;

inline int grid_for(long long total, int block) {
  long long b = (total + block - 1) / block;
  if (b < 1) b = 1;
  if (b > kMaxBlocks) b = kMaxBlocks;
  return (int)b;
}

// U (FP64) -> Uf (FP32) over whole component blocks (ghosts included).
__global__ void __launch_bounds__(kThreads) to_f32_kernel(const double* __restrict__ U,
                                                          float* __restrict__ Uf, long long n) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    Uf[t] = mirror_of(U[t]);
}

// |v| + cs of one cell in FP32; bad marks non-positive density or a
// non-finite value.

// Interior cell t: its FP32 mirror, written to Uf from U, and its signal
// speed.
template <int D>
__device__ __forceinline__ float signal_speed_f32(const MixedParams& M, const double* __restrict__ U,
                                                  float* __restrict__ Uf, const Geom& g, long long t, int& bad) {
  const long long n0 = g.n[0], n1 = g.n[1];
  const int i = (int)(t % n0) + 1;
  const long long q = t / n0;
  const int j = (int)(q % n1) + 1;
  const int k = (int)(q / n1) + 1;
  const long long o = g.at(D, i, j, k);
  float u[D + 2];
#pragma unroll
  for (int c = 0; c < D + 2; ++c) {
    u[c] = mirror_of(U[(long long)c * g.field + o]);
    Uf[(long long)c * g.field + o] = u[c];
  }
  return speed_f32<D>(M, u, bad);
}

// Block-wide maximum and or of (m, bad), folded into *bits and *status by
// one thread.
__device__ __forceinline__ void block_fold(float m, int bad, unsigned long long* bits, int* status) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float o = __shfl_down_sync(0xffffffffu, m, off);
    if (o > m) m = o;
    bad |= __shfl_down_sync(0xffffffffu, bad, off);
  }
  __shared__ float sm[kThreads / 32];
  __shared__ int sb[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sm[warp] = m;
    sb[warp] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kThreads / 32; ++k) {
      if (sm[k] > m) m = sm[k];
      bad |= sb[k];
    }
    atomicMax(bits, (unsigned long long)__float_as_uint(m));
    if (bad) atomicOr(status, 1);
  }
}

// The arrival of rows [e0, e1) (elements of every component block; whole
// rows of the outermost axis, ghosts included) of a box just copied into U:
// the FP32 mirror Uf of every cell is written, the ghost cells are copied
// into the other state buffer V, whose interior the next solve writes, and
// the FP32 signal speed of every interior cell (the arithmetic of
// cfl_f32_kernel) is folded into *bits, so that the CFL maximum is ready
// when the last row has arrived.
template <int D>
__global__ void __launch_bounds__(kThreads)
    ingest_kernel(MixedParams M, const double* __restrict__ U, double* __restrict__ V, float* __restrict__ Uf,
                  Geom g, long long e0, long long e1, unsigned long long* bits, int* status) {
  const long long F = g.field;
  const long long E0 = g.s[1];                       // row length along x, ghosts included
  const long long E1 = (D > 2) ? g.s[2] / g.s[1] : 1;  // rows per plane
  float m = 0.f;
  int bad = 0;
  for (long long t = e0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; t < e1;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % E0);
    const long long r = t / E0;
    const int j = (D > 2) ? (int)(r % E1) : (int)r;
    const int k = (D > 2) ? (int)(r / E1) : 0;
    bool in = i >= 2 && i <= g.n[0] + 1;
    if (D > 1) in = in && j >= 2 && j <= g.n[1] + 1;
    if (D > 2) in = in && k >= 2 && k <= g.n[2] + 1;
    float u[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      const double x = U[(long long)c * F + t];
      u[c] = mirror_of(x);
      Uf[(long long)c * F + t] = u[c];
      if (!in) V[(long long)c * F + t] = x;
    }
    if (in) {
      const float v = speed_f32<D>(M, u, bad);
      if (v > m) m = v;
    }
  }
  block_fold(m, bad, bits, status);
}

// dt from a maximum folded by ingest_kernel: the last step of cfl_f32_kernel.
__global__ void cfl_finish_kernel(const unsigned long long* __restrict__ bits, double courant, double mdx,
                                  StepScratch s) {
  const float mu = __uint_as_float((unsigned int)*bits);
  const double dt = courant * mdx / (double)mu;
  *s.dt = dt;
  if (s.dt_trace) {
    const int pos = *s.trace_pos;
    if (pos >= 0 && pos < s.trace_cap) s.dt_trace[pos] = dt;
    *s.trace_pos = pos + 1;
  }
}

// FP32 mirror of the interior of U and its signal-speed maximum; the last
// block forms dt = courant * min(dx) / max in FP64 and resets the
// accumulators.
template <int D>
__global__ void __launch_bounds__(kThreads)
    cfl_f32_kernel(MixedParams M, const double* __restrict__ U, float* __restrict__ Uf, Geom g, double courant,
                   double mdx, StepScratch s) {
  const long long total = (long long)g.n[0] * g.n[1] * (long long)g.n[2];
  float m = 0.f;
  int bad = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const float v = signal_speed_f32<D>(M, U, Uf, g, t, bad);
    if (v > m) m = v;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float o = __shfl_down_sync(0xffffffffu, m, off);
    if (o > m) m = o;
    bad |= __shfl_down_sync(0xffffffffu, bad, off);
  }
  __shared__ float sm[kThreads / 32];
  __shared__ int sb[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sm[warp] = m;
    sb[warp] = bad;
  }
  __syncthreads();
  if (warp == 0) {
    m = (lane < kThreads / 32) ? sm[lane] : 0.f;
    bad = (lane < kThreads / 32) ? sb[lane] : 0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float o = __shfl_down_sync(0xffffffffu, m, off);
      if (o > m) m = o;
      bad |= __shfl_down_sync(0xffffffffu, bad, off);
    }
    if (lane == 0) {
      // non-negative floats order like their bit patterns
      atomicMax(s.max_bits, (unsigned long long)__float_as_uint(m));
      if (bad) atomicOr(s.status, 1);
      __threadfence();
      const unsigned int prev = atomicAdd(s.counter, 1u);
      if (prev == gridDim.x - 1) {
        __threadfence();
        const float mu = __uint_as_float((unsigned int)atomicAdd(s.max_bits, 0ull));
        const double dt = courant * mdx / (double)mu;
        *s.dt = dt;
        if (s.dt_trace) {
          const int pos = *s.trace_pos;
          if (pos >= 0 && pos < s.trace_cap) s.dt_trace[pos] = dt;
          *s.trace_pos = pos + 1;
        }
        atomicExch(s.max_bits, 0ull);
        atomicExch(s.counter, 0u);
      }
    }
  }
}

// The CFL of a step after a carrying step: dt from the carried maximum when
// it is the current state's (no FP64 fix-up changed cells after it), else
// the pass of cfl_f32_kernel; then the carry is cleared for this step's own
// carrying sweep.
template <int D>
__global__ void __launch_bounds__(kThreads)
    cfl_carry_kernel(MixedParams M, const double* __restrict__ U, float* __restrict__ Uf, Geom g, double courant,
                     double mdx, StepScratch s, unsigned long long* carry_bits, int* carry_ok,
                     const int* __restrict__ prev_fix) {
  const bool use = *carry_ok != 0 && *prev_fix == 0;
  if (use) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      const float mu = __uint_as_float((unsigned int)*carry_bits);
      const double dt = courant * mdx / (double)mu;
      *s.dt = dt;
      if (s.dt_trace) {
        const int pos = *s.trace_pos;
        if (pos >= 0 && pos < s.trace_cap) s.dt_trace[pos] = dt;
        *s.trace_pos = pos + 1;
      }
      *carry_bits = 0ull;
    }
    return;
  }
  const long long total = (long long)g.n[0] * g.n[1] * (long long)g.n[2];
  float m = 0.f;
  int bad = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const float v = signal_speed_f32<D>(M, U, Uf, g, t, bad);
    if (v > m) m = v;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float o = __shfl_down_sync(0xffffffffu, m, off);
    if (o > m) m = o;
    bad |= __shfl_down_sync(0xffffffffu, bad, off);
  }
  __shared__ float sm[kThreads / 32];
  __shared__ int sb[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sm[warp] = m;
    sb[warp] = bad;
  }
  __syncthreads();
  if (warp == 0) {
    m = (lane < kThreads / 32) ? sm[lane] : 0.f;
    bad = (lane < kThreads / 32) ? sb[lane] : 0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float o = __shfl_down_sync(0xffffffffu, m, off);
      if (o > m) m = o;
      bad |= __shfl_down_sync(0xffffffffu, bad, off);
    }
    if (lane == 0) {
      atomicMax(s.max_bits, (unsigned long long)__float_as_uint(m));
      if (bad) atomicOr(s.status, 1);
      __threadfence();
      const unsigned int prev = atomicAdd(s.counter, 1u);
      if (prev == gridDim.x - 1) {
        __threadfence();
        const float mu = __uint_as_float((unsigned int)atomicAdd(s.max_bits, 0ull));
        const double dt = courant * mdx / (double)mu;
        *s.dt = dt;
        if (s.dt_trace) {
          const int pos = *s.trace_pos;
          if (pos >= 0 && pos < s.trace_cap) s.dt_trace[pos] = dt;
          *s.trace_pos = pos + 1;
        }
        atomicExch(s.max_bits, 0ull);
        atomicExch(s.counter, 0u);
        *carry_bits = 0ull;
        *carry_ok = 1;
      }
    }
  }
}

// FP64 flux of the interface between cell o (index ga along AX) and cell
// o + s_AX, from U^n: face states of both cells (cells ga-1 .. ga+2, the
// ghost layer included) and the exact Riemann problem at x/t = 0.
template <int D, int AX>
__device__ __noinline__ void redo_interface(const MixedParams& M, int limiter, double omega,
                                            const double* __restrict__ U, const Geom& g, long long o,
                                            double hdtdx, double* f) {
  const long long F = g.field, sa = g.s[AX];
  double w0[D + 2], w1[D + 2], w2[D + 2], w3[D + 2];
#pragma unroll
  for (int c = 0; c < D + 2; ++c) {
    const double* p = U + (long long)c * F + o;
    w0[c] = p[-sa];
    w1[c] = p[0];
    w2[c] = p[sa];
    w3[c] = p[2 * sa];
  }
  // a non-finite U^n (a box the scheme has already lost) makes the FP64
  // solve iterate to its cap for a NaN result: give the NaN directly
  bool finite = true;
#pragma unroll
  for (int c = 0; c < D + 2; ++c) finite = finite && isfinite(w0[c]) && isfinite(w1[c]) && isfinite(w2[c]) && isfinite(w3[c]);
  if (!finite) {
#pragma unroll
    for (int c = 0; c < D + 2; ++c) f[c] = CUDART_NAN;
    return;
  }
  double lo[D + 2], ro[D + 2], l1[D + 2], r1[D + 2];
  face_states<D, AX>(M.G64, limiter, omega, w0, w1, w2, hdtdx, lo, ro);
  face_states<D, AX>(M.G64, limiter, omega, w1, w2, w3, hdtdx, l1, r1);
  interface_flux<D, AX>(M.G64, M.rp64, ro, l1, f);
}

template <int D>
__device__ __forceinline__ void redo_any_axis(const MixedParams& M, int limiter, double omega,
                                              const double* __restrict__ U, const Geom& g, int axis,
                                              long long o, double hdtdx, double* f) {
  if (axis == 0) redo_interface<D, 0>(M, limiter, omega, U, g, o, hdtdx, f);
  if constexpr (D > 1) {
    if (axis == 1) redo_interface<D, 1>(M, limiter, omega, U, g, o, hdtdx, f);
  }
  if constexpr (D > 2) {
    if (axis == 2) redo_interface<D, 2>(M, limiter, omega, U, g, o, hdtdx, f);
  }
}

// FP64 redo of the queued interfaces; -+ dt/dx * F applied to the adjacent
// interior cells of U^{n+1} (atomically: a cell can border two queued
// interfaces).
// Entries from *from (0 when from is null) to the queue's end: a solve in
// slabs fixes the entries of each slab after its sweeps.
template <int D>
__global__ void __launch_bounds__(128)
    fallback_fix_kernel(MixedParams M, FallbackQueue q, Geom g, Dx dx, const double* __restrict__ dtp,
                        const double* __restrict__ U, double* __restrict__ Unew, const int* __restrict__ from) {
  const int n = min(*q.n, q.cap);
  const int lo = from ? min(*from, n) : 0;
  if (blockIdx.x == 0 && threadIdx.x == 0 && n > lo) atomicAdd(q.total, n - lo);
  const double dt = *dtp;
  const long long F = g.field;
  for (int i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const FallbackEntry e = q.e[i];
    double f[D + 2];
    redo_any_axis<D>(M, M.limiter, M.omega64, U, g, e.axis, e.o, 0.5 * dt / dx.v[e.axis], f);
    const double dtdx = dt / dx.v[e.axis];
    const long long sa = g.s[e.axis];
    const int NA = g.n[e.axis];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      const double corr = dtdx * f[c];
      if (e.ga >= 1) atomicAdd(&Unew[(long long)c * F + e.o], -corr);
      if (e.ga + 1 <= NA) atomicAdd(&Unew[(long long)c * F + e.o + sa], corr);
    }
  }
}

template <int D>
cudaError_t launch_fallback(const MixedParams& M, const FallbackQueue& q, const Geom& g, const Dx& dx,
                            const double* dtp, const double* U, double* Unew, cudaStream_t st,
                            const int* from = nullptr) {
  fallback_fix_kernel<D><<<152, 128, 0, st>>>(M, q, g, dx, dtp, U, Unew, from);
  return cudaGetLastError();
}

// Batched FP32 CFL over work items (chunks of 256 cells of a box): per-box
// maximum through atomics, the last item of a box forms its dt in FP64.
template <int D>
__global__ void __launch_bounds__(256)
    batch_cfl_f32_kernel(MixedParams M, double courant, const BoxDesc* __restrict__ TB,
                         const WorkItem* __restrict__ items, int n, int* head) {
  __shared__ float sm[8];
  __shared__ int sb[8];
  __shared__ int s_item;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= n) break;
    const WorkItem w = items[it];
    const BoxDesc& b = TB[w.box];
    const long long total = (long long)b.g.n[0] * b.g.n[1] * b.g.n[2];
    const long long t = w.chunk * kBatchChunk + threadIdx.x;
    float m = 0.f;
    int bad = 0;
    if (t < total) {
      const float v = signal_speed_f32<D>(M, b.U, b.Uf, b.g, t, bad);
      if (v > m) m = v;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float o = __shfl_down_sync(0xffffffffu, m, off);
      if (o > m) m = o;
      bad |= __shfl_down_sync(0xffffffffu, bad, off);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
      sm[warp] = m;
      sb[warp] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 1; k < 8; ++k) {
        if (sm[k] > m) m = sm[k];
        bad |= sb[k];
      }
      unsigned long long* max_bits = (unsigned long long*)(b.ctl + 1);
      unsigned int* counter = (unsigned int*)(b.ctl + 2);
      int* status = (int*)(b.ctl + 2) + 1;
      atomicMax(max_bits, (unsigned long long)__float_as_uint(m));
      if (bad) atomicOr(status, 1);
      __threadfence();
      if (atomicAdd(counter, 1u) == (unsigned int)(b.cfl_items - 1)) {
        __threadfence();
        const float mu = __uint_as_float((unsigned int)atomicAdd(max_bits, 0ull));
        b.ctl[0] = courant * b.dx.min / (double)mu;
        atomicExch(max_bits, 0ull);
        atomicExch(counter, 0u);
      }
    }
  }
}

// Batched FP64 fix-up: as fallback_fix_kernel, with the box of each entry.
template <int D>
__global__ void __launch_bounds__(128)
    batch_fallback_fix_kernel(MixedParams M, FallbackQueue q, const BoxDesc* __restrict__ TB) {
  const int n = min(*q.n, q.cap);
  if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0) atomicAdd(q.total, n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const FallbackEntry e = q.e[i];
    const BoxDesc& b = TB[e.box];
    double f[D + 2];
    redo_any_axis<D>(M, b.limiter, b.omega, b.U, b.g, e.axis, e.o, 0.5 * b.ctl[0] / b.dx.v[e.axis], f);
    const double dtdx = b.ctl[0] / b.dx.v[e.axis];
    const long long sa = b.g.s[e.axis];
    const int NA = b.g.n[e.axis];
    const long long F = b.g.field;
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      const double corr = dtdx * f[c];
      if (e.ga >= 1) atomicAdd(&b.V[(long long)c * F + e.o], -corr);
      if (e.ga + 1 <= NA) atomicAdd(&b.V[(long long)c * F + e.o + sa], corr);
    }
  }
}

template <int D>
cudaError_t launch_batch_fallback(const MixedParams& M, const BoxDesc* TB, const FallbackQueue& q,
                                  cudaStream_t st) {
  batch_fallback_fix_kernel<D><<<152, 128, 0, st>>>(M, q, TB);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_to_f32(const double* U, float* Uf, long long n, cudaStream_t st) {
  to_f32_kernel<<<grid_for(n, kThreads), kThreads, 0, st>>>(U, Uf, n);
  return cudaGetLastError();
}

cudaError_t launch_cfl_mixed(const MixedParams& M, const double* U, float* Uf, const Geom& g, double courant,
                             const Dx& dx, const StepScratch& s, cudaStream_t st) {
  const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
  int grid = grid_for(total, kThreads);
  if (grid > 152 * 4) grid = 152 * 4;
  switch (M.ndim) {
    case 1: cfl_f32_kernel<1><<<grid, kThreads, 0, st>>>(M, U, Uf, g, courant, dx.min, s); break;
    case 2: cfl_f32_kernel<2><<<grid, kThreads, 0, st>>>(M, U, Uf, g, courant, dx.min, s); break;
    case 3: cfl_f32_kernel<3><<<grid, kThreads, 0, st>>>(M, U, Uf, g, courant, dx.min, s); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_cfl_carry(const MixedParams& M, const double* U, float* Uf, const Geom& g, double courant,
                             const Dx& dx, const StepScratch& s, unsigned long long* carry_bits, int* carry_ok,
                             const int* prev_fix, cudaStream_t st) {
  const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
  int grid = grid_for(total, kThreads);
  if (grid > 152 * 4) grid = 152 * 4;
  switch (M.ndim) {
    case 1:
      cfl_carry_kernel<1><<<grid, kThreads, 0, st>>>(M, U, Uf, g, courant, dx.min, s, carry_bits, carry_ok, prev_fix);
      break;
    case 2:
      cfl_carry_kernel<2><<<grid, kThreads, 0, st>>>(M, U, Uf, g, courant, dx.min, s, carry_bits, carry_ok, prev_fix);
      break;
    case 3:
      cfl_carry_kernel<3><<<grid, kThreads, 0, st>>>(M, U, Uf, g, courant, dx.min, s, carry_bits, carry_ok, prev_fix);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_mh_solve_mixed(const MixedParams& M, const double* U, const float* Uf,
                                  double* Unew, float* acc, const Geom& g,
                                  const Dx& dx, const StepScratch& s, const FallbackQueue& q,
                                  const SweepPlan& plan, cudaStream_t st, cudaEvent_t* ev,
                                  const SweepCarry& carry, int* fused) {
  // ev (optional, 3 events): recorded after the x sweep, after the y sweep
  // and at the end (the z sweep and the FP64 fix-up); absent axes record
  // at the same point, and so do both when one kernel ran the x and y
  // sweeps (*fused, optional, is then 1).
  const int D = M.ndim;
  if (D < 1 || D > 3) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(q.n, 0, sizeof(int), st);
  int first = 0;
  if (fused) *fused = 0;
  if (e == cudaSuccess && D == 3 && plan.fuse_xy) {
    // the x and y sweeps in one kernel where the mirror's rows allow the
    // plane's tensor copy (bit-identical to the two sweeps)
    e = launch_sweep_xy_3(M, Uf, g, dx, s.dt, acc, q, st);
    if (e == cudaSuccess) {
      first = 2;
      if (fused) *fused = 1;
      if (ev) e = cudaEventRecord(ev[0], st);
      if (e == cudaSuccess && ev) e = cudaEventRecord(ev[1], st);
    } else if (e == cudaErrorNotSupported) {
      e = cudaSuccess;
    }
  }
  for (int a = first; a < D; ++a) {
    if (e == cudaSuccess)
      e = launch_sweep_axis(D, a, plan.shape[a], M, Uf, U, g, dx, s.dt, acc, Unew, q, st,
                            a == D - 1 ? carry : SweepCarry());
    if (e == cudaSuccess && ev && a < 2) e = cudaEventRecord(ev[a], st);
  }
  for (int a = D; a < 2; ++a)
    if (e == cudaSuccess && ev) e = cudaEventRecord(ev[a], st);
  if (e == cudaSuccess) {
    switch (D) {
      case 1: e = launch_fallback<1>(M, q, g, dx, s.dt, U, Unew, st); break;
      case 2: e = launch_fallback<2>(M, q, g, dx, s.dt, U, Unew, st); break;
      case 3: e = launch_fallback<3>(M, q, g, dx, s.dt, U, Unew, st); break;
    }
  }
  if (e == cudaSuccess && ev) e = cudaEventRecord(ev[2], st);
  return e;
}

cudaError_t launch_mh_solve_mixed_slab(const MixedParams& M, const double* U, const float* Uf, double* Unew,
                                       float* acc, const Geom& g, const Dx& dx, const StepScratch& s,
                                       const FallbackQueue& q, int* done, const SweepPlan& plan, int lo, int hi,
                                       cudaStream_t st) {
  const int D = M.ndim;
  if (D < 1 || D > 3) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  for (int a = 0; a < D && e == cudaSuccess; ++a)
    e = launch_sweep_slab(D, a, plan.shape[a], M, Uf, U, g, dx, s.dt, acc, Unew, q, lo, hi, st);
  if (e == cudaSuccess) {
    switch (D) {
      case 1: e = launch_fallback<1>(M, q, g, dx, s.dt, U, Unew, st, done); break;
      case 2: e = launch_fallback<2>(M, q, g, dx, s.dt, U, Unew, st, done); break;
      case 3: e = launch_fallback<3>(M, q, g, dx, s.dt, U, Unew, st, done); break;
    }
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(done, q.n, sizeof(int), cudaMemcpyDeviceToDevice, st);
  return e;
}

cudaError_t launch_ingest_mixed(const MixedParams& M, const double* U, double* V, float* Uf, const Geom& g,
                                long long e0, long long e1, unsigned long long* bits, int* status,
                                cudaStream_t st) {
  if (e1 <= e0) return cudaSuccess;
  int grid = grid_for(e1 - e0, kThreads);
  if (grid > 152 * 8) grid = 152 * 8;
  switch (M.ndim) {
    case 1: ingest_kernel<1><<<grid, kThreads, 0, st>>>(M, U, V, Uf, g, e0, e1, bits, status); break;
    case 2: ingest_kernel<2><<<grid, kThreads, 0, st>>>(M, U, V, Uf, g, e0, e1, bits, status); break;
    case 3: ingest_kernel<3><<<grid, kThreads, 0, st>>>(M, U, V, Uf, g, e0, e1, bits, status); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_cfl_finish(const unsigned long long* bits, double courant, const Dx& dx, const StepScratch& s,
                              cudaStream_t st) {
  cfl_finish_kernel<<<1, 1, 0, st>>>(bits, courant, dx.min, s);
  return cudaGetLastError();
}

long long sweep_tile_count(int ndim, int axis, int shape, const int* n) {
  int S, P;
  sweep_shape(ndim, shape, &S, &P);
  const int bax = (ndim == 1) ? 1 : (axis == 0 ? 1 : 0);
  const int cax = (ndim == 3) ? 3 - axis - bax : 2;
  const long long nB = (bax < ndim) ? n[bax] : 1;
  const long long nC = (cax < ndim) ? n[cax] : 1;
  const long long nA = (n[axis] + S - 1) / S;
  return nA * ((nB + P - 1) / P) * nC;
}

cudaError_t launch_batch_cfl_mixed(const MixedParams& M, double courant, const BoxDesc* TB,
                                   const BatchLists& L, cudaStream_t st) {
  if (!L.n_cfl) return cudaSuccess;
  switch (M.ndim) {
    case 1: batch_cfl_f32_kernel<1><<<152 * 4, 256, 0, st>>>(M, courant, TB, L.cfl, L.n_cfl, L.heads + 0); break;
    case 2: batch_cfl_f32_kernel<2><<<152 * 4, 256, 0, st>>>(M, courant, TB, L.cfl, L.n_cfl, L.heads + 0); break;
    case 3: batch_cfl_f32_kernel<3><<<152 * 4, 256, 0, st>>>(M, courant, TB, L.cfl, L.n_cfl, L.heads + 0); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// The mixed passes of one batch step after the CFL and ghost passes: the
// sweeps of every box, axis by axis (one launch per tile shape in use, each
// with its own queue head), then the FP64 fix-up of the queued interfaces.
cudaError_t launch_batch_sweeps(const MixedParams& M, const BoxDesc* TB, const BatchLists& L,
                                const FallbackQueue& q, cudaStream_t st) {
  const int D = M.ndim;
  if (D < 1 || D > 3) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(q.n, 0, sizeof(int), st);
  for (int a = 0; a < D; ++a)
    for (int k = 0; k < kSweepShapes; ++k)
      if (e == cudaSuccess && L.n_sweep[a][k])
        e = launch_batch_sweep_axis(D, a, k, M, TB, L.sweep[a][k], L.n_sweep[a][k],
                                    L.heads + kHeadSweep0 + kSweepShapes * a + k, q, st);
  if (e == cudaSuccess) {
    switch (D) {
      case 1: e = launch_batch_fallback<1>(M, TB, q, st); break;
      case 2: e = launch_batch_fallback<2>(M, TB, q, st); break;
      case 3: e = launch_batch_fallback<3>(M, TB, q, st); break;
    }
  }
  return e;
}

// ---- tensor maps of the FP32 mirror (TMA staging of the sweeps) --------------
namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

std::atomic<long long> g_tma_launches{0};

EncodeTiledFn encoder() {
  const char* env = getenv("RHYME_GPU_TMA");
  if (env && env[0] == '0') return nullptr;
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (EncodeTiledFn) nullptr;
    }
    return (EncodeTiledFn)p;
  }();
  return fn;
}

}  // namespace

bool encode_mirror_map(CUtensorMap* out, const float* Uf, const Geom& g, int D, int A, int S, int P) {
  if (D < 2 || A < 0 || A >= D) return false;
  const EncodeTiledFn fn = encoder();
  if (!fn) return false;
  const long long X = g.s[1], Y = g.s[2] / g.s[1], Z = g.field / g.s[2];
  // rows (and so every stride) a multiple of 16 bytes; base 16-byte aligned
  if (X % 4 != 0 || ((uintptr_t)Uf % 16) != 0) return false;
  cuuint64_t dim[4] = {(cuuint64_t)X, (cuuint64_t)Y, (cuuint64_t)Z, (cuuint64_t)(D + 2)};
  cuuint64_t stride[3] = {(cuuint64_t)X * 4, (cuuint64_t)(X * Y) * 4, (cuuint64_t)g.field * 4};
  // the slab: S+4 cells along A; along x P pencils (A = y, z: P+4 cells from
  // an aligned start); one cell along the third axis
  cuuint32_t box[4] = {1, 1, 1, (cuuint32_t)(D + 2)};
  box[A] = (cuuint32_t)(S + 4);
  if (A == 0) {
    box[1] = (cuuint32_t)P;
  } else {
    box[0] = (cuuint32_t)(P + 4);
  }
  for (int i = 0; i < 4; ++i)
    if (box[i] > 256 || box[i] > dim[i]) return false;
  if ((box[0] * 4) % 16 != 0) return false;
  cuuint32_t estride[4] = {1, 1, 1, 1};
  const CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (void*)Uf, dim, stride, box, estride,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  g_tma_launches.fetch_add(1, std::memory_order_relaxed);
  return true;
}

bool encode_xy_map(CUtensorMap* out, const float* Uf, const Geom& g, int TX, int TY) {
  const EncodeTiledFn fn = encoder();
  if (!fn) return false;
  const long long X = g.s[1], Y = g.s[2] / g.s[1], Z = g.field / g.s[2];
  if (X % 4 != 0 || ((uintptr_t)Uf % 16) != 0) return false;
  cuuint64_t dim[4] = {(cuuint64_t)X, (cuuint64_t)Y, (cuuint64_t)Z, 5};
  cuuint64_t stride[3] = {(cuuint64_t)X * 4, (cuuint64_t)(X * Y) * 4, (cuuint64_t)g.field * 4};
  // one z plane of the tile with its 2-cell halo along x and y, every component
  cuuint32_t box[4] = {(cuuint32_t)(TX + 4), (cuuint32_t)(TY + 4), 1, 5};
  for (int i = 0; i < 4; ++i)
    if (box[i] > 256 || box[i] > dim[i]) return false;
  if ((box[0] * 4) % 16 != 0) return false;
  cuuint32_t estride[4] = {1, 1, 1, 1};
  const CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (void*)Uf, dim, stride, box, estride,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  g_tma_launches.fetch_add(1, std::memory_order_relaxed);
  return true;
}

}  // namespace rgpu

extern "C" int rhyme_gpu_tma_launches(long long* n) {
  if (!n) return RHYME_GPU_EINVAL;
  *n = rgpu::g_tma_launches.load(std::memory_order_relaxed);
  return RHYME_GPU_OK;
}

namespace rgpu {

}  // namespace rgpu
