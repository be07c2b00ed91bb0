// kernels_box.cu -- plain FP64 box kernels of the MUSCL-Hancock step.
//
//   K1 ghost_fill_kernel  rhyme_samr_bc_set_*_boundary.f90 (faces only)
//   K2 cfl_kernel         rhyme_cfl_time_step.f90:63-84 (grid max + dt)
//   K3 faces/flux/update  rhyme_muscl_hancock_solve_memory_intensive.f90
//                         loops 1-3 (and the cpu-intensive update order)
//
// The plain path on GB300 is bound by the FP64 pipe (about 1.2 TFLOP/s, with
// pow near 6 G/s and div/sqrt near 58 G/s), not by HBM: one interface solve
// costs thousands of FP64 operations against 80 bytes of state per 3-D cell.
// So K3 is laid out to do every face state and every interface solve exactly
// once with full parallelism (one thread per cell-axis, then one thread per
// interface-axis) and keeps face states and fluxes in device scratch; that
// traffic is well under 1% of HBM bandwidth at the FP64 rate.
//
// This file is compiled with --fmad=false so the double arithmetic performs
// the same IEEE operations, in the same order, as the reference.
#include <cstdio>

#include "rgpu_internal.h"

namespace rgpu {

namespace {

constexpr int kFillBlock = 256;
constexpr int kCflBlock = 256;
constexpr int kFaceBlock = 128;
constexpr int kFluxBlock = 128;
constexpr int kUpdBlock = 256;
constexpr int kMaxBlocks = 152 * 32;

inline int grid_for(long long total, int block) {
  long long b = (total + block - 1) / block;
  if (b < 1) b = 1;
  if (b > kMaxBlocks) b = kMaxBlocks;
  return (int)b;
}

// ------------------------------------------------------------------ K1 ---
// One thread per (axis, component, transverse position): fills the left then
// the right 2-cell ghost layer of its line in the order of
// rhyme_samr_bc_set_boundaries.f90:9-20, writing U and (if given) the mirror
// buffer, so both state buffers carry the ghost values the reference array
// holds after the fill.
template <int D, typename T>
__global__ void __launch_bounds__(kFillBlock)
    ghost_fill_kernel(DevParams P, T* __restrict__ U, T* __restrict__ M, Geom g,
                      long long off1, long long off2, long long total) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int axis;
    long long r;
    if (t < off1) {
      axis = 0;
      r = t;
    } else if (t < off2) {
      axis = 1;
      r = t - off1;
    } else {
      axis = 2;
      r = t - off2;
    }
    const int t1 = (axis == 0) ? 1 : 0, t2 = (axis == 2) ? 1 : 2;
    const int n1 = (t1 < D) ? g.n[t1] : 1, n2 = (t2 < D) ? g.n[t2] : 1;
    const long long per_c = (long long)n1 * n2;
    const int c = (int)(r / per_c);
    const long long q = r - (long long)c * per_c;
    int idx[3] = {1, 1, 1};
    idx[t1] = (int)(q % n1) + 1;
    idx[t2] = (int)(q / n1) + 1;
    idx[axis] = 0;
    const long long base = g.at(D, idx[0], idx[1], idx[2]);  // cell 0 of the line
    const long long sa = g.s[axis];
    const long long N = g.n[axis];
    T* f = U + (long long)c * g.field;
    for (int side = 0; side < 2; ++side) {
      const int type = P.bc[2 * axis + side];
      long long g0, g1, s0, s1;
      if (side == 0) {
        g0 = base;
        g1 = base - sa;
        s0 = (type == 3) ? base + N * sa : base + sa;
        s1 = (type == 3) ? base + (N - 1) * sa : base + 2 * sa;
      } else {
        g0 = base + (N + 1) * sa;
        g1 = base + (N + 2) * sa;
        s0 = (type == 3) ? base + sa : base + N * sa;
        s1 = (type == 3) ? base + 2 * sa : base + (N - 1) * sa;
      }
      if (type == 4) {  // inflow
        const T v = (T)P.inflow[2 * axis + side][c];
        f[g0] = v;
        f[g1] = v;
      } else if (type >= 1 && type <= 3) {
        f[g0] = f[s0];
        f[g1] = f[s1];
        if (type == 1 && c == 1 + axis) {  // reflective: negate normal momentum
          f[g0] = -f[s0];
          f[g1] = -f[s1];
        }
      } else {
        continue;
      }
      if (M) {
        T* m = M + (long long)c * g.field;
        m[g0] = f[g0];
        m[g1] = f[g1];
      }
    }
  }
}

// ------------------------------------------------------------------ K2 ---
// max over the interior of sqrt(sum m^2)/rho + cs, as a block reduction with
// warp shuffles, then an atomicMax on the bits of the (non-negative) double.
// The last block to finish turns the maximum into dt = courant*min(dx)/max,
// appends it to the optional trace and resets the accumulators for the next
// launch. NaNs are skipped as in the reference's `if (u > max_u)` update.
template <int D>
__global__ void __launch_bounds__(kCflBlock)
    cfl_kernel(DevParams P, const double* __restrict__ U, Geom g, double mdx, StepScratch s) {
  const long long n0 = g.n[0], n1 = g.n[1];
  const long long total = n0 * n1 * (long long)g.n[2];
  double m = 0.0;
  int bad = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n0) + 1;
    const long long q = t / n0;
    const int j = (int)(q % n1) + 1;
    const int k = (int)(q / n1) + 1;
    const long long o = g.at(D, i, j, k);
    double u[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) u[c] = U[(long long)c * g.field + o];
    double ss = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) ss = ss + u[1 + a] * u[1 + a];
    const double v = sqrt(ss) / u[0] + sound_speed<D>(P.G, u);
    if (v > m) m = v;
    if (!(u[0] > 0.0) || !isfinite(v)) bad = 1;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_down_sync(0xffffffffu, m, off);
    if (o > m) m = o;
    bad |= __shfl_down_sync(0xffffffffu, bad, off);
  }
  __shared__ double sm[kCflBlock / 32];
  __shared__ int sb[kCflBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sm[warp] = m;
    sb[warp] = bad;
  }
  __syncthreads();
  if (warp == 0) {
    m = (lane < kCflBlock / 32) ? sm[lane] : 0.0;
    bad = (lane < kCflBlock / 32) ? sb[lane] : 0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double o = __shfl_down_sync(0xffffffffu, m, off);
      if (o > m) m = o;
      bad |= __shfl_down_sync(0xffffffffu, bad, off);
    }
    if (lane == 0) {
      atomicMax(s.max_bits, (unsigned long long)__double_as_longlong(m));
      if (bad) atomicOr(s.status, 1);
      __threadfence();
      const unsigned int prev = atomicAdd(s.counter, 1u);
      if (prev == gridDim.x - 1) {
        __threadfence();
        const double mu = __longlong_as_double((long long)atomicAdd(s.max_bits, 0ull));
        const double dt = P.courant * mdx / mu;
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

// ------------------------------------------------------------------ K3 ---
// Pass 1 (loop 1 of the memory-intensive solver): limited slopes and
// half-step face states ul, ur of every cell with i_AX in [0, N+1] and
// interior transverse coordinates, along axis AX.
template <int D, int AX>
__device__ __forceinline__ void faces_body(const DevParams& P, const double* __restrict__ U,
                                           const Geom& g, double hdtdx, double* __restrict__ FS) {
  int e[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) e[a] = (a == AX) ? g.n[a] + 2 : g.n[a];
  const long long total = (long long)e[0] * e[1] * e[2];
  const long long F = g.field;
  const long long sa = g.s[AX];
  double* ul = FS + (long long)(AX * 2 + 0) * (D + 2) * F;
  double* ur = FS + (long long)(AX * 2 + 1) * (D + 2) * F;
  const double w = P.omega;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int c3[3];
    c3[0] = (int)(t % e[0]);
    const long long q = t / e[0];
    c3[1] = (int)(q % e[1]);
    c3[2] = (int)(q / e[1]);
#pragma unroll
    for (int a = 0; a < 3; ++a) c3[a] += (a == AX) ? 0 : 1;
    const long long o = g.at(D, c3[0], c3[1], c3[2]);
    double um[D + 2], u0[D + 2], up[D + 2], l[D + 2], r[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      const double* f = U + (long long)c * F + o;
      um[c] = f[-sa];
      u0[c] = f[0];
      up[c] = f[sa];
    }
    face_states<D, AX>(P.G, P.limiter, w, um, u0, up, hdtdx, l, r);
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      ul[(long long)c * F + o] = l[c];
      ur[(long long)c * F + o] = r[c];
    }
  }
}

template <int D>
__global__ void __launch_bounds__(kFaceBlock)
    faces_kernel(DevParams P, const double* __restrict__ U, Geom g, Dx dx, const double* dtp,
                 double* __restrict__ FS) {
  const double dt = *dtp;
  const int axis = blockIdx.y;
  if (axis == 0) faces_body<D, 0>(P, U, g, 0.5 * dt / dx.v[0], FS);
  if constexpr (D > 1) {
    if (axis == 1) faces_body<D, 1>(P, U, g, 0.5 * dt / dx.v[1], FS);
  }
  if constexpr (D > 2) {
    if (axis == 2) faces_body<D, 2>(P, U, g, 0.5 * dt / dx.v[2], FS);
  }
}

// Pass 2 (loop 2): exact Riemann problem between ur of cell i and ul of
// cell i+1 along AX, sampled at x/t = 0, and its flux, for i_AX in [0, N].
template <int D, int AX>
__device__ __forceinline__ void flux_body(const DevParams& P, const double* __restrict__ FS,
                                          const Geom& g, double* __restrict__ FR) {
  int e[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) e[a] = (a == AX) ? g.n[a] + 1 : g.n[a];
  const long long total = (long long)e[0] * e[1] * e[2];
  const long long F = g.field;
  const long long sa = g.s[AX];
  const double* ul = FS + (long long)(AX * 2 + 0) * (D + 2) * F;
  const double* ur = FS + (long long)(AX * 2 + 1) * (D + 2) * F;
  double* fr = FR + (long long)AX * (D + 2) * F;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int c3[3];
    c3[0] = (int)(t % e[0]);
    const long long q = t / e[0];
    c3[1] = (int)(q % e[1]);
    c3[2] = (int)(q / e[1]);
#pragma unroll
    for (int a = 0; a < 3; ++a) c3[a] += (a == AX) ? 0 : 1;
    const long long o = g.at(D, c3[0], c3[1], c3[2]);
    double l[D + 2], r[D + 2], f[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      l[c] = ur[(long long)c * F + o];
      r[c] = ul[(long long)c * F + o + sa];
    }
    interface_flux<D, AX>(P.G, P.rp, l, r, f);
#pragma unroll
    for (int c = 0; c < D + 2; ++c) fr[(long long)c * F + o] = f[c];
  }
}

template <int D>
__global__ void __launch_bounds__(kFluxBlock)
    flux_kernel(DevParams P, const double* __restrict__ FS, Geom g, double* __restrict__ FR) {
  const int axis = blockIdx.y;
  if (axis == 0) flux_body<D, 0>(P, FS, g, FR);
  if constexpr (D > 1) {
    if (axis == 1) flux_body<D, 1>(P, FS, g, FR);
  }
  if constexpr (D > 2) {
    if (axis == 2) flux_body<D, 2>(P, FS, g, FR);
  }
}

// Pass 3 (loop 3): U^{n+1} = U + ((X + Y) + Z) with X = dt/dx*(F(i-1)-F(i)),
// written to the other state buffer; or, for the cpu-intensive solver,
// ((U + X) + Y) + Z (rhyme_muscl_hancock_solve_cpu_intensive.f90:117-136).
template <int D>
__global__ void __launch_bounds__(kUpdBlock)
    update_kernel(DevParams P, const double* __restrict__ U, const double* __restrict__ FR,
                  Geom g, Dx dx, const double* dtp, double* __restrict__ Unew) {
  const double dt = *dtp;
  double dtdx[3];
#pragma unroll
  for (int a = 0; a < D; ++a) dtdx[a] = dt / dx.v[a];
  const long long n0 = g.n[0], n1 = g.n[1];
  const long long total = n0 * n1 * (long long)g.n[2];
  const long long F = g.field;
  const bool cpu_order = (P.solver_type == 1);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n0) + 1;
    const long long q = t / n0;
    const int j = (int)(q % n1) + 1;
    const int k = (int)(q / n1) + 1;
    const long long o = g.at(D, i, j, k);
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      double d[3];
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const double* fr = FR + ((long long)a * (D + 2) + c) * F + o;
        d[a] = dtdx[a] * (fr[-g.s[a]] - fr[0]);
      }
      const double u = U[(long long)c * F + o];
      double out;
      if (cpu_order) {
        out = u;
#pragma unroll
        for (int a = 0; a < D; ++a) out = out + d[a];
      } else {
        double acc = d[0];
#pragma unroll
        for (int a = 1; a < D; ++a) acc = acc + d[a];
        out = u + acc;
      }
      Unew[(long long)c * F + o] = out;
    }
  }
}

template <int D>
cudaError_t mh_solve_d(const DevParams& P, const double* U, double* Unew, const Geom& g,
                       const Dx& dx, const StepScratch& s, cudaStream_t st, cudaEvent_t* ev) {
  long long tot_f = 0, tot_r = 0;
  for (int a = 0; a < D; ++a) {
    long long f = 1, r = 1;
    for (int b = 0; b < 3; ++b) {
      f *= (b == a) ? g.n[b] + 2 : g.n[b];
      r *= (b == a) ? g.n[b] + 1 : g.n[b];
    }
    if (f > tot_f) tot_f = f;
    if (r > tot_r) tot_r = r;
  }
  if (ev) cudaEventRecord(ev[0], st);
  dim3 gf(grid_for(tot_f, kFaceBlock), D);
  faces_kernel<D><<<gf, kFaceBlock, 0, st>>>(P, U, g, dx, s.dt, s.faces);
  if (ev) cudaEventRecord(ev[1], st);
  dim3 gr(grid_for(tot_r, kFluxBlock), D);
  flux_kernel<D><<<gr, kFluxBlock, 0, st>>>(P, s.faces, g, s.fluxes);
  if (ev) cudaEventRecord(ev[2], st);
  const long long tot_u = (long long)g.n[0] * g.n[1] * g.n[2];
  update_kernel<D><<<grid_for(tot_u, kUpdBlock), kUpdBlock, 0, st>>>(P, U, s.fluxes, g, dx, s.dt,
                                                                     Unew);
  if (ev) cudaEventRecord(ev[3], st);
  return cudaGetLastError();
}

}  // namespace

int max_cfl_blocks() { return kMaxBlocks; }

template <typename T>
cudaError_t ghost_fill_any(const DevParams& P, T* U, T* U_mirror, const Geom& g, cudaStream_t st) {
  const int D = P.ndim;
  long long per_axis[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    long long t = D + 2;
    for (int b = 0; b < D; ++b)
      if (b != a) t *= g.n[b];
    per_axis[a] = t;
  }
  const long long off1 = per_axis[0], off2 = off1 + per_axis[1], total = off2 + per_axis[2];
  const int grid = grid_for(total, kFillBlock);
  switch (D) {
    case 1: ghost_fill_kernel<1, T><<<grid, kFillBlock, 0, st>>>(P, U, U_mirror, g, off1, off2, total); break;
    case 2: ghost_fill_kernel<2, T><<<grid, kFillBlock, 0, st>>>(P, U, U_mirror, g, off1, off2, total); break;
    case 3: ghost_fill_kernel<3, T><<<grid, kFillBlock, 0, st>>>(P, U, U_mirror, g, off1, off2, total); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_ghost_fill(const DevParams& P, double* U, double* U_mirror, const Geom& g,
                              cudaStream_t st) {
  return ghost_fill_any<double>(P, U, U_mirror, g, st);
}

cudaError_t launch_ghost_fill_f32(const DevParams& P, float* Uf, const Geom& g, cudaStream_t st) {
  return ghost_fill_any<float>(P, Uf, nullptr, g, st);
}

cudaError_t launch_cfl(const DevParams& P, const double* U, const Geom& g, const Dx& dx,
                       const StepScratch& s, cudaStream_t st) {
  const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
  int grid = grid_for(total, kCflBlock);
  if (grid > 152 * 4) grid = 152 * 4;
  switch (P.ndim) {
    case 1: cfl_kernel<1><<<grid, kCflBlock, 0, st>>>(P, U, g, dx.min, s); break;
    case 2: cfl_kernel<2><<<grid, kCflBlock, 0, st>>>(P, U, g, dx.min, s); break;
    case 3: cfl_kernel<3><<<grid, kCflBlock, 0, st>>>(P, U, g, dx.min, s); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_mh_solve(const DevParams& P, const double* U, double* Unew, const Geom& g,
                            const Dx& dx, const StepScratch& s, cudaStream_t st, cudaEvent_t* ev) {
  switch (P.ndim) {
    case 1: return mh_solve_d<1>(P, U, Unew, g, dx, s, st, ev);
    case 2: return mh_solve_d<2>(P, U, Unew, g, dx, s, st, ev);
    case 3: return mh_solve_d<3>(P, U, Unew, g, dx, s, st, ev);
  }
  return cudaErrorInvalidValue;
}

}  // namespace rgpu
