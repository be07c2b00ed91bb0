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

#include "box_elems.cuh"

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
    ghost_fill_kernel(BoxRules R, T* __restrict__ U, T* __restrict__ M, Geom g, long long off1,
                      long long off2, long long total, float* __restrict__ Mf) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x)
    ghost_elem<D, T>(R, U, M, g, off1, off2, t, Mf);
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
  const long long total = (long long)g.n[0] * g.n[1] * (long long)g.n[2];
  double m = 0.0;
  int bad = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const double v = signal_speed_elem<D>(P.G, U, g, t, bad);
    if (v > m) m = v;
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
// Pass 1: face states of every cell with i_AX in [0, N+1] (box_elems.cuh).
template <int D>
__global__ void __launch_bounds__(kFaceBlock)
    faces_kernel(DevParams P, BoxRules R, const double* __restrict__ U, Geom g, Dx dx,
                 const double* dtp, double* __restrict__ FS) {
  const double dt = *dtp;
  const int axis = blockIdx.y;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (axis == 0) {
    const double h = 0.5 * dt / dx.v[0];
    for (long long t = t0; t < face_count<0>(g); t += stride) faces_elem<D, 0>(P.G, R, U, g, h, FS, t);
  }
  if constexpr (D > 1) {
    if (axis == 1) {
      const double h = 0.5 * dt / dx.v[1];
      for (long long t = t0; t < face_count<1>(g); t += stride) faces_elem<D, 1>(P.G, R, U, g, h, FS, t);
    }
  }
  if constexpr (D > 2) {
    if (axis == 2) {
      const double h = 0.5 * dt / dx.v[2];
      for (long long t = t0; t < face_count<2>(g); t += stride) faces_elem<D, 2>(P.G, R, U, g, h, FS, t);
    }
  }
}

// Pass 2: exact Riemann problem and flux of every interface, i_AX in [0, N].
template <int D>
__device__ __forceinline__ void flux_pass(const DevParams& P, const double* __restrict__ FS, const Geom& g,
                                          double* __restrict__ FR) {
  const int axis = blockIdx.y;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (axis == 0)
    for (long long t = t0; t < iface_count<0>(g); t += stride) flux_elem<D, 0>(P.G, P.rp, FS, g, FR, t);
  if constexpr (D > 1) {
    if (axis == 1)
      for (long long t = t0; t < iface_count<1>(g); t += stride) flux_elem<D, 1>(P.G, P.rp, FS, g, FR, t);
  }
  if constexpr (D > 2) {
    if (axis == 2)
      for (long long t = t0; t < iface_count<2>(g); t += stride) flux_elem<D, 2>(P.G, P.rp, FS, g, FR, t);
  }
}

template <int D>
__global__ void __launch_bounds__(kFluxBlock)
    flux_kernel(DevParams P, const double* __restrict__ FS, Geom g, double* __restrict__ FR) {
  flux_pass<D>(P, FS, g, FR);
}

// The 3-D pass with at least 3 CTAs per SM (<= 168 registers, some spilled):
// the FP64 pipe needs the warps to hide its latency more than the solver
// needs the registers (at 216 registers and 2 CTAs per SM the 256^3 step
// was 5 % slower). In 1-D and 2-D the unbounded kernel is the faster one.
template <int D>
__global__ void __launch_bounds__(kFluxBlock, 3)
    flux_kernel_3cta(DevParams P, const double* __restrict__ FS, Geom g, double* __restrict__ FR) {
  flux_pass<D>(P, FS, g, FR);
}

// Pass 3: U^{n+1} of every interior cell, written to the other buffer.
template <int D>
__global__ void __launch_bounds__(kUpdBlock)
    update_kernel(DevParams P, const double* __restrict__ U, const double* __restrict__ FR,
                  Geom g, Dx dx, const double* dtp, double* __restrict__ Unew) {
  const double dt = *dtp;
  double dtdx[3];
#pragma unroll
  for (int a = 0; a < D; ++a) dtdx[a] = dt / dx.v[a];
  const long long total = (long long)g.n[0] * g.n[1] * (long long)g.n[2];
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x)
    update_elem<D>(P.solver_type, U, FR, g, dtdx, Unew, t);
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
  faces_kernel<D><<<gf, kFaceBlock, 0, st>>>(P, rules_of(P), U, g, dx, s.dt, s.faces);
  if (ev) cudaEventRecord(ev[1], st);
  dim3 gr(grid_for(tot_r, kFluxBlock), D);
  if constexpr (D == 3)
    flux_kernel_3cta<D><<<gr, kFluxBlock, 0, st>>>(P, s.faces, g, s.fluxes);
  else
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

template <int D, typename T>
cudaError_t ghost_fill_d(const BoxRules& R, T* U, T* U_mirror, const Geom& g, cudaStream_t st, float* Uf) {
  long long off1, off2, total;
  ghost_offsets<D>(g, off1, off2, total);
  ghost_fill_kernel<D, T><<<grid_for(total, kFillBlock), kFillBlock, 0, st>>>(R, U, U_mirror, g, off1, off2,
                                                                              total, Uf);
  return cudaGetLastError();
}

template <typename T>
cudaError_t ghost_fill_any(const DevParams& P, T* U, T* U_mirror, const Geom& g, cudaStream_t st,
                           float* Uf = nullptr) {
  const BoxRules R = rules_of(P);
  switch (P.ndim) {
    case 1: return ghost_fill_d<1, T>(R, U, U_mirror, g, st, Uf);
    case 2: return ghost_fill_d<2, T>(R, U, U_mirror, g, st, Uf);
    case 3: return ghost_fill_d<3, T>(R, U, U_mirror, g, st, Uf);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_ghost_fill(const DevParams& P, double* U, double* U_mirror, const Geom& g,
                              cudaStream_t st, float* Uf) {
  return ghost_fill_any<double>(P, U, U_mirror, g, st, Uf);
}

cudaError_t launch_ghost_fill_f32(const DevParams& P, float* Uf, const Geom& g, cudaStream_t st) {
  return ghost_fill_any<float>(P, Uf, nullptr, g, st);
}

namespace {
__global__ void set_double_kernel(double* dst, double v) { *dst = v; }
}  // namespace

cudaError_t launch_set_double(double* dst, double v, cudaStream_t st) {
  set_double_kernel<<<1, 1, 0, st>>>(dst, v);
  return cudaGetLastError();
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
