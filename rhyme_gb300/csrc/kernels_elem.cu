// kernels_elem.cu -- element-level kernels: the same device functions as the
// box solver applied to n independent inputs, for the Fortran interfaces that
// Rhyme's unit tests call directly (rhyme_riemann_problem_solve,
// rhyme_irs_exec, rhyme_slope_limiter_run,
// rhyme_muscl_hancock_half_step_extrapolation). Compiled with --fmad=false.
#include "rgpu_internal.h"

namespace rgpu {

namespace {

constexpr int kBlock = 128;

inline int grid_for(long long n) {
  long long b = (n + kBlock - 1) / kBlock;
  if (b < 1) b = 1;
  if (b > 152 * 64) b = 152 * 64;
  return (int)b;
}

template <int D>
__global__ void __launch_bounds__(kBlock)
    riemann_solve_kernel(DevParams P, const double* __restrict__ l, const double* __restrict__ r,
                         long long n, double dxdt, int axis, double* __restrict__ u) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double a[D + 2], b[D + 2], o[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      a[c] = l[i * (D + 2) + c];
      b[c] = r[i * (D + 2) + c];
    }
    if (axis == 0) rp_solve<D, 0>(P.G, P.rp, a, b, dxdt, o);
    if constexpr (D > 1) {
      if (axis == 1) rp_solve<D, 1>(P.G, P.rp, a, b, dxdt, o);
    }
    if constexpr (D > 2) {
      if (axis == 2) rp_solve<D, 2>(P.G, P.rp, a, b, dxdt, o);
    }
#pragma unroll
    for (int c = 0; c < D + 2; ++c) u[i * (D + 2) + c] = o[c];
  }
}

__global__ void __launch_bounds__(kBlock)
    irs_exec_kernel(DevParams P, const double* __restrict__ s, long long n, double* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double* q = s + i * 8;
    double lf = 0.0, rf = 0.0;
    const double p = irs_exec<double, false>(P.G, P.rp.tol, P.rp.n_iter, q[0], q[1], q[2], q[3], lf, q[4], q[5],
                              q[6], q[7], rf);
    out[i * 3 + 0] = p;
    out[i * 3 + 1] = lf;
    out[i * 3 + 2] = rf;
  }
}

__global__ void __launch_bounds__(kBlock)
    slope_limiter_kernel(DevParams P, const double* __restrict__ ul, const double* __restrict__ u,
                         const double* __restrict__ ur, long long n, double* __restrict__ d) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    d[i] = limited_slope(P.limiter, P.omega, ul[i], u[i], ur[i]);
}

template <int D>
__global__ void __launch_bounds__(kBlock)
    half_step_kernel(DevParams P, const double* __restrict__ u, const double* __restrict__ delta,
                     long long n, int axis, double hdtdx, double* __restrict__ l,
                     double* __restrict__ r) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double a[D + 2], d[D + 2], lo[D + 2], ro[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      a[c] = u[i * (D + 2) + c];
      d[c] = delta[i * (D + 2) + c];
    }
    if (axis == 0) half_step<D, 0>(P.G, a, d, hdtdx, lo, ro);
    if constexpr (D > 1) {
      if (axis == 1) half_step<D, 1>(P.G, a, d, hdtdx, lo, ro);
    }
    if constexpr (D > 2) {
      if (axis == 2) half_step<D, 2>(P.G, a, d, hdtdx, lo, ro);
    }
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      l[i * (D + 2) + c] = lo[c];
      r[i * (D + 2) + c] = ro[c];
    }
  }
}

}  // namespace

cudaError_t launch_riemann_solve(const DevParams& P, const double* l, const double* r, long long n,
                                 double dxdt, int axis, double* u, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  switch (P.ndim) {
    case 1: riemann_solve_kernel<1><<<grid_for(n), kBlock, 0, st>>>(P, l, r, n, dxdt, axis, u); break;
    case 2: riemann_solve_kernel<2><<<grid_for(n), kBlock, 0, st>>>(P, l, r, n, dxdt, axis, u); break;
    case 3: riemann_solve_kernel<3><<<grid_for(n), kBlock, 0, st>>>(P, l, r, n, dxdt, axis, u); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_irs_exec(const DevParams& P, const double* states, long long n, double* out,
                            cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  irs_exec_kernel<<<grid_for(n), kBlock, 0, st>>>(P, states, n, out);
  return cudaGetLastError();
}

cudaError_t launch_slope_limiter(const DevParams& P, const double* ul, const double* u,
                                 const double* ur, long long n, double* delta, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  slope_limiter_kernel<<<grid_for(n), kBlock, 0, st>>>(P, ul, u, ur, n, delta);
  return cudaGetLastError();
}

cudaError_t launch_half_step(const DevParams& P, const double* u, const double* delta, long long n,
                             int axis, double hdtdx, double* l, double* r, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  switch (P.ndim) {
    case 1: half_step_kernel<1><<<grid_for(n), kBlock, 0, st>>>(P, u, delta, n, axis, hdtdx, l, r); break;
    case 2: half_step_kernel<2><<<grid_for(n), kBlock, 0, st>>>(P, u, delta, n, axis, hdtdx, l, r); break;
    case 3: half_step_kernel<3><<<grid_for(n), kBlock, 0, st>>>(P, u, delta, n, axis, hdtdx, l, r); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace rgpu
