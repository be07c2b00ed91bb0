// kernels_paint.cu -- initial conditions painted on the device.
//
// The hydro part of rhyme_drawing_init.f90:20-78: the canvas, then the shapes
// in order (each overwrites the cells it covers), then the perturbations,
// summed per cell and added once as a conserved vector
// (rhyme_drawing_apply_perturbations.f90:74-185). Covered: uniform canvas
// (rhyme_drawing_uniform_canvas.f90), sharp cuboid
// (rhyme_drawing_sharp_cuboid.f90:44-60), sphere with tanh smoothing
// (rhyme_drawing_sphere.f90:85-110,189-209), smoothed 2-D slab
// (rhyme_drawing_smoothed_slab_2d.f90:33-85) and the harmonic and
// symmetric-decaying perturbations. One thread per interior cell.
#include "rgpu_internal.h"

namespace rgpu {

namespace {

template <int D>
__device__ __forceinline__ void to_cons(const Gas<double>& G, const double* w, double* u) {
  double v[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int a = 0; a < D; ++a) v[a] = w[1 + a];
  prim_vars_to_cons<D>(G, w[0], v, w[D + 1], u);
}

template <int D>
__global__ void __launch_bounds__(256)
    paint_kernel(const PaintShape* __restrict__ shapes, int n, Gas<double> G, Geom g, int le0, int le1, int le2,
                 double* __restrict__ U, float* __restrict__ Uf) {
  constexpr int K = D + 2;
  const double pi = 4.0 * atan(1.0);
  const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
  const int le[3] = {le0, le1, le2};
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int idx[3];
    idx[0] = (int)(t % g.n[0]) + 1;
    const long long q = t / g.n[0];
    idx[1] = (int)(q % g.n[1]) + 1;
    idx[2] = (int)(q / g.n[1]) + 1;
    const long long o = g.at(D, idx[0], idx[1], idx[2]);
    double u[K];
#pragma unroll
    for (int c = 0; c < K; ++c) u[c] = U[(long long)c * g.field + o];  // a transparent canvas keeps these
    // cell centres: box-local for the sphere (rhyme_drawing_sphere.f90:96),
    // level-0 coordinates for the slab and the perturbations
    double xl[3], xg[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      xl[a] = (double)idx[a] - 0.5;
      xg[a] = (double)idx[a] - 0.5 + (double)le[a] - 1.0;
    }
    double h[K], dterm[K];
    bool has_h = false, has_d = false;
#pragma unroll
    for (int c = 0; c < K; ++c) h[c] = dterm[c] = 0.0;
    for (int s = 0; s < n; ++s) {
      const PaintShape& S = shapes[s];
      switch (S.type) {
        case PAINT_CANVAS:
          to_cons<D>(G, S.prim[0], u);
          break;
        case PAINT_SHARP_CUBOID: {
          bool in = true;
#pragma unroll
          for (int a = 0; a < D; ++a) in = in && idx[a] >= S.lb[a] && idx[a] <= S.ub[a];
          if (in) to_cons<D>(G, S.prim[0], u);
          break;
        }
        case PAINT_SPHERE: {
          double ss = 0.0;
#pragma unroll
          for (int a = 0; a < D; ++a) {
            double d = xl[a] - S.origin[a];
            if (S.periodic) {
              d = fabs(d);
              const double e = (double)g.n[a] - d;
              if (e < d) d = e;
            }
            ss = ss + d * d;
          }
          const double dist = sqrt(ss);
          double f;
          if (S.sigma > 0.0) {
            f = (1.0 + tanh((S.r - dist) / S.sigma)) / 2.0;
          } else {
            f = (dist < S.r) ? 1.0 : 0.0;
            if (f == 0.0 && S.keep_outside) break;
          }
          double w[K];
#pragma unroll
          for (int c = 0; c < K; ++c) w[c] = f * S.prim[0][c] + (1.0 - f) * S.prim[1][c];
          to_cons<D>(G, w, u);
          break;
        }
        case PAINT_SMOOTHED_SLAB: {
          const double x = xg[S.axis];
          const double centre = (S.pos[0] + S.pos[1]) / 2.0;
          const double Rs = fabs(centre - S.pos[0]);
          const double factor =
              (1.0 + tanh((Rs - (x - centre)) / S.slab_sigma[0])) * (1.0 + tanh((Rs + (x - centre)) / S.slab_sigma[1]));
          double w[K];
#pragma unroll
          for (int c = 0; c < K; ++c) w[c] = S.prim[0][c] + 0.25 * (S.prim[1][c] - S.prim[0][c]) * factor;
          to_cons<D>(G, w, u);
          break;
        }
        case PAINT_HARMONIC: {
          const double kx = 2.0 * pi / S.wavelength * xg[S.axis] + S.phase;
          const double ak = S.amplitude * cos(kx);
#pragma unroll
          for (int c = 0; c < K; ++c) h[c] = h[c] + ak * S.base[c];
          has_h = true;
          break;
        }
        case PAINT_SYMMETRIC_DECAYING: {
          const double xr = xg[S.axis] - S.pos[0];
          const double ad = S.amplitude * exp(-(xr * xr) / S.sigma);
#pragma unroll
          for (int c = 0; c < K; ++c) dterm[c] = dterm[c] + ad * S.base[c];
          has_d = true;
          break;
        }
        default:
          break;
      }
    }
    if (has_h || has_d) {
      double w[K], du[K];
#pragma unroll
      for (int c = 0; c < K; ++c) w[c] = has_h ? (has_d ? h[c] * dterm[c] : h[c]) : dterm[c];
      to_cons<D>(G, w, du);
#pragma unroll
      for (int c = 0; c < K; ++c) u[c] = u[c] + du[c];
    }
#pragma unroll
    for (int c = 0; c < K; ++c) {
      U[(long long)c * g.field + o] = u[c];
      if (Uf) Uf[(long long)c * g.field + o] = mirror_of(u[c]);
    }
  }
}

}  // namespace

cudaError_t launch_paint(int ndim, const PaintShape* shapes, int n, const Gas<double>& G, const Geom& g,
                         const int* left_edge, double* U, float* Uf, cudaStream_t st) {
  const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
  long long blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  switch (ndim) {
    case 1: paint_kernel<1><<<(int)blocks, 256, 0, st>>>(shapes, n, G, g, left_edge[0], left_edge[1], left_edge[2], U, Uf); break;
    case 2: paint_kernel<2><<<(int)blocks, 256, 0, st>>>(shapes, n, G, g, left_edge[0], left_edge[1], left_edge[2], U, Uf); break;
    case 3: paint_kernel<3><<<(int)blocks, 256, 0, st>>>(shapes, n, G, g, left_edge[0], left_edge[1], left_edge[2], U, Uf); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace rgpu
