// box_elems.cuh -- per-element bodies of the plain FP64 box kernels.
//
// Each function processes element t of one box's index space for one pass
// (a ghost line, a cell's face states, an interface, a cell update). The
// single-box kernels (kernels_box.cu) run them over a grid-stride range; the
// batched kernels (kernels_batch.cu) run them over (box, chunk) work items of
// a box table. Both therefore execute the same arithmetic, so a box stepped
// alone and inside a batch gives bit-identical results.
#pragma once

#include "rgpu_internal.h"

namespace rgpu {

// Per-box values of the boundary and limiter modules.
struct BoxRules {
  int bc[6];
  double inflow[6][5];
  int limiter;
  double omega;
  int solver_type;
};

__host__ __device__ inline BoxRules rules_of(const DevParams& P) {
  BoxRules r;
  for (int i = 0; i < 6; ++i) {
    r.bc[i] = P.bc[i];
    for (int c = 0; c < 5; ++c) r.inflow[i][c] = P.inflow[i][c];
  }
  r.limiter = P.limiter;
  r.omega = P.omega;
  r.solver_type = P.solver_type;
  return r;
}

// Ghost lines of a box: axis a contributes (D+2) * prod_{b != a} n_b lines.
template <int D>
__host__ __device__ inline void ghost_offsets(const Geom& g, long long& off1, long long& off2,
                                              long long& total) {
  long long per_axis[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    long long t = D + 2;
    for (int b = 0; b < D; ++b)
      if (b != a) t *= g.n[b];
    per_axis[a] = t;
  }
  off1 = per_axis[0];
  off2 = off1 + per_axis[1];
  total = off2 + per_axis[2];
}

// K1 element: fills the left then the right 2-cell ghost layer of one line
// (axis, component, transverse position) in the order of
// rhyme_samr_bc_set_boundaries.f90:9-20; writes U and (if given) M.
// M (optional) receives the same ghost values (the other state buffer); Mf
// (optional) their FP32 images (the mirror of the mixed form), equal to what
// a fill of the mirror from its own interior would write.
template <int D, typename T>
__device__ __forceinline__ void ghost_elem(const BoxRules& R, T* __restrict__ U, T* __restrict__ M,
                                           const Geom& g, long long off1, long long off2, long long t,
                                           float* __restrict__ Mf = nullptr) {
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
  int i1 = (int)(q % n1) + 1, i2 = (int)(q / n1) + 1;
  int idx0 = 1, idx1 = 1, idx2 = 1;
  if (t1 == 0) idx0 = i1; else idx1 = i1;
  if (t2 == 1) idx1 = i2; else idx2 = i2;
  if (axis == 0) idx0 = 0; else if (axis == 1) idx1 = 0; else idx2 = 0;
  const long long base = g.at(D, idx0, idx1, idx2);  // cell 0 of the line
  const long long sa = g.s[axis];
  const long long N = g.n[axis];
  T* f = U + (long long)c * g.field;
  for (int side = 0; side < 2; ++side) {
    const int type = R.bc[2 * axis + side];
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
      const T v = (T)R.inflow[2 * axis + side][c];
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
    if (Mf) {
      float* m = Mf + (long long)c * g.field;
      m[g0] = mirror_of(f[g0]);
      m[g1] = mirror_of(f[g1]);
    }
  }
}

// Extents of the face (cells 0..N+1 along AX) and interface (0..N) passes.
template <int AX>
__host__ __device__ inline long long face_count(const Geom& g) {
  long long t = 1;
  for (int a = 0; a < 3; ++a) t *= (a == AX) ? g.n[a] + 2 : g.n[a];
  return t;
}
template <int AX>
__host__ __device__ inline long long iface_count(const Geom& g) {
  long long t = 1;
  for (int a = 0; a < 3; ++a) t *= (a == AX) ? g.n[a] + 1 : g.n[a];
  return t;
}

template <int D, int AX>
__device__ __forceinline__ long long pass_offset(const Geom& g, int extra, long long t) {
  int e[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) e[a] = (a == AX) ? g.n[a] + extra : g.n[a];
  int c0 = (int)(t % e[0]);
  const long long q = t / e[0];
  int c1 = (int)(q % e[1]);
  int c2 = (int)(q / e[1]);
  if (AX != 0) c0 += 1;
  if (AX != 1) c1 += 1;
  if (AX != 2) c2 += 1;
  return g.at(D, c0, c1, c2);
}

// K3a element: limited slopes and half-step face states of one cell
// (loop 1 of rhyme_muscl_hancock_solve_memory_intensive.f90:56-98).
template <int D, int AX>
__device__ __forceinline__ void faces_elem(const Gas<double>& G, const BoxRules& R,
                                           const double* __restrict__ U, const Geom& g, double hdtdx,
                                           double* __restrict__ FS, long long t) {
  const long long F = g.field;
  const long long sa = g.s[AX];
  double* ul = FS + (long long)(AX * 2 + 0) * (D + 2) * F;
  double* ur = FS + (long long)(AX * 2 + 1) * (D + 2) * F;
  const long long o = pass_offset<D, AX>(g, 2, t);
  double um[D + 2], u0[D + 2], up[D + 2], l[D + 2], r[D + 2];
#pragma unroll
  for (int c = 0; c < D + 2; ++c) {
    const double* f = U + (long long)c * F + o;
    um[c] = f[-sa];
    u0[c] = f[0];
    up[c] = f[sa];
  }
  face_states<D, AX>(G, R.limiter, R.omega, um, u0, up, hdtdx, l, r);
#pragma unroll
  for (int c = 0; c < D + 2; ++c) {
    ul[(long long)c * F + o] = l[c];
    ur[(long long)c * F + o] = r[c];
  }
}

// K3b element: exact Riemann problem at x/t = 0 and its flux for one
// interface (loop 2, :107-140).
template <int D, int AX>
__device__ __forceinline__ void flux_elem(const Gas<double>& G, const Rp<double>& rp,
                                          const double* __restrict__ FS, const Geom& g,
                                          double* __restrict__ FR, long long t) {
  const long long F = g.field;
  const long long sa = g.s[AX];
  const double* ul = FS + (long long)(AX * 2 + 0) * (D + 2) * F;
  const double* ur = FS + (long long)(AX * 2 + 1) * (D + 2) * F;
  double* fr = FR + (long long)AX * (D + 2) * F;
  const long long o = pass_offset<D, AX>(g, 1, t);
  double l[D + 2], r[D + 2], f[D + 2];
#pragma unroll
  for (int c = 0; c < D + 2; ++c) {
    l[c] = ur[(long long)c * F + o];
    r[c] = ul[(long long)c * F + o + sa];
  }
  interface_flux<D, AX, double, true>(G, rp, l, r, f);
#pragma unroll
  for (int c = 0; c < D + 2; ++c) fr[(long long)c * F + o] = f[c];
}

// K3c element: U^{n+1} of one interior cell, U + ((X + Y) + Z) or, for the
// cpu-intensive solver, ((U + X) + Y) + Z (loop 3, :148-180;
// rhyme_muscl_hancock_solve_cpu_intensive.f90:117-136).
template <int D>
__device__ __forceinline__ void update_elem(int solver_type, const double* __restrict__ U,
                                            const double* __restrict__ FR, const Geom& g,
                                            const double* dtdx, double* __restrict__ Unew,
                                            long long t) {
  const long long n0 = g.n[0], n1 = g.n[1];
  const int i = (int)(t % n0) + 1;
  const long long q = t / n0;
  const int j = (int)(q % n1) + 1;
  const int k = (int)(q / n1) + 1;
  const long long o = g.at(D, i, j, k);
  const long long F = g.field;
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
    if (solver_type == 1) {
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

// Signal speed |v| + cs of one interior cell for the CFL maximum
// (rhyme_cfl_time_step.f90:77-84); sets bad for non-positive density or a
// non-finite value.
template <int D>
__device__ __forceinline__ double signal_speed_elem(const Gas<double>& G, const double* __restrict__ U,
                                                    const Geom& g, long long t, int& bad) {
  const long long n0 = g.n[0], n1 = g.n[1];
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
  const double v = sqrt(ss) / u[0] + sound_speed<D>(G, u);
  if (!(u[0] > 0.0) || !isfinite(v)) bad = 1;
  return v;
}

}  // namespace rgpu
