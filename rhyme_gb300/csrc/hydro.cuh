// hydro.cuh -- device functions of the MUSCL-Hancock step: ideal-gas EOS,
// slope limiters, half-step extrapolation and the exact Riemann solver.
//
// Templated on NDIM (D), on the normal axis (AX, compile-time so no state
// vector is indexed dynamically) and on the arithmetic type T (double for the
// plain path, float for the FP32 stages of the mixed path). Each routine keeps
// the floating-point evaluation order of the Fortran routine it restates
// (operators of equal precedence left to right), so that with FMA contraction
// disabled the double instantiation performs the same IEEE operations as the
// reference; the only intended difference is that the six p* guesses of
// rhyme_irs_guess_p_star.f90 are evaluated lazily, in order, when the Newton
// iteration from the previous guess fails (identical values, less work).
//
// State vectors are (rho, m_1..m_D, E); reference paths are relative to
// Rhyme's src/.
#pragma once

#include <cfloat>
#include <cstdint>

#include "libm_pow.h"

namespace rgpu {

// ---- math by type --------------------------------------------------------
// Double powers go through libm_pow::pow, a restatement of the C library's
// pow that the compiled reference calls for every real `**`, so the FP64 path
// returns the reference's bits even in flows that amplify a one-ulp
// difference.
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_pow(double x, double y) { return libm_pow::pow(x, y); }
// Float powers as 2^(y log2 x) with CUDA's log2f and exp2f: the rounding of
// the product adds a relative error of about 2^-24 |y log2 x| to the result
// (for the positive bases of this path), against powf's ~1 ulp, for a
// fraction of its instructions; two powers of one base share the logarithm.
__device__ __forceinline__ float m_pow(float x, float y) { return exp2f(y * log2f(x)); }
// x**y1 and x**y2 of one base (one logarithm).
__device__ __forceinline__ void m_pow2(double x, double y1, double y2, double& r1, double& r2) {
  libm_pow::pow2(x, y1, y2, &r1, &r2);
}
__device__ __forceinline__ void m_pow2(float x, float y1, float y2, float& r1, float& r2) {
  const float l = log2f(x);
  r1 = exp2f(y1 * l);
  r2 = exp2f(y2 * l);
}
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }

template <typename T> struct Limits;
template <> struct Limits<double> {
  __device__ static constexpr double tiny() { return DBL_MIN; }
};
template <> struct Limits<float> {
  __device__ static constexpr float tiny() { return FLT_MIN; }
};

// Fortran MAX/MIN of two reals (same ternary as the CPU oracle).
template <typename T> __device__ __forceinline__ T fmax_ref(T a, T b) { return (b > a) ? b : a; }
template <typename T> __device__ __forceinline__ T fmin_ref(T a, T b) { return (b < a) ? b : a; }

// Ideal-gas constants (rhyme_riemann_problem_init.f90:20-27,
// rhyme_irs_init.f90:21-27) plus the literal quotients the reference
// recomputes at each use (2/gp1, 2/gm1, 1/gm1_2g, gm1/2): the same values.
template <typename T>
struct Gas {
  T g, gm1, gp1, gm1_gp1, gm1_2g, gp1_2g, g_inv, kb_amu;
  T two_gp1, two_gm1, inv_gm1_2g, gm1_half, half_gm1, g_kb_amu;
};

// Run parameters used inside kernels.
template <typename T>
struct Rp {
  T vac_rho, vac_p, vac_rho_next;  // w_vacuum(rho), w_vacuum(p), nearest(w_vac_rho, +1)
  T tol;
  int n_iter;
};

struct Limiter {
  int type;
  double w;
};

// ---- EOS: rhyme_hydro_base / rhyme_ideal_gas ------------------------------

// rhyme_hydro_base_specific_kinetic_energy.f90:9
template <int D, typename T>
__device__ __forceinline__ T sp_kin_e(const T* u) {
  T s = T(0);
#pragma unroll
  for (int a = 0; a < D; ++a) s = s + u[1 + a] * u[1 + a];
  return (T(0.5) * s) / (u[0] * u[0]);
}

// rhyme_hydro_base_specific_internal_energy.f90:9
template <int D, typename T>
__device__ __forceinline__ T sp_int_e(const T* u) {
  return u[D + 1] / u[0] - sp_kin_e<D>(u);
}

// The FP32 forms of the mixed sweeps (pressure, sound speed, flux) are the
// same quantities with fewer divisions: p = (E - |m|^2 / (2 rho)) (gamma-1)
// for rho e_int (gamma-1), cs = sqrt(gamma p / rho) for
// sqrt(gamma kB/amu T/mu), and the flux from one reciprocal of rho. FP32
// division is a reciprocal and a multiply plus range handling; the sweeps
// divide a lot (256^3 mixed step 2.43 -> 2.20 ms, L1(rho) against FP64 a
// little lower). The double forms keep the reference's operations.

// rhyme_ideal_gas_pressure.f90:9
template <int D, typename T>
__device__ __forceinline__ T pressure(const Gas<T>& G, const T* u) {
  if constexpr (sizeof(T) == sizeof(float)) {
    T s = T(0);
#pragma unroll
    for (int a = 0; a < D; ++a) s = s + u[1 + a] * u[1 + a];
    return (u[D + 1] - T(0.5) * s / u[0]) * G.gm1;
  }
  return u[0] * sp_int_e<D>(u) * G.gm1;
}

// rhyme_ideal_gas_temperature_per_mu.f90:9-10, _speed_of_sound.f90:9
template <int D, typename T>
__device__ __forceinline__ T sound_speed(const Gas<T>& G, const T* u) {
  if constexpr (sizeof(T) == sizeof(float)) return m_sqrt(G.g * pressure<D>(G, u) / u[0]);
  T t_mu = sp_int_e<D>(u) * G.gm1 / G.kb_amu;
  return m_sqrt(G.g_kb_amu * t_mu);
}

// rhyme_ideal_gas_flux.f90:12-23 along axis AX
template <int D, int AX, typename T>
__device__ __forceinline__ void flux(const Gas<T>& G, const T* u, T* f) {
  if (m_abs(u[0]) < Limits<T>::tiny()) {
#pragma unroll
    for (int c = 0; c < D + 2; ++c) f[c] = T(0);
    return;
  }
  if constexpr (sizeof(T) == sizeof(float)) {
    const T inv = T(1) / u[0];
    T s = T(0);
#pragma unroll
    for (int a = 0; a < D; ++a) s = s + u[1 + a] * u[1 + a];
    const T p = (u[D + 1] - T(0.5) * s * inv) * G.gm1;
    const T vn = u[1 + AX] * inv;
    f[0] = u[1 + AX];
#pragma unroll
    for (int a = 0; a < D; ++a) f[1 + a] = u[1 + a] * vn;
    f[1 + AX] = f[1 + AX] + p;
    f[D + 1] = vn * (u[D + 1] + p);
    return;
  }
  T p = pressure<D>(G, u);
  f[0] = u[1 + AX];
#pragma unroll
  for (int a = 0; a < D; ++a) f[1 + a] = u[1 + a] * f[0] / u[0];
  f[1 + AX] = f[1 + AX] + p;
  f[D + 1] = f[0] / u[0] * (u[D + 1] + p);
}

// rhyme_ideal_gas_primitive_vars_to_conserved.f90:9-11
template <int D, typename T>
__device__ __forceinline__ void prim_vars_to_cons(const Gas<T>& G, T rho, const T* v, T p, T* u) {
  u[0] = rho;
  T s = T(0);
#pragma unroll
  for (int a = 0; a < D; ++a) {
    u[1 + a] = rho * v[a];
    s = s + v[a] * v[a];
  }
  u[D + 1] = T(0.5) * rho * s + p / G.gm1;
}

// ---- slope limiter: rhyme_slope_limiter*.f90 -------------------------------

// rhyme_slope_limiter_xi_r.f90:11
template <typename T>
__device__ __forceinline__ T xi_r(T w, T r) {
  return T(2) / (T(1) - w + (T(1) + w) * r);
}

// r (rhyme_slope_limiter.f90:62-82) and delta of the four limiters
// (van Leer :13-27, minmod :13-29, van Albada :13-27, superbee :13-31).
template <typename T>
__device__ __forceinline__ T limited_slope(int type, T w, T ul, T u, T ur) {
  T d_L = u - ul;
  T d_R = ur - u;
  T d = T(0.5) * (T(1) + w) * d_L + T(0.5) * (T(1) + w) * d_R;
  T denom = ur - u;
  T r = (m_abs(denom) < Limits<T>::tiny()) ? T(0) : (u - ul) / denom;
  if (type == 1) {  // van Leer
    return (r > T(0)) ? fmin_ref(T(2) * r / (T(1) + r), xi_r(w, r)) * d : T(0);
  } else if (type == 2) {  // minmod
    if (r > T(1)) return fmin_ref(T(1), xi_r(w, r)) * d;
    if (r > T(0)) return r * d;
    return T(0);
  } else if (type == 3) {  // van Albada; r**2.d0 folds to r*r
    if constexpr (sizeof(T) == sizeof(float)) {
      // r(1+r)/(1+r^2) is 1 to float precision once r > 2^24, and beyond
      // ~1.8e19 both products overflow and give inf/inf = NaN: take the
      // limit. (A noise-level d_R against a resolved d_L reaches such r in
      // the mixed form's FP32 state; the FP64 path keeps the literal form.)
      const T phi = (r < T(1e18f)) ? r * (T(1) + r) / (T(1) + r * r) : T(1);
      return (r > T(0)) ? fmin_ref(phi, xi_r(w, r)) * d : T(0);
    }
    return (r > T(0)) ? fmin_ref(r * (T(1) + r) / (T(1) + r * r), xi_r(w, r)) * d : T(0);
  } else {  // superbee
    if (r > T(1)) return fmin_ref(fmin_ref(r, xi_r(w, r)), T(2)) * d;
    if (r > T(0.5)) return d;
    if (r > T(0)) return T(2) * r * d;
    return T(0);
  }
}

// rhyme_muscl_hancock_half_step_extrapolation.f90:15-21; hdtdx = (.5*dt)/dx
template <int D, int AX, typename T>
__device__ __forceinline__ void half_step(const Gas<T>& G, const T* u, const T* delta, T hdtdx,
                                          T* l, T* r) {
  T fl[D + 2], fr[D + 2];
#pragma unroll
  for (int c = 0; c < D + 2; ++c) {
    l[c] = u[c] - T(0.5) * delta[c];
    r[c] = u[c] + T(0.5) * delta[c];
  }
  flux<D, AX>(G, l, fl);
  flux<D, AX>(G, r, fr);
#pragma unroll
  for (int c = 0; c < D + 2; ++c) {
    T df = fl[c] - fr[c];
    l[c] = l[c] + hdtdx * df;
    r[c] = r[c] + hdtdx * df;
  }
}

// Face states of one cell along AX from its neighbours um, u0, up.
template <int D, int AX, typename T>
__device__ __forceinline__ void face_states(const Gas<T>& G, int lim, T w, const T* um, const T* u0,
                                            const T* up, T hdtdx, T* l, T* r) {
  T delta[D + 2];
#pragma unroll
  for (int c = 0; c < D + 2; ++c) delta[c] = limited_slope(lim, w, um[c], u0[c], up[c]);
  half_step<D, AX>(G, u0, delta, hdtdx, l, r);
}

// ---- exact Riemann solver: rhyme_irs_*, rhyme_riemann_problem_* -----------

// Loop-invariant terms of rhyme_irs_nonlinear_wave_function.f90:15-23 for one
// side (Ak, Bk, 2cs/gm1, 1/(rho cs)): the reference recomputes them every
// Newton iteration with the same operations, so computing them once gives the
// same values. With LAZY (double only) the pair a branch needs is formed on
// its first use (a side usually stays a shock or a rarefaction through the
// iteration, and FP64 divisions are scarce on GB300): the plain FP64 flux
// kernels take it (2-D slab 117 -> 126 M cell-updates/s); the FP64 fix-up of
// the mixed form does not (its kernel would spill, and the mixed batch and
// the server's latency suffered); float forms all four up front.
template <typename T>
struct WaveSide {
  T rho, p, cs, Ak, Bk, c2g, irc;
  bool shock_ready, fan_ready;
};

template <typename T>
__device__ __forceinline__ void wave_shock_terms(const Gas<T>& G, WaveSide<T>& w) {
  w.Ak = T(2) / (G.gp1 * w.rho);
  w.Bk = G.gm1 * w.p / G.gp1;
  w.shock_ready = true;
}

template <typename T>
__device__ __forceinline__ void wave_fan_terms(const Gas<T>& G, WaveSide<T>& w) {
  w.c2g = T(2) * w.cs / G.gm1;
  w.irc = T(1) / (w.rho * w.cs);
  w.fan_ready = true;
}

template <typename T, bool LAZY>
__device__ __forceinline__ WaveSide<T> wave_side(const Gas<T>& G, T s_rho, T s_p, T s_cs) {
  WaveSide<T> w;
  w.rho = s_rho;
  w.p = s_p;
  w.cs = s_cs;
  w.shock_ready = w.fan_ready = false;
  if constexpr (!LAZY) {
    wave_shock_terms(G, w);
    wave_fan_terms(G, w);
  }
  return w;
}

// rhyme_irs_nonlinear_wave_function.f90:13-24
template <typename T, bool LAZY>
__device__ __forceinline__ void nonlinear_wave(const Gas<T>& G, WaveSide<T>& w, T p, T& f, T& fprime) {
  if (p > w.p) {
    if constexpr (LAZY) {
      if (!w.shock_ready) wave_shock_terms(G, w);
    }
    const T bp = w.Bk + p;
    const T factor = m_sqrt(w.Ak / bp);
    f = (p - w.p) * factor;
    fprime = factor * (T(1) - (p - w.p) / (T(2) * bp));
  } else if constexpr (sizeof(T) == sizeof(float)) {
    // (p/p_k)^e - 1 as expm1(e log1p((p - p_k)/p_k)): the same quantity
    // without the cancellation of the literal form when p is close to p_k
    // (a float power near 1 carries an ulp of 1, a large relative error of
    // the difference); p - p_k is exact there.
    const float t = log1pf((p - w.p) / w.p);
    f = w.c2g * expm1f(G.gm1_2g * t);
    fprime = w.irc * expf(-G.gp1_2g * t);
  } else {
    if constexpr (LAZY) {
      if (!w.fan_ready) wave_fan_terms(G, w);
    }
    T y, z;
    m_pow2(p / w.p, G.gm1_2g, -G.gp1_2g, y, z);
    f = w.c2g * (y - T(1));
    fprime = w.irc * z;
  }
}

// Guess 0 of rhyme_irs_guess_p_star.f90:14-38 (the adaptive PVRS /
// two-rarefaction / two-shock choice), not yet floored.
template <typename T>
__device__ __forceinline__ T guess_p_star_adaptive(const Gas<T>& G, T l_rho, T vl, T l_p, T l_cs, T r_rho, T vr,
                                                   T r_p, T r_cs) {
  T p;
  const T q_user = T(2);
  T cup = T(0.25) * (l_rho + r_rho) * (l_cs + r_cs);
  T ppv = fmax_ref(T(0.5) * (l_p + r_p) + T(0.5) * (vl - vr) * cup, T(0));
  T p_min = fmin_ref(l_p, r_p);
  T p_max = fmax_ref(l_p, r_p);
  T q_max = p_max / p_min;
  if (q_max <= q_user && (p_min < ppv && ppv < p_max)) {
    p = ppv;  // PVRS
  } else if (ppv < p_min) {  // two-rarefaction
    T pq = m_pow(l_p / r_p, G.gm1_2g);
    T um = (pq * vl / l_cs + vr / r_cs + G.two_gm1 * (pq - T(1))) / (pq / l_cs + T(1) / r_cs);
    T ptl = T(1) + G.half_gm1 * (vl - um) / l_cs;
    T ptr = T(1) + G.half_gm1 * (um - vr) / r_cs;
    p = T(0.5) * (l_p * m_pow(ptl, G.inv_gm1_2g) + r_p * m_pow(ptr, G.inv_gm1_2g));
  } else {  // two-shock
    T gel = m_sqrt((G.two_gp1 / l_rho) / (G.gm1_gp1 * l_p + ppv));
    T ger = m_sqrt((G.two_gp1 / r_rho) / (G.gm1_gp1 * r_p + ppv));
    p = (gel * l_p + ger * r_p - (vr - vl)) / (gel + ger);
  }
  return p;
}

// Guess number k (0..5) of rhyme_irs_guess_p_star.f90:14-71, floored at tiny.
template <typename T>
__device__ __noinline__ T guess_p_star(const Gas<T>& G, int k, T l_rho, T vl, T l_p, T l_cs, T r_rho,
                                       T vr, T r_p, T r_cs) {
  T p;
  if (k == 0) {
    p = guess_p_star_adaptive(G, l_rho, vl, l_p, l_cs, r_rho, vr, r_p, r_cs);
  } else if (k == 1) {  // Ramses
    p = (r_rho * r_cs * l_p + l_rho * l_cs * r_p + r_cs * l_cs * (l_rho * vl - r_rho * vr)) /
        (r_rho * r_cs + l_rho * l_cs);
  } else if (k == 2) {  // two-rarefaction approximation
    p = m_pow((l_cs + r_cs - G.gm1_half * (vr - vl)) /
                  (m_pow(l_cs / l_p, G.gm1_2g) + m_pow(r_cs / r_p, G.gm1_2g)),
              G.inv_gm1_2g);
  } else if (k == 3) {  // two-shock approximation; g_K at :74-80
    T l_g = m_sqrt((T(2) / (G.gp1 * l_rho)) / (l_p + G.gm1_gp1 * l_p));
    T r_g = m_sqrt((T(2) / (G.gp1 * r_rho)) / (r_p + G.gm1_gp1 * r_p));
    p = (l_g * l_p + r_g * r_p - (vr - vl)) / (l_g + r_g);
  } else if (k == 4) {  // p_PV
    p = T(0.5) * (l_p + r_p) - T(0.125) * (vr - vl) * (l_rho + r_rho) * (l_cs + r_cs);
  } else {  // arithmetic mean
    p = T(0.5) * (l_p + r_p);
  }
  return fmax_ref(p, Limits<T>::tiny());
}

// rhyme_irs_exec.f90:19-44 with lazily evaluated guesses. l_f / r_f are the
// wave functions at the last iterate before the final update.
template <typename T, bool LAZY>
__device__ __forceinline__ T irs_exec(const Gas<T>& G, T tol, int n_iter, T l_rho, T vl, T l_p, T l_cs,
                                      T& l_f, T r_rho, T vr, T r_p, T r_cs, T& r_f) {
  T p_star = T(0), p_prev, l_fp, r_fp;
  WaveSide<T> WL = wave_side<T, LAZY>(G, l_rho, l_p, l_cs);
  WaveSide<T> WR = wave_side<T, LAZY>(G, r_rho, r_p, r_cs);
  for (int gid = 0; gid < 6; ++gid) {
    p_star = guess_p_star(G, gid, l_rho, vl, l_p, l_cs, r_rho, vr, r_p, r_cs);
    p_prev = p_star;
    for (int i = 1; i <= n_iter; ++i) {
      nonlinear_wave<T, LAZY>(G, WL, p_star, l_f, l_fp);
      nonlinear_wave<T, LAZY>(G, WR, p_star, r_f, r_fp);
      p_star = p_prev - (l_f + r_f + (vr - vl)) / (l_fp + r_fp);
      if (p_star < T(0)) break;
      if (T(2) * m_abs(p_star - p_prev) / (p_star + p_prev) < tol) break;
      p_prev = p_star;
    }
    if (p_star > T(0)) break;
  }
  if (p_star < T(0)) p_star = T(0);
  return p_star;
}

// rp_side_t (rhyme_riemann_problem.f90:53-56)
template <int D, typename T>
struct Side {
  T rho, v[D], p, cs;
};

// Sampled star-region summary (rhyme_riemann_problem.f90:33-51).
template <typename T>
struct Star {
  T u, p;
  bool l_shock, r_shock;
  T l_rho, l_speed, l_cs, l_speedH, l_speedT;  // speed = shock speed
  T r_rho, r_speed, r_cs, r_speedH, r_speedT;
  T l_f, r_f;
};

// rhyme_riemann_problem_star.f90:12-65, split so that only the side the
// sampling reads is formed: p* and u* (:12-38), then the left (:40, 43-53)
// or the right (:41, 55-65) star state, each with the reference's
// operations.
template <int D, int AX, typename T, bool LAZY>
__device__ __forceinline__ void rp_star_pu(const Gas<T>& G, const Rp<T>& rp, const Side<D, T>& L,
                                           const Side<D, T>& R, Star<T>& s) {
  s.p = irs_exec<T, LAZY>(G, rp.tol, rp.n_iter, L.rho, L.v[AX], L.p, L.cs, s.l_f, R.rho, R.v[AX], R.p, R.cs,
                          s.r_f);
  if (s.p < rp.vac_p) s.p = rp.vac_p;
  s.u = T(0.5) * ((R.v[AX] + L.v[AX]) + (s.r_f - s.l_f));
}

template <int D, int AX, typename T>
__device__ __forceinline__ void rp_star_left(const Gas<T>& G, const Side<D, T>& L, Star<T>& s) {
  T ps_pl = s.p / L.p;
  if (s.p > L.p) {
    s.l_shock = true;
    s.l_rho = L.rho * (G.gm1_gp1 + ps_pl) / (G.gm1_gp1 * ps_pl + T(1));
    s.l_speed = L.v[AX] - L.cs * m_sqrt(G.gp1_2g * ps_pl + G.gm1_2g);
  } else {
    s.l_shock = false;
    T pg, pa;
    m_pow2(ps_pl, G.g_inv, G.gm1_2g, pg, pa);
    s.l_rho = L.rho * pg;
    s.l_cs = L.cs * pa;
    s.l_speedH = L.v[AX] - L.cs;
    s.l_speedT = s.u - s.l_cs;
  }
}

template <int D, int AX, typename T>
__device__ __forceinline__ void rp_star_right(const Gas<T>& G, const Side<D, T>& R, Star<T>& s) {
  T ps_pr = s.p / R.p;
  if (s.p > R.p) {
    s.r_shock = true;
    s.r_rho = R.rho * (G.gm1_gp1 + ps_pr) / (G.gm1_gp1 * ps_pr + T(1));
    s.r_speed = R.v[AX] + R.cs * m_sqrt(G.gp1_2g * ps_pr + G.gm1_2g);
  } else {
    s.r_shock = false;
    T pg, pa;
    m_pow2(ps_pr, G.g_inv, G.gm1_2g, pg, pa);
    s.r_rho = R.rho * pg;
    s.r_cs = R.cs * pa;
    s.r_speedH = R.v[AX] + R.cs;
    s.r_speedT = s.u + s.r_cs;
  }
}

// rhyme_riemann_problem_w_kfan.f90:14-31
template <int D, int AX, typename T>
__device__ __forceinline__ void w_kfan_body(const Gas<T>& G, const Side<D, T>& s, T dxdt, bool is_right, T* u) {
  T cs = is_right ? -s.cs : s.cs;
  const T base = G.two_gp1 + G.gm1_gp1 / cs * (s.v[AX] - dxdt);
  T prho, pp;
  m_pow2(base, G.two_gm1, G.inv_gm1_2g, prho, pp);
  T rho = s.rho * prho;
  T v[D];
#pragma unroll
  for (int a = 0; a < D; ++a) v[a] = s.v[a];
  v[AX] = G.two_gp1 * (cs + G.half_gm1 * s.v[AX] + dxdt);
  T p = s.p * pp;
  prim_vars_to_cons<D>(G, rho, v, p, u);
}

template <int D, int AX, typename T>
__device__ __noinline__ void w_kfan_call(const Gas<T>& G, const Side<D, T>& s, T dxdt, bool is_right, T* u) {
  w_kfan_body<D, AX>(G, s, dxdt, is_right, u);
}

// The double form is a call (its powers are long and rarely sampled); the
// float form is inlined: a call would keep the caller's state vector in
// local memory (its address escapes), a load and store per component on
// every interface of the FP32 sweeps.
template <int D, int AX, typename T>
__device__ __forceinline__ void w_kfan(const Gas<T>& G, const Side<D, T>& s, T dxdt, bool is_right, T* u) {
  if constexpr (sizeof(T) == sizeof(float)) w_kfan_body<D, AX>(G, s, dxdt, is_right, u);
  else w_kfan_call<D, AX>(G, s, dxdt, is_right, u);
}

// rhyme_riemann_problem_w_star{L,R}_{sho,fan}.f90:12-15
template <int D, int AX, typename T>
__device__ __forceinline__ void w_star(const Gas<T>& G, const Side<D, T>& side, const Star<T>& s, T rho,
                                       T* u) {
  T v[D];
#pragma unroll
  for (int a = 0; a < D; ++a) v[a] = side.v[a];
  v[AX] = s.u;
  prim_vars_to_cons<D>(G, rho, v, s.p, u);
}

// rhyme_riemann_problem_sampling.f90:13-47 at x/t = dxdt
// (the reference forms both sides' star states, and both sides' velocities
// across AX, first; only the side read here gets them, from its conserved
// state q, which leaves every value read unchanged)
template <int D, int AX, typename T>
__device__ __forceinline__ void side_transverse(Side<D, T>& S, const T* q) {
#pragma unroll
  for (int a = 0; a < D; ++a)
    if (a != AX) S.v[a] = q[1 + a] / q[0];
}

template <int D, int AX, typename T>
__device__ __forceinline__ void rp_sampling(const Gas<T>& G, Side<D, T>& L, Side<D, T>& R, const T* l,
                                            const T* r, Star<T>& s, T dxdt, T* u) {
  if (dxdt > s.u) {
    side_transverse<D, AX>(R, r);
    rp_star_right<D, AX>(G, R, s);
    if (s.r_shock) {
      if (dxdt < s.r_speed) w_star<D, AX>(G, R, s, s.r_rho, u);
      else prim_vars_to_cons<D>(G, R.rho, R.v, R.p, u);
    } else {
      if (dxdt < s.r_speedT) w_star<D, AX>(G, R, s, s.r_rho, u);
      else if (dxdt < s.r_speedH) w_kfan<D, AX>(G, R, dxdt, true, u);
      else prim_vars_to_cons<D>(G, R.rho, R.v, R.p, u);
    }
  } else {
    side_transverse<D, AX>(L, l);
    rp_star_left<D, AX>(G, L, s);
    if (s.l_shock) {
      if (dxdt > s.l_speed) w_star<D, AX>(G, L, s, s.l_rho, u);
      else prim_vars_to_cons<D>(G, L.rho, L.v, L.p, u);
    } else {
      if (dxdt > s.l_speedT) w_star<D, AX>(G, L, s, s.l_rho, u);
      else if (dxdt > s.l_speedH) w_kfan<D, AX>(G, L, dxdt, false, u);
      else prim_vars_to_cons<D>(G, L.rho, L.v, L.p, u);
    }
  }
}

// Vacuum state W_0: prim_to_cons of w_vacuum (rho, 0.., p).
template <int D, typename T>
__device__ __forceinline__ void vacuum_state(const Gas<T>& G, const Rp<T>& rp, T* u) {
  T v[D];
#pragma unroll
  for (int a = 0; a < D; ++a) v[a] = T(0);
  prim_vars_to_cons<D>(G, rp.vac_rho, v, rp.vac_p, u);
}

// rhyme_riemann_problem_solve.f90:17-103 sampled at x/t = dxdt. (The mixed
// sweeps' FP32 interfaces go through rp_flux_f32 instead, which sends the
// interfaces this solver handles in its vacuum branches to the FP64 one.)
template <int D, int AX, typename T, bool LAZY = false>
__device__ __forceinline__ void rp_solve(const Gas<T>& G, const Rp<T>& rp, const T* l, const T* r,
                                         T dxdt, T* u) {
  Side<D, T> L, R;
  L.rho = fmax_ref(l[0], rp.vac_rho);
  R.rho = fmax_ref(r[0], rp.vac_rho);
  const T e_rho = rp.vac_rho_next;
  const bool vacuum_right = R.rho < e_rho && L.rho > e_rho;
  const bool vacuum_left = L.rho < e_rho && R.rho > e_rho;
  const bool vacuum_both = L.rho < e_rho && R.rho < e_rho;
  const T tiny = Limits<T>::tiny();

  if (vacuum_right) {
#pragma unroll
    for (int a = 0; a < D; ++a) L.v[a] = l[1 + a] / l[0];
    L.p = fmax_ref(pressure<D>(G, l), rp.vac_p);
    L.cs = fmax_ref(sound_speed<D>(G, l), tiny);
#pragma unroll
    for (int a = 0; a < D; ++a) R.v[a] = T(0);
    R.p = rp.vac_p;
    R.cs = T(0);
    T s_starl = L.v[AX] - T(2) * L.cs / G.gm1;
    if (dxdt > s_starl) vacuum_state<D>(G, rp, u);
    else if (dxdt > L.v[AX] - L.cs) w_kfan<D, AX>(G, L, dxdt, false, u);
    else prim_vars_to_cons<D>(G, L.rho, L.v, L.p, u);
  } else if (vacuum_left) {
#pragma unroll
    for (int a = 0; a < D; ++a) L.v[a] = T(0);
    L.p = rp.vac_p;
    L.cs = T(0);
#pragma unroll
    for (int a = 0; a < D; ++a) R.v[a] = r[1 + a] / r[0];
    R.p = fmax_ref(pressure<D>(G, r), rp.vac_p);
    R.cs = fmax_ref(sound_speed<D>(G, r), tiny);
    T s_starr = R.v[AX] + T(2) * R.cs / G.gm1;
    if (dxdt > R.v[AX] + R.cs) prim_vars_to_cons<D>(G, R.rho, R.v, R.p, u);
    else if (dxdt > s_starr) w_kfan<D, AX>(G, R, dxdt, true, u);
    else vacuum_state<D>(G, rp, u);
  } else if (vacuum_both) {
    vacuum_state<D>(G, rp, u);
  } else {
    // velocities across AX: only for the side sampled (side_transverse)
    L.v[AX] = l[1 + AX] / l[0];
    L.p = fmax_ref(pressure<D>(G, l), rp.vac_p);
    L.cs = fmax_ref(sound_speed<D>(G, l), tiny);
    R.v[AX] = r[1 + AX] / r[0];
    R.p = fmax_ref(pressure<D>(G, r), rp.vac_p);
    R.cs = fmax_ref(sound_speed<D>(G, r), tiny);
    T du = R.v[AX] - L.v[AX];
    T du_crit = T(2) * (L.cs + R.cs) / G.gm1;
    if (du_crit < du) {  // vacuum generation
      const T s_starl = L.v[AX] - T(2) * L.cs / G.gm1;
      const T s_starr = R.v[AX] + T(2) * R.cs / G.gm1;
      if (dxdt > s_starr) {
        side_transverse<D, AX>(R, r);
        if (dxdt > R.v[AX] + R.cs) prim_vars_to_cons<D>(G, R.rho, R.v, R.p, u);
        else w_kfan<D, AX>(G, R, dxdt, true, u);
      } else if (dxdt > s_starl) {
        vacuum_state<D>(G, rp, u);
      } else {
        side_transverse<D, AX>(L, l);
        if (dxdt > L.v[AX] - L.cs) w_kfan<D, AX>(G, L, dxdt, false, u);
        else prim_vars_to_cons<D>(G, L.rho, L.v, L.p, u);
      }
    } else {
      Star<T> s;
      rp_star_pu<D, AX, T, LAZY>(G, rp, L, R, s);
      rp_sampling<D, AX>(G, L, R, l, r, s, dxdt, u);
    }
  }
}

// ---- the mixed form's FP32 interface flux ----------------------------------
// rhyme_riemann_problem_solve.f90:17-103 sampled at x/t = 0 (every interface
// of the sweeps) followed by rhyme_ideal_gas_flux.f90, in FP32, for the
// interfaces the FP64 solver need not redo: a density at or below the
// vacuum density on either side (every vacuum branch), vacuum generation or
// an interface within 10 % of it, a density or pressure ratio beyond 1e6,
// and a first guess whose Newton iteration misses the tolerance set *need64
// instead, and the caller queues the interface for rp_solve<double>. The
// algorithm is the FP64 one's: the adaptive first guess of
// rhyme_irs_guess_p_star.f90:14-38, the Newton iteration of
// rhyme_irs_exec.f90:28-39 on the wave functions of
// rhyme_irs_nonlinear_wave_function.f90, the sampled side's star state
// (rhyme_riemann_problem_star.f90:40-65) and the tests of
// rhyme_riemann_problem_sampling.f90:13-47 at x/t = 0, including the fan of
// rhyme_riemann_problem_w_kfan.f90. The FP32 arithmetic is arranged for
// fewer divisions (one reciprocal per side of rho, p and rho cs; the
// quotients of gamma from Gas; the convergence test multiplied out; the flux
// formed from the sampled primitive state instead of from its conserved
// form), which also skips the cancellation of E - |m|^2/(2 rho).
__device__ __forceinline__ void wave_f32(const Gas<float>& G, float Ak, float Bk, float c2g, float irc, float pk,
                                         float ipk, float p, float& f, float& fprime) {
  if (p > pk) {
    const float rb = 1.f / (Bk + p);
    const float factor = sqrtf(Ak * rb);
    f = (p - pk) * factor;
    fprime = factor * (1.f - 0.5f * (p - pk) * rb);
  } else {
    // (p/p_k)^e - 1 as expm1(e log1p((p - p_k)/p_k)) (see nonlinear_wave)
    const float t = log1pf((p - pk) * ipk);
    f = c2g * expm1f(G.gm1_2g * t);
    fprime = irc * expf(-G.gp1_2g * t);
  }
}

template <int D, int AX>
__device__ __forceinline__ void rp_flux_f32(const Gas<float>& G, const Rp<float>& rp, const float* l,
                                            const float* r, float* f, bool* need64) {
  const float e_rho = rp.vac_rho_next;
  if (!(fmax_ref(l[0], rp.vac_rho) >= e_rho) || !(fmax_ref(r[0], rp.vac_rho) >= e_rho)) {
    *need64 = true;
    return;
  }
  // both densities above the vacuum density: the clamp of rho is inactive
  const float rl = l[0], rr = r[0];
  const float il = 1.f / rl, ir = 1.f / rr;
  float sl = 0.f, sr = 0.f;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    sl = sl + l[1 + a] * l[1 + a];
    sr = sr + r[1 + a] * r[1 + a];
  }
  const float pl_raw = (l[D + 1] - 0.5f * sl * il) * G.gm1;
  const float pr_raw = (r[D + 1] - 0.5f * sr * ir) * G.gm1;
  const float pl = fmax_ref(pl_raw, rp.vac_p), pr = fmax_ref(pr_raw, rp.vac_p);
  const float cl = fmax_ref(sqrtf(G.g * pl_raw * il), FLT_MIN);
  const float cr = fmax_ref(sqrtf(G.g * pr_raw * ir), FLT_MIN);
  const float vl = l[1 + AX] * il, vr = r[1 + AX] * ir;
  const float du = vr - vl;
  const float du_crit = G.two_gm1 * (cl + cr);
  const float rmin = fmin_ref(rl, rr), rmax = fmax_ref(rl, rr);
  const float pmin = fmin_ref(pl, pr), pmax = fmax_ref(pl, pr);
  if (!(du_crit - du > 0.1f * du_crit) || !(rmin * 1e6f > rmax) || !(pmin * 1e6f > pmax)) {
    *need64 = true;
    return;
  }
  const float ipl = 1.f / pl, ipr = 1.f / pr;
  const float ircl = il / cl, ircr = ir / cr;  // 1/(rho cs)
  // the adaptive first guess
  float p;
  {
    const float cup = 0.25f * (rl + rr) * (cl + cr);
    const float ppv = fmax_ref(0.5f * (pl + pr) + 0.5f * (vl - vr) * cup, 0.f);
    if (pmax <= 2.f * pmin && (pmin < ppv && ppv < pmax)) {
      p = ppv;  // PVRS
    } else if (ppv < pmin) {  // two-rarefaction
      const float icl = ircl * rl, icr = ircr * rr;  // 1/cs
      const float pq = m_pow(pl * ipr, G.gm1_2g);
      const float um = (pq * vl * icl + vr * icr + G.two_gm1 * (pq - 1.f)) / (pq * icl + icr);
      const float ptl = 1.f + G.half_gm1 * (vl - um) * icl;
      const float ptr = 1.f + G.half_gm1 * (um - vr) * icr;
      p = 0.5f * (pl * m_pow(ptl, G.inv_gm1_2g) + pr * m_pow(ptr, G.inv_gm1_2g));
    } else {  // two-shock
      const float gel = sqrtf(G.two_gp1 * il / (G.gm1_gp1 * pl + ppv));
      const float ger = sqrtf(G.two_gp1 * ir / (G.gm1_gp1 * pr + ppv));
      p = (gel * pl + ger * pr - du) / (gel + ger);
    }
    p = fmax_ref(p, FLT_MIN);
  }
  // Newton iteration from it
  const float Akl = G.two_gp1 * il, Bkl = G.gm1_gp1 * pl, c2gl = G.two_gm1 * cl;
  const float Akr = G.two_gp1 * ir, Bkr = G.gm1_gp1 * pr, c2gr = G.two_gm1 * cr;
  float p_prev = p, fl = 0.f, fr = 0.f, fpl, fpr;
  bool conv = false;
  for (int i = 1; i <= rp.n_iter; ++i) {
    wave_f32(G, Akl, Bkl, c2gl, ircl, pl, ipl, p, fl, fpl);
    wave_f32(G, Akr, Bkr, c2gr, ircr, pr, ipr, p, fr, fpr);
    p = p_prev - (fl + fr + du) / (fpl + fpr);
    if (p < 0.f) break;
    if (2.f * fabsf(p - p_prev) < rp.tol * (p + p_prev)) {
      conv = true;
      break;
    }
    p_prev = p;
  }
  if (!conv) {
    *need64 = true;
    return;
  }
  const float ps = (p < rp.vac_p) ? rp.vac_p : p;
  const float us = 0.5f * ((vr + vl) + (fr - fl));
  // the sampled side at x/t = 0: its density, normal velocity and pressure
  float rho, vn, pp;
  const bool right = 0.f > us;
  bool fan = false;
  float fan_cs = 0.f, fan_ic = 0.f, fan_v = 0.f, fan_rho = 0.f, fan_p = 0.f;
  if (right) {  // right of the contact
    const float ps_pr = ps * ipr;
    if (ps > pr) {
      const float rs = rr * (G.gm1_gp1 + ps_pr) / (G.gm1_gp1 * ps_pr + 1.f);
      const float speed = vr + cr * sqrtf(G.gp1_2g * ps_pr + G.gm1_2g);
      if (0.f < speed) { rho = rs; vn = us; pp = ps; } else { rho = rr; vn = vr; pp = pr; }
    } else {
      float pg, pa;
      m_pow2(ps_pr, G.g_inv, G.gm1_2g, pg, pa);
      if (0.f < us + cr * pa) { rho = rr * pg; vn = us; pp = ps; }
      else if (0.f < vr + cr) { fan = true; fan_cs = -cr; fan_ic = -(ircr * rr); fan_v = vr; fan_rho = rr; fan_p = pr; }
      else { rho = rr; vn = vr; pp = pr; }
    }
  } else {  // left of the contact
    const float ps_pl = ps * ipl;
    if (ps > pl) {
      const float rs = rl * (G.gm1_gp1 + ps_pl) / (G.gm1_gp1 * ps_pl + 1.f);
      const float speed = vl - cl * sqrtf(G.gp1_2g * ps_pl + G.gm1_2g);
      if (0.f > speed) { rho = rs; vn = us; pp = ps; } else { rho = rl; vn = vl; pp = pl; }
    } else {
      float pg, pa;
      m_pow2(ps_pl, G.g_inv, G.gm1_2g, pg, pa);
      if (0.f > us - cl * pa) { rho = rl * pg; vn = us; pp = ps; }
      else if (0.f > vl - cl) { fan = true; fan_cs = cl; fan_ic = ircl * rl; fan_v = vl; fan_rho = rl; fan_p = pl; }
      else { rho = rl; vn = vl; pp = pl; }
    }
  }
  if (fan) {  // inside the rarefaction fan (w_kfan at x/t = 0)
    const float base = G.two_gp1 + G.gm1_gp1 * fan_ic * fan_v;
    float prho, ppw;
    m_pow2(base, G.two_gm1, G.inv_gm1_2g, prho, ppw);
    rho = fan_rho * prho;
    vn = G.two_gp1 * (fan_cs + G.half_gm1 * fan_v);
    pp = fan_p * ppw;
  }
  // the flux of the sampled primitive state
  float v[D];
  float s = 0.f;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    v[a] = (a == AX) ? vn : (right ? r[1 + a] * ir : l[1 + a] * il);
    s = s + v[a] * v[a];
  }
  const float mn = rho * vn;
  f[0] = mn;
#pragma unroll
  for (int a = 0; a < D; ++a) f[1 + a] = mn * v[a];
  f[1 + AX] = f[1 + AX] + pp;
  f[D + 1] = vn * (0.5f * rho * s + pp * (0.5f * G.two_gm1) + pp);
}

// Interface flux: Riemann state at x/t = 0 (dx = 0 in
// rhyme_muscl_hancock_solve_memory_intensive.f90:110-116), then calc_flux.
// LAZY: see WaveSide.
template <int D, int AX, typename T, bool LAZY = false>
__device__ __forceinline__ void interface_flux(const Gas<T>& G, const Rp<T>& rp, const T* l, const T* r,
                                               T* f) {
  T u[D + 2];
  rp_solve<D, AX, T, LAZY>(G, rp, l, r, T(0), u);
  flux<D, AX>(G, u, f);
}

}  // namespace rgpu
