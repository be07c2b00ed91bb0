// rhyme_oracle.hpp -- CPU restatement of Rhyme's MUSCL-Hancock hydro path.
//
// TEST INFRASTRUCTURE ONLY. This file is the parity checker for the CUDA
// library and the timed CPU baseline ("port"). Nothing in the shipped
// library includes, links or calls it; only tests/, __graft_entry__.smoke()
// and bench.py's CPU legs load it (through oracle_capi.cpp).
//
// Every function restates one reference Fortran routine and keeps its
// floating-point evaluation order literally (Fortran evaluates operators of
// equal precedence left to right; integer and default-real literals that
// appear in the reference are exact in double). Build with
// -O2 -ffp-contract=off so no multiply-add is contracted.
//
// Pinning: the pieces below are checked against every golden vector the
// reference's own tests hold for this path (p_stars.txt, the Sod t=0.2
// analytic profile, Toro's star states, the limiter / BC / CFL / flux /
// half-step known answers); see tests/test_oracle_*.py. The reference's
// whole-box solve tests carry no expectations, so whole-step results rest on
// this restatement (rhyme_muscl_hancock_solve_memory_intensive_test.f90:69-85
// has no `expect`).
//
// Reference file paths are relative to the Rhyme source tree (src/...).
#pragma once

#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../rhyme_gb300/csrc/libm_pow.h"

namespace rhyme_oracle {

// Power function used for every real `**` of the reference. Mode 0 is the C
// library's pow, as the compiled Fortran calls it: the reference arithmetic
// the GPU is checked against. Mode 1 is libm_pow::pow, the restatement of
// that function which the CUDA library runs; it lets the tests show, on the
// CPU, that the restatement returns the C library's bits.
inline int& pow_mode() {
  static int mode = 0;
  return mode;
}
inline double opow(double x, double y) {
  return pow_mode() == 1 ? libm_pow::pow(x, y) : std::pow(x, y);
}

// tiny(0d0) in Fortran is the smallest positive normal double.
constexpr double kTiny = DBL_MIN;

// Fortran MAX/MIN of two reals. Without NaNs every compiler agrees; with a
// NaN the reference is compiler-defined, and both the oracle and the CUDA
// kernels use this same ternary so they agree with each other.
inline double fmax_ref(double a, double b) { return (b > a) ? b : a; }
inline double fmin_ref(double a, double b) { return (b < a) ? b : a; }

// Ideal-gas constants. rhyme_riemann_problem_init.f90:20-27 and
// rhyme_irs_init.f90:21-27 derive the same six values from get_gamma().
struct Gas {
  double g, gm1, gp1, gm1_gp1, gm1_2g, gp1_2g, g_inv, kb_amu;
};

inline Gas make_gas(double g, double kb_amu) {
  Gas s;
  s.g = g;
  s.gm1 = g - 1.0;
  s.gp1 = g + 1.0;
  s.gm1_gp1 = s.gm1 / s.gp1;
  s.gm1_2g = s.gm1 / (2.0 * g);
  s.gp1_2g = s.gp1 / (2.0 * g);
  s.g_inv = 1.0 / g;
  s.kb_amu = kb_amu;
  return s;
}

// Slope limiter ids, rhyme_slope_limiter.f90:6-10 (slid).
enum { kVanLeer = 1, kMinmod = 2, kVanAlbada = 3, kSuperbee = 4 };
// Boundary ids, rhyme_samr_bc.f90:9-12 (bcid).
enum { kReflective = 1, kOutflow = 2, kPeriodic = 3, kInflow = 4 };
// Solver ids, rhyme_muscl_hancock.f90:10-15 (mhid via mhwsid).
enum { kCpuIntensive = 1, kMemoryIntensive = 2 };

struct Params {
  int ndim;
  double gamma, kb_amu, courant;
  int limiter;
  double omega;
  double vac_rho, vac_p, tol;
  int n_iter;
  int bc[6];
  int solver_type;
  double inflow[6][5];  // conserved inflow state per face (rho, m.., E)
};

// ---------------------------------------------------------------------------
// EOS: rhyme_hydro_base + rhyme_ideal_gas. u = (rho, m_1..m_D, E).
// ---------------------------------------------------------------------------

// rhyme_hydro_base_specific_kinetic_energy.f90:9
//   .5d0*sum(u(rho_u:..)**2)/u(rho)**2
template <int D>
inline double sp_kin_e(const double* u) {
  double s = 0.0;
  for (int a = 0; a < D; ++a) s = s + u[1 + a] * u[1 + a];
  return (0.5 * s) / (u[0] * u[0]);
}

// rhyme_hydro_base_specific_internal_energy.f90:9
template <int D>
inline double sp_int_e(const double* u) {
  return u[D + 1] / u[0] - sp_kin_e<D>(u);
}

// rhyme_ideal_gas_pressure.f90:9  p = u(rho)*e_int*(gamma - 1)
template <int D>
inline double pressure(const Gas& G, const double* u) {
  return u[0] * sp_int_e<D>(u) * (G.g - 1.0);
}

// rhyme_ideal_gas_temperature_per_mu.f90:9-10 and
// rhyme_ideal_gas_speed_of_sound.f90:9
template <int D>
inline double sound_speed(const Gas& G, const double* u) {
  double t_mu = sp_int_e<D>(u) * (G.g - 1.0) / G.kb_amu;
  return std::sqrt(G.g * G.kb_amu * t_mu);
}

// rhyme_ideal_gas_flux.f90:12-23
template <int D>
inline void flux(const Gas& G, const double* u, int axis, double* f) {
  if (std::fabs(u[0]) < kTiny) {
    for (int c = 0; c < D + 2; ++c) f[c] = 0.0;
    return;
  }
  double p = pressure<D>(G, u);
  f[0] = u[1 + axis];
  for (int a = 0; a < D; ++a) f[1 + a] = u[1 + a] * f[0] / u[0];
  f[1 + axis] = f[1 + axis] + p;
  f[D + 1] = f[0] / u[0] * (u[D + 1] + p);
}

// rhyme_ideal_gas_primitive_vars_to_conserved.f90:9-11
template <int D>
inline void prim_vars_to_cons(const Gas& G, double rho, const double* v,
                              double p, double* u) {
  u[0] = rho;
  double s = 0.0;
  for (int a = 0; a < D; ++a) {
    u[1 + a] = rho * v[a];
    s = s + v[a] * v[a];
  }
  u[D + 1] = 0.5 * rho * s + p / (G.g - 1.0);
}

// rhyme_ideal_gas_primitive_to_conserved.f90:9-12 applied to w_vacuum
// (rho, 0.., p): the vacuum state W_0 used by the Riemann solver.
template <int D>
inline void vacuum_to_cons(const Gas& G, double vac_rho, double vac_p,
                           double* u) {
  double v[3] = {0.0, 0.0, 0.0};
  prim_vars_to_cons<D>(G, vac_rho, v, vac_p, u);
}

// ---------------------------------------------------------------------------
// Slope limiter: rhyme_slope_limiter*.f90
// ---------------------------------------------------------------------------

// rhyme_slope_limiter_xi_r.f90:11
inline double xi_r(double w, double r) {
  return 2.0 / (1.0 - w + (1.0 + w) * r);
}

// Per-component limited slope; rhyme_slope_limiter.f90:62-82 gives r, the
// four limiter files give delta (van Leer :13-27, minmod :13-29,
// van Albada :13-27, superbee :13-31).
inline double limited_slope(int type, double w, double ul, double u,
                            double ur) {
  double d_L = u - ul;
  double d_R = ur - u;
  double d = 0.5 * (1.0 + w) * d_L + 0.5 * (1.0 + w) * d_R;
  double denom = ur - u;
  double r = (std::fabs(denom) < kTiny) ? 0.0 : (u - ul) / denom;
  switch (type) {
    case kVanLeer:
      if (r > 0.0) return fmin_ref(2.0 * r / (1.0 + r), xi_r(w, r)) * d;
      return 0.0;
    case kMinmod:
      if (r > 1.0) return fmin_ref(1.0, xi_r(w, r)) * d;
      if (r > 0.0) return r * d;
      return 0.0;
    case kVanAlbada:
      // r**2.d0 is folded to r*r by the Fortran compiler.
      if (r > 0.0)
        return fmin_ref(r * (1.0 + r) / (1.0 + r * r), xi_r(w, r)) * d;
      return 0.0;
    case kSuperbee:
      if (r > 1.0) return fmin_ref(fmin_ref(r, xi_r(w, r)), 2.0) * d;
      if (r > 0.5) return d;
      if (r > 0.0) return 2.0 * r * d;
      return 0.0;
    default:
      // rhyme_slope_limiter_run.f90:10-19 leaves delta unset; callers
      // validate the id before reaching here.
      return 0.0;
  }
}

// rhyme_slope_limiter_run.f90:10-19 for a (D+2)-vector.
template <int D>
inline void slope_limiter_run(int type, double w, const double* ul,
                              const double* u, const double* ur,
                              double* delta) {
  for (int c = 0; c < D + 2; ++c)
    delta[c] = limited_slope(type, w, ul[c], u[c], ur[c]);
}

// rhyme_muscl_hancock_half_step_extrapolation.f90:15-21
template <int D>
inline void half_step(const Gas& G, const double* u, const double* delta,
                      int axis, double dx, double dt, double* l, double* r) {
  double fl[D + 2], fr[D + 2];
  for (int c = 0; c < D + 2; ++c) {
    l[c] = u[c] - 0.5 * delta[c];
    r[c] = u[c] + 0.5 * delta[c];
  }
  flux<D>(G, l, axis, fl);
  flux<D>(G, r, axis, fr);
  for (int c = 0; c < D + 2; ++c) {
    double df = fl[c] - fr[c];
    l[c] = l[c] + 0.5 * dt / dx * df;
    r[c] = r[c] + 0.5 * dt / dx * df;
  }
}

// ---------------------------------------------------------------------------
// Exact Riemann solver: rhyme_irs_* and rhyme_riemann_problem_*
// ---------------------------------------------------------------------------

// rhyme_irs_nonlinear_wave_function.f90:13-24
inline void nonlinear_wave(const Gas& G, double s_rho, double s_p,
                           double s_cs, double p, double& f,
                           double& fprime) {
  if (p > s_p) {
    double Ak = 2.0 / (G.gp1 * s_rho);
    double Bk = G.gm1 * s_p / G.gp1;
    double factor = std::sqrt(Ak / (Bk + p));
    f = (p - s_p) * factor;
    fprime = factor * (1.0 - (p - s_p) / (2.0 * (Bk + p)));
  } else {
    f = 2.0 * s_cs / G.gm1 * (opow(p / s_p, G.gm1_2g) - 1.0);
    fprime = 1.0 / (s_rho * s_cs) * opow(p / s_p, -G.gp1_2g);
  }
}

// rhyme_irs_guess_p_star.f90:74-80
inline double guess_g_k(const Gas& G, double rho, double p) {
  return std::sqrt((2.0 / (G.gp1 * rho)) / (p + G.gm1_gp1 * p));
}

// rhyme_irs_guess_p_star.f90:14-71; all six guesses, evaluated eagerly as
// the reference does. vl/vr are the normal velocities.
inline void guess_p_star(const Gas& G, double l_rho, double vl, double l_p,
                         double l_cs, double r_rho, double vr, double r_p,
                         double r_cs, double ps[6]) {
  const double q_user = 2.0;
  double cup = 0.25 * (l_rho + r_rho) * (l_cs + r_cs);
  double ppv = fmax_ref(0.5 * (l_p + r_p) + 0.5 * (vl - vr) * cup, 0.0);
  double p_min = fmin_ref(l_p, r_p);
  double p_max = fmax_ref(l_p, r_p);
  double q_max = p_max / p_min;

  if (q_max <= q_user && (p_min < ppv && ppv < p_max)) {
    ps[0] = ppv;  // PVRS
  } else if (ppv < p_min) {
    // Two-rarefaction
    double pq = opow(l_p / r_p, G.gm1_2g);
    double um = (pq * vl / l_cs + vr / r_cs + 2.0 / G.gm1 * (pq - 1.0)) /
                (pq / l_cs + 1.0 / r_cs);
    double ptl = 1.0 + G.gm1 / 2.0 * (vl - um) / l_cs;
    double ptr = 1.0 + G.gm1 / 2.0 * (um - vr) / r_cs;
    ps[0] = 0.5 * (l_p * opow(ptl, 1.0 / G.gm1_2g) +
                   r_p * opow(ptr, 1.0 / G.gm1_2g));
  } else {
    // Two-shock
    double gel = std::sqrt(((2.0 / (G.gp1)) / l_rho) / (G.gm1_gp1 * l_p + ppv));
    double ger = std::sqrt(((2.0 / (G.gp1)) / r_rho) / (G.gm1_gp1 * r_p + ppv));
    ps[0] = (gel * l_p + ger * r_p - (vr - vl)) / (gel + ger);
  }

  // Ramses guess
  ps[1] = (r_rho * r_cs * l_p + l_rho * l_cs * r_p +
           r_cs * l_cs * (l_rho * vl - r_rho * vr)) /
          (r_rho * r_cs + l_rho * l_cs);

  // Two-rarefaction approximation
  ps[2] = opow((l_cs + r_cs - 0.5 * G.gm1 * (vr - vl)) /
                       (opow(l_cs / l_p, G.gm1_2g) +
                        opow(r_cs / r_p, G.gm1_2g)),
                   1.0 / G.gm1_2g);

  // Two-shock approximation
  double l_g = guess_g_k(G, l_rho, l_p);
  double r_g = guess_g_k(G, r_rho, r_p);
  ps[3] = (l_g * l_p + r_g * r_p - (vr - vl)) / (l_g + r_g);

  // p_PV
  ps[4] = 0.5 * (l_p + r_p) -
          0.125 * (vr - vl) * (l_rho + r_rho) * (l_cs + r_cs);

  // Arithmetic mean
  ps[5] = 0.5 * (l_p + r_p);

  for (int i = 0; i < 6; ++i) ps[i] = fmax_ref(ps[i], kTiny);
}

// Optional per-solve counters (Newton iterations, guesses used).
struct IrsStats {
  long long solves = 0, iterations = 0, extra_guesses = 0;
};

// rhyme_irs_exec.f90:19-44. l_f / r_f return the wave functions evaluated at
// the last iterate before the final Newton update.
inline double irs_exec(const Gas& G, double tol, int n_iter, double l_rho,
                       double vl, double l_p, double l_cs, double& l_f,
                       double r_rho, double vr, double r_p, double r_cs,
                       double& r_f, IrsStats* st = nullptr) {
  double guessed[6];
  guess_p_star(G, l_rho, vl, l_p, l_cs, r_rho, vr, r_p, r_cs, guessed);
  double p_star = 0.0, p_prev = 0.0, l_fp = 0.0, r_fp = 0.0;
  for (int gid = 0; gid < 6; ++gid) {
    p_star = guessed[gid];
    p_prev = p_star;
    if (st && gid > 0) st->extra_guesses++;
    for (int i = 1; i <= n_iter; ++i) {
      if (st) st->iterations++;
      nonlinear_wave(G, l_rho, l_p, l_cs, p_star, l_f, l_fp);
      nonlinear_wave(G, r_rho, r_p, r_cs, p_star, r_f, r_fp);
      p_star = p_prev - (l_f + r_f + (vr - vl)) / (l_fp + r_fp);
      if (p_star < 0.0) break;
      if (2.0 * std::fabs(p_star - p_prev) / (p_star + p_prev) < tol) break;
      p_prev = p_star;
    }
    if (p_star > 0.0) break;
  }
  if (st) st->solves++;
  if (p_star < 0.0) p_star = 0.0;
  return p_star;
}

// rhyme_riemann_problem.f90:33-61 (rp_side_t, rp_star_side_t, ...).
template <int D>
struct Side {
  double rho = 0.0, v[D] = {}, p = 0.0, cs = 0.0;
};
struct StarSide {
  bool is_shock = false;
  double shock_rho = 0.0, shock_speed = 0.0;
  double fan_rho = 0.0, fan_cs = 0.0, fan_speedH = 0.0, fan_speedT = 0.0;
  double f = 0.0, fprime = 0.0;
};
template <int D>
struct Solution {
  double star_u = 0.0, star_p = 0.0;
  StarSide sl, sr;
  Side<D> left, right;
};

// rhyme_riemann_problem_star.f90:12-65
template <int D>
inline void rp_star(const Gas& G, double vac_p, double tol, int n_iter,
                    Solution<D>& s, int axis, IrsStats* st = nullptr) {
  s.star_p = irs_exec(G, tol, n_iter, s.left.rho, s.left.v[axis], s.left.p,
                      s.left.cs, s.sl.f, s.right.rho, s.right.v[axis],
                      s.right.p, s.right.cs, s.sr.f, st);
  if (s.star_p < vac_p) s.star_p = vac_p;
  s.star_u = 0.5 * ((s.right.v[axis] + s.left.v[axis]) + (s.sr.f - s.sl.f));

  double ps_pl = s.star_p / s.left.p;
  double ps_pr = s.star_p / s.right.p;

  if (s.star_p > s.left.p) {
    s.sl.is_shock = true;
    s.sl.shock_rho =
        s.left.rho * (G.gm1_gp1 + ps_pl) / (G.gm1_gp1 * ps_pl + 1.0);
    s.sl.shock_speed =
        s.left.v[axis] - s.left.cs * std::sqrt(G.gp1_2g * ps_pl + G.gm1_2g);
  } else {
    s.sl.is_shock = false;
    s.sl.fan_rho = s.left.rho * opow(ps_pl, G.g_inv);
    s.sl.fan_cs = s.left.cs * opow(ps_pl, G.gm1_2g);
    s.sl.fan_speedH = s.left.v[axis] - s.left.cs;
    s.sl.fan_speedT = s.star_u - s.sl.fan_cs;
  }

  if (s.star_p > s.right.p) {
    s.sr.is_shock = true;
    s.sr.shock_rho =
        s.right.rho * (G.gm1_gp1 + ps_pr) / (G.gm1_gp1 * ps_pr + 1.0);
    s.sr.shock_speed =
        s.right.v[axis] + s.right.cs * std::sqrt(G.gp1_2g * ps_pr + G.gm1_2g);
  } else {
    s.sr.is_shock = false;
    s.sr.fan_rho = s.right.rho * opow(ps_pr, G.g_inv);
    s.sr.fan_cs = s.right.cs * opow(ps_pr, G.gm1_2g);
    s.sr.fan_speedH = s.right.v[axis] + s.right.cs;
    s.sr.fan_speedT = s.star_u + s.sr.fan_cs;
  }
}

// rhyme_riemann_problem_w_kfan.f90:14-31
template <int D>
inline void w_kfan(const Gas& G, const Side<D>& s, double dxdt, int axis,
                   bool is_right, double* u) {
  double cs = is_right ? -s.cs : s.cs;
  double rho = s.rho * opow(2.0 / G.gp1 + G.gm1_gp1 / cs * (s.v[axis] - dxdt),
                                2.0 / G.gm1);
  double v[D];
  for (int a = 0; a < D; ++a) v[a] = s.v[a];
  v[axis] = 2.0 / G.gp1 * (cs + G.gm1 / 2.0 * s.v[axis] + dxdt);
  double p = s.p * opow(2.0 / G.gp1 + G.gm1_gp1 / cs * (s.v[axis] - dxdt),
                            1.0 / G.gm1_2g);
  prim_vars_to_cons<D>(G, rho, v, p, u);
}

// rhyme_riemann_problem_w_k.f90:9 / rp_side_to_cons.f90:9
template <int D>
inline void side_to_cons(const Gas& G, const Side<D>& s, double* u) {
  prim_vars_to_cons<D>(G, s.rho, s.v, s.p, u);
}

// rhyme_riemann_problem_w_star{L,R}_{sho,fan}.f90:12-15
template <int D>
inline void w_star(const Gas& G, const Solution<D>& s, bool right, double rho,
                   int axis, double* u) {
  double v[D];
  for (int a = 0; a < D; ++a) v[a] = right ? s.right.v[a] : s.left.v[a];
  v[axis] = s.star_u;
  prim_vars_to_cons<D>(G, rho, v, s.star_p, u);
}

// rhyme_riemann_problem_sampling.f90:13-47
template <int D>
inline void rp_sampling(const Gas& G, const Solution<D>& s, int axis,
                        double dx, double dt, double* u) {
  double dxdt = dx / dt;
  if (dxdt > s.star_u) {
    if (s.sr.is_shock) {
      if (dxdt < s.sr.shock_speed)
        w_star<D>(G, s, true, s.sr.shock_rho, axis, u);
      else
        side_to_cons<D>(G, s.right, u);
    } else {
      if (dxdt < s.sr.fan_speedT)
        w_star<D>(G, s, true, s.sr.fan_rho, axis, u);
      else if (dxdt < s.sr.fan_speedH)
        w_kfan<D>(G, s.right, dxdt, axis, true, u);
      else
        side_to_cons<D>(G, s.right, u);
    }
  } else {
    if (s.sl.is_shock) {
      if (dxdt > s.sl.shock_speed)
        w_star<D>(G, s, false, s.sl.shock_rho, axis, u);
      else
        side_to_cons<D>(G, s.left, u);
    } else {
      if (dxdt > s.sl.fan_speedT)
        w_star<D>(G, s, false, s.sl.fan_rho, axis, u);
      else if (dxdt > s.sl.fan_speedH)
        w_kfan<D>(G, s.left, dxdt, axis, false, u);
      else
        side_to_cons<D>(G, s.left, u);
    }
  }
}

// rhyme_riemann_problem_solve.f90:17-103
template <int D>
inline void rp_solve(const Gas& G, double vac_rho, double vac_p, double tol,
                     int n_iter, const double* l, const double* r, double dx,
                     double dt, int axis, double* u,
                     IrsStats* st = nullptr) {
  Solution<D> sol;
  double dxdt = dx / dt;

  sol.left.rho = fmax_ref(l[0], vac_rho);
  sol.right.rho = fmax_ref(r[0], vac_rho);

  double e_rho = std::nextafter(vac_rho, 1.0);
  bool vacuum_right = sol.right.rho < e_rho && sol.left.rho > e_rho;
  bool vacuum_left = sol.left.rho < e_rho && sol.right.rho > e_rho;
  bool vacuum_both = sol.left.rho < e_rho && sol.right.rho < e_rho;

  if (vacuum_right) {
    for (int a = 0; a < D; ++a) sol.left.v[a] = l[1 + a] / l[0];
    sol.left.p = fmax_ref(pressure<D>(G, l), vac_p);
    sol.left.cs = fmax_ref(sound_speed<D>(G, l), kTiny);
    for (int a = 0; a < D; ++a) sol.right.v[a] = 0.0;
    sol.right.p = vac_p;
    sol.right.cs = 0.0;

    double s_starl = sol.left.v[axis] - 2.0 * sol.left.cs / G.gm1;
    if (dxdt > s_starl)
      vacuum_to_cons<D>(G, vac_rho, vac_p, u);
    else if (dxdt > sol.left.v[axis] - sol.left.cs)
      w_kfan<D>(G, sol.left, dxdt, axis, false, u);
    else
      side_to_cons<D>(G, sol.left, u);
  } else if (vacuum_left) {
    for (int a = 0; a < D; ++a) sol.left.v[a] = 0.0;
    sol.left.p = vac_p;
    sol.left.cs = 0.0;
    for (int a = 0; a < D; ++a) sol.right.v[a] = r[1 + a] / r[0];
    sol.right.p = fmax_ref(pressure<D>(G, r), vac_p);
    sol.right.cs = fmax_ref(sound_speed<D>(G, r), kTiny);

    double s_starr = sol.right.v[axis] + 2.0 * sol.right.cs / G.gm1;
    if (dxdt > sol.right.v[axis] + sol.right.cs)
      side_to_cons<D>(G, sol.right, u);
    else if (dxdt > s_starr)
      w_kfan<D>(G, sol.right, dxdt, axis, true, u);
    else
      vacuum_to_cons<D>(G, vac_rho, vac_p, u);
  } else if (vacuum_both) {
    vacuum_to_cons<D>(G, vac_rho, vac_p, u);
  } else {
    for (int a = 0; a < D; ++a) sol.left.v[a] = l[1 + a] / l[0];
    sol.left.p = fmax_ref(pressure<D>(G, l), vac_p);
    sol.left.cs = fmax_ref(sound_speed<D>(G, l), kTiny);
    for (int a = 0; a < D; ++a) sol.right.v[a] = r[1 + a] / r[0];
    sol.right.p = fmax_ref(pressure<D>(G, r), vac_p);
    sol.right.cs = fmax_ref(sound_speed<D>(G, r), kTiny);

    double s_starl = sol.left.v[axis] - 2.0 * sol.left.cs / G.gm1;
    double s_starr = sol.right.v[axis] + 2.0 * sol.right.cs / G.gm1;

    double du = sol.right.v[axis] - sol.left.v[axis];
    double du_crit = 2.0 * (sol.left.cs + sol.right.cs) / G.gm1;

    if (du_crit < du) {  // vacuum generation
      if (dxdt > s_starr) {
        if (dxdt > sol.right.v[axis] + sol.right.cs)
          side_to_cons<D>(G, sol.right, u);
        else
          w_kfan<D>(G, sol.right, dxdt, axis, true, u);
      } else if (dxdt > s_starl) {
        vacuum_to_cons<D>(G, vac_rho, vac_p, u);
      } else {
        if (dxdt > sol.left.v[axis] - sol.left.cs)
          w_kfan<D>(G, sol.left, dxdt, axis, false, u);
        else
          side_to_cons<D>(G, sol.left, u);
      }
    } else {
      rp_star<D>(G, vac_p, tol, n_iter, sol, axis, st);
      rp_sampling<D>(G, sol, axis, dx, dt, u);
    }
  }
}

// ---------------------------------------------------------------------------
// Box layout. cells(-1:N1+2, -1:N2+2, -1:N3+2, 1:NCMP) in Fortran order; the
// hydro fields are the first D+2 component blocks. Axes beyond D have extent
// 1 and no ghosts. `field` is the number of doubles in one component block.
// ---------------------------------------------------------------------------
struct BoxGeom {
  int D;
  int n[3];        // interior cells per axis (1 for inactive axes)
  int ext[3];      // allocated extent per axis (n+4 active, 1 inactive)
  long long s[3];  // element stride per axis
  long long field; // elements per component block
  // linear index of cell (i,j,k), 1-based interior coordinates
  long long at(int i, int j, int k) const {
    long long o = (long long)(i + 1) * s[0];
    if (D > 1) o += (long long)(j + 1) * s[1];
    if (D > 2) o += (long long)(k + 1) * s[2];
    return o;
  }
};

inline BoxGeom make_geom(int D, const int* dims) {
  BoxGeom g;
  g.D = D;
  for (int a = 0; a < 3; ++a) {
    g.n[a] = (a < D) ? dims[a] : 1;
    g.ext[a] = (a < D) ? dims[a] + 4 : 1;
  }
  g.s[0] = 1;
  g.s[1] = g.ext[0];
  g.s[2] = (long long)g.ext[0] * g.ext[1];
  g.field = g.s[2] * g.ext[2];
  return g;
}

// rhyme_cfl_time_step.f90:63-84
template <int D>
inline double cfl_time_step(const Gas& G, double courant, const double* cells,
                            const BoxGeom& g, const double* dx) {
  double max_u = 0.0;
  const int nk = (D > 2) ? g.n[2] : 1, nj = (D > 1) ? g.n[1] : 1;
  for (int k = 1; k <= nk; ++k)
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= g.n[0]; ++i) {
        long long o = g.at(i, j, k);
        double u[D + 2];
        for (int c = 0; c < D + 2; ++c) u[c] = cells[c * g.field + o];
        double s = 0.0;
        for (int a = 0; a < D; ++a) s = s + u[1 + a] * u[1 + a];
        double v = std::sqrt(s) / u[0] + sound_speed<D>(G, u);
        if (v > max_u) max_u = v;
      }
  double mdx = dx[0];
  for (int a = 1; a < D; ++a) mdx = fmin_ref(mdx, dx[a]);
  return courant * mdx / max_u;
}

// rhyme_samr_bc_set_{left,right,bottom,top,back,front}_boundary.f90 for the
// hydro fields (inflow also writes the extra components in the reference;
// those are outside the hydro state mirrored here). Faces only, no corners.
template <int D>
inline void set_boundaries(const Params& P, double* cells, const BoxGeom& g) {
  const long long F = g.field;
  for (int axis = 0; axis < D; ++axis) {
    const int N = g.n[axis];
    const long long sa = g.s[axis];
    // transverse ranges: interior 1..n for the other active axes
    int t1 = (axis == 0) ? 1 : 0, t2 = (axis == 2) ? 1 : 2;
    int n1 = (t1 < D) ? g.n[t1] : 1, n2 = (t2 < D) ? g.n[t2] : 1;
    for (int side = 0; side < 2; ++side) {
      int type = P.bc[2 * axis + side];
      for (int c = 0; c < D + 2; ++c) {
        for (int b = 1; b <= n2; ++b)
          for (int a = 1; a <= n1; ++a) {
            int idx[3] = {1, 1, 1};
            idx[t1] = a;
            if (t2 < 3) idx[t2] = b;
            idx[axis] = 0;
            const long long base = g.at(idx[0], idx[1], idx[2]);  // cell 0
            double* f = cells + c * F;
            long long g0, g1, s0, s1;  // ghost targets and sources
            if (side == 0) {
              g0 = base;            // cell 0
              g1 = base - sa;       // cell -1
              if (type == kPeriodic) {
                s0 = base + (long long)N * sa;        // cell N
                s1 = base + (long long)(N - 1) * sa;  // cell N-1
              } else {
                s0 = base + sa;        // cell 1
                s1 = base + 2 * sa;    // cell 2
              }
            } else {
              g0 = base + (long long)(N + 1) * sa;  // cell N+1
              g1 = base + (long long)(N + 2) * sa;  // cell N+2
              if (type == kPeriodic) {
                s0 = base + sa;      // cell 1
                s1 = base + 2 * sa;  // cell 2
              } else {
                s0 = base + (long long)N * sa;        // cell N
                s1 = base + (long long)(N - 1) * sa;  // cell N-1
              }
            }
            if (type == kInflow) {
              f[g0] = P.inflow[2 * axis + side][c];
              f[g1] = P.inflow[2 * axis + side][c];
            } else if (type == kOutflow || type == kPeriodic ||
                       type == kReflective) {
              f[g0] = f[s0];
              f[g1] = f[s1];
              if (type == kReflective && c == 1 + axis) {
                f[g0] = -f[s0];
                f[g1] = -f[s1];
              }
            }
          }
      }
    }
  }
}

// Workspace of the memory-intensive solver (rhyme_mh_workspace_check.f90:
// 36-77): ul, ur, fr(-1:N+2,..., rho:e_tot, NDIM).
struct Workspace {
  std::vector<double> ul, ur, fr;
  void ensure(const BoxGeom& g) {
    size_t n = (size_t)g.D * (g.D + 2) * g.field;
    if (ul.size() != n) {
      ul.assign(n, 0.0);
      ur.assign(n, 0.0);
      fr.assign(n, 0.0);
    }
  }
};

// rhyme_muscl_hancock_solve_memory_intensive.f90:47-180. The outermost loop
// is shared among OpenMP threads as in the reference.
template <int D>
inline void mh_solve_memory_intensive(const Params& P, const Gas& G,
                                      double* cells, const BoxGeom& g,
                                      const double* dx, double dt,
                                      Workspace& ws, IrsStats* st = nullptr) {
  ws.ensure(g);
  const long long F = g.field;
  const long long W = (long long)(D + 2) * F;  // per-axis workspace block
  double* ul = ws.ul.data();
  double* ur = ws.ur.data();
  double* fr = ws.fr.data();
  const int n0 = g.n[0], n1 = (D > 1) ? g.n[1] : 1, n2 = (D > 2) ? g.n[2] : 1;
  const int lo1 = (D > 1) ? 0 : 1, lo2 = (D > 2) ? 0 : 1;

  // LOOP 1: i,j,k in [0, N+1]
  {
    const int hi0 = n0 + 1, hi1 = (D > 1) ? n1 + 1 : 1, hi2 = (D > 2) ? n2 + 1 : 1;
    const int outer_lo = (D == 1) ? 0 : ((D == 2) ? lo1 : lo2);
    const int outer_hi = (D == 1) ? hi0 : ((D == 2) ? hi1 : hi2);
#pragma omp parallel for schedule(static)
    for (int o = outer_lo; o <= outer_hi; ++o) {
      int klo = (D == 3) ? o : 1, khi = (D == 3) ? o : 1;
      int jlo = (D == 2) ? o : ((D == 3) ? lo1 : 1);
      int jhi = (D == 2) ? o : ((D == 3) ? hi1 : 1);
      int ilo = (D == 1) ? o : 0, ihi = (D == 1) ? o : hi0;
      for (int k = klo; k <= khi; ++k)
        for (int j = jlo; j <= jhi; ++j)
          for (int i = ilo; i <= ihi; ++i) {
            long long c0 = g.at(i, j, k);
            for (int axis = 0; axis < D; ++axis) {
              long long sa = g.s[axis];
              double um[D + 2], u0[D + 2], up[D + 2], delta[D + 2];
              double l[D + 2], r[D + 2];
              for (int c = 0; c < D + 2; ++c) {
                um[c] = cells[c * F + c0 - sa];
                u0[c] = cells[c * F + c0];
                up[c] = cells[c * F + c0 + sa];
              }
              slope_limiter_run<D>(P.limiter, P.omega, um, u0, up, delta);
              half_step<D>(G, u0, delta, axis, dx[axis], dt, l, r);
              for (int c = 0; c < D + 2; ++c) {
                ul[axis * W + c * F + c0] = l[c];
                ur[axis * W + c * F + c0] = r[c];
              }
            }
          }
    }
  }

  // LOOP 2: i,j,k in [0, N]
  {
    const int outer_lo = (D == 1) ? 0 : ((D == 2) ? lo1 : lo2);
    const int outer_hi = (D == 1) ? n0 : ((D == 2) ? n1 : n2);
    IrsStats local_total;
#pragma omp parallel
    {
      IrsStats local;
#pragma omp for schedule(static)
      for (int o = outer_lo; o <= outer_hi; ++o) {
        int klo = (D == 3) ? o : 1, khi = (D == 3) ? o : 1;
        int jlo = (D == 2) ? o : ((D == 3) ? lo1 : 1);
        int jhi = (D == 2) ? o : ((D == 3) ? n1 : 1);
        int ilo = (D == 1) ? o : 0, ihi = (D == 1) ? o : n0;
        for (int k = klo; k <= khi; ++k)
          for (int j = jlo; j <= jhi; ++j)
            for (int i = ilo; i <= ihi; ++i) {
              long long c0 = g.at(i, j, k);
              for (int axis = 0; axis < D; ++axis) {
                long long sa = g.s[axis];
                double l[D + 2], r[D + 2], u[D + 2], f[D + 2];
                for (int c = 0; c < D + 2; ++c) {
                  l[c] = ur[axis * W + c * F + c0];
                  r[c] = ul[axis * W + c * F + c0 + sa];
                }
                rp_solve<D>(G, P.vac_rho, P.vac_p, P.tol, P.n_iter, l, r, 0.0,
                            dt, axis, u, st ? &local : nullptr);
                flux<D>(G, u, axis, f);
                for (int c = 0; c < D + 2; ++c) fr[axis * W + c * F + c0] = f[c];
              }
            }
      }
      if (st) {
#pragma omp critical
        {
          local_total.solves += local.solves;
          local_total.iterations += local.iterations;
          local_total.extra_guesses += local.extra_guesses;
        }
      }
    }
    if (st) {
      st->solves += local_total.solves;
      st->iterations += local_total.iterations;
      st->extra_guesses += local_total.extra_guesses;
    }
  }

  // LOOP 3: i,j,k in [1, N]
  {
    const int outer_hi = (D == 1) ? n0 : ((D == 2) ? n1 : n2);
#pragma omp parallel for schedule(static)
    for (int o = 1; o <= outer_hi; ++o) {
      int klo = (D == 3) ? o : 1, khi = (D == 3) ? o : 1;
      int jlo = (D == 2) ? o : 1, jhi = (D == 2) ? o : ((D == 3) ? n1 : 1);
      int ilo = (D == 1) ? o : 1, ihi = (D == 1) ? o : n0;
      for (int k = klo; k <= khi; ++k)
        for (int j = jlo; j <= jhi; ++j)
          for (int i = ilo; i <= ihi; ++i) {
            long long c0 = g.at(i, j, k);
            for (int c = 0; c < D + 2; ++c) {
              double acc = dt / dx[0] *
                           (fr[0 * W + c * F + c0 - g.s[0]] - fr[0 * W + c * F + c0]);
              if (D > 1)
                acc = acc + dt / dx[1] *
                                (fr[1 * W + c * F + c0 - g.s[1]] - fr[1 * W + c * F + c0]);
              if (D > 2)
                acc = acc + dt / dx[2] *
                                (fr[2 * W + c * F + c0 - g.s[2]] - fr[2 * W + c * F + c0]);
              cells[c * F + c0] = cells[c * F + c0] + acc;
            }
          }
    }
  }
}

// rhyme_muscl_hancock_solve_cpu_intensive.f90:55-150: the same face states
// and interface states, with the per-axis update u = u + dt/dx*df applied in
// sequence (a different rounding order from the memory-intensive solver).
template <int D>
inline void mh_solve_cpu_intensive(const Params& P, const Gas& G,
                                   double* cells, const BoxGeom& g,
                                   const double* dx, double dt) {
  const long long F = g.field;
  const int n0 = g.n[0], n1 = (D > 1) ? g.n[1] : 1, n2 = (D > 2) ? g.n[2] : 1;
  std::vector<double> unew((size_t)(D + 2) * n0 * n1 * n2);
  const int outer_hi = (D == 1) ? n0 : ((D == 2) ? n1 : n2);
#pragma omp parallel for schedule(static)
  for (int o = 1; o <= outer_hi; ++o) {
    int klo = (D == 3) ? o : 1, khi = (D == 3) ? o : 1;
    int jlo = (D == 2) ? o : 1, jhi = (D == 2) ? o : ((D == 3) ? n1 : 1);
    int ilo = (D == 1) ? o : 1, ihi = (D == 1) ? o : n0;
    for (int k = klo; k <= khi; ++k)
      for (int j = jlo; j <= jhi; ++j)
        for (int i = ilo; i <= ihi; ++i) {
          long long c0 = g.at(i, j, k);
          double u[D + 2];
          for (int c = 0; c < D + 2; ++c) u[c] = cells[c * F + c0];
          for (int axis = 0; axis < D; ++axis) {
            long long sa = g.s[axis];
            double hl[3][D + 2], hr[3][D + 2];
            for (int idx = -1; idx <= 1; ++idx) {
              double um[D + 2], u0[D + 2], up[D + 2], delta[D + 2];
              long long cc = c0 + idx * sa;
              for (int c = 0; c < D + 2; ++c) {
                um[c] = cells[c * F + cc - sa];
                u0[c] = cells[c * F + cc];
                up[c] = cells[c * F + cc + sa];
              }
              slope_limiter_run<D>(P.limiter, P.omega, um, u0, up, delta);
              half_step<D>(G, u0, delta, axis, dx[axis], dt, hl[idx + 1], hr[idx + 1]);
            }
            double fl[2][D + 2];
            for (int idx = -1; idx <= 0; ++idx) {
              double es[D + 2];
              rp_solve<D>(G, P.vac_rho, P.vac_p, P.tol, P.n_iter, hr[idx + 1],
                          hl[idx + 2], 0.0, dt, axis, es);
              flux<D>(G, es, axis, fl[idx + 1]);
            }
            for (int c = 0; c < D + 2; ++c) {
              double df = fl[0][c] - fl[1][c];
              u[c] = u[c] + dt / dx[axis] * df;
            }
          }
          long long lin = (long long)(i - 1) + (long long)n0 * ((j - 1) + (long long)n1 * (k - 1));
          for (int c = 0; c < D + 2; ++c)
            unew[(size_t)c * n0 * n1 * n2 + lin] = u[c];
        }
  }
  for (int k = 1; k <= n2; ++k)
    for (int j = 1; j <= n1; ++j)
      for (int i = 1; i <= n0; ++i) {
        long long lin = (long long)(i - 1) + (long long)n0 * ((j - 1) + (long long)n1 * (k - 1));
        for (int c = 0; c < D + 2; ++c)
          cells[c * F + g.at(i, j, k)] = unew[(size_t)c * n0 * n1 * n2 + lin];
      }
}

// One driver iteration in the order of src/main.f90:109-136:
// dt from the state before the ghost fill, then the ghost fill, then the
// solve. Returns dt.
template <int D>
inline double step(const Params& P, const Gas& G, double* cells,
                   const BoxGeom& g, const double* dx, Workspace& ws,
                   IrsStats* st = nullptr) {
  double dt = cfl_time_step<D>(G, P.courant, cells, g, dx);
  set_boundaries<D>(P, cells, g);
  if (P.solver_type == kCpuIntensive)
    mh_solve_cpu_intensive<D>(P, G, cells, g, dx, dt);
  else
    mh_solve_memory_intensive<D>(P, G, cells, g, dx, dt, ws, st);
  return dt;
}

}  // namespace rhyme_oracle
