// oracle_capi.cpp -- extern "C" entry points over rhyme_oracle.hpp.
//
// TEST INFRASTRUCTURE ONLY: loaded through ctypes by tests/, by
// __graft_entry__.smoke() as the checker, and by bench.py's CPU baseline
// legs. The CUDA library never links or calls this file.
//
// Arrays of states are row-major [n][D+2] (rho, m_1..m_D, E). Box arrays are
// the Fortran cells(-1:N1+2, -1:N2+2, -1:N3+2, 1:D+2) hydro blocks.
#include <omp.h>

#include <cstring>

#include "rhyme_oracle.hpp"

using namespace rhyme_oracle;

extern "C" {

// Flat parameter block (mirrors the values the reference's modules hold).
struct oracle_params {
  int ndim, limiter, n_iter, solver_type;
  int bc[6];
  double gamma, kb_amu, courant, omega, vac_rho, vac_p, tol;
  double inflow[6][5];
};

static Params to_params(const oracle_params* p) {
  Params P;
  P.ndim = p->ndim;
  P.gamma = p->gamma;
  P.kb_amu = p->kb_amu;
  P.courant = p->courant;
  P.limiter = p->limiter;
  P.omega = p->omega;
  P.vac_rho = p->vac_rho;
  P.vac_p = p->vac_p;
  P.tol = p->tol;
  P.n_iter = p->n_iter;
  P.solver_type = p->solver_type;
  for (int i = 0; i < 6; ++i) {
    P.bc[i] = p->bc[i];
    for (int c = 0; c < 5; ++c) P.inflow[i][c] = p->inflow[i][c];
  }
  return P;
}

int oracle_abi_version(void) { return 1; }

// 0: C library pow (as the compiled reference); 1: libm_pow::pow (its restatement).
int oracle_set_pow_mode(int mode) {
  if (mode != 0 && mode != 1) return -1;
  pow_mode() = mode;
  return 0;
}

// libm_pow::pow and the C library pow over n (x, y) pairs, for the bit check.
int oracle_pow_pair(const double* x, const double* y, long long n, double* mine, double* lib) {
  for (long long i = 0; i < n; ++i) {
    mine[i] = libm_pow::pow(x[i], y[i]);
    lib[i] = std::pow(x[i], y[i]);
  }
  return 0;
}

// Runs `nsteps` driver iterations (dt -> ghost fill -> solve) on one box.
// dt_trace[nsteps] receives each dt; stats[3] (optional) receives Riemann
// solves, Newton iterations and extra guesses tried.
int oracle_run(const oracle_params* p, double* cells, const int* dims,
               const double* dx, int nsteps, double* dt_trace, int nthreads,
               long long* stats) {
  Params P = to_params(p);
  Gas G = make_gas(P.gamma, P.kb_amu);
  if (nthreads > 0) omp_set_num_threads(nthreads);
  BoxGeom g = make_geom(P.ndim, dims);
  Workspace ws;
  IrsStats st;
  IrsStats* stp = stats ? &st : nullptr;
  for (int s = 0; s < nsteps; ++s) {
    double dt;
    switch (P.ndim) {
      case 1: dt = step<1>(P, G, cells, g, dx, ws, stp); break;
      case 2: dt = step<2>(P, G, cells, g, dx, ws, stp); break;
      case 3: dt = step<3>(P, G, cells, g, dx, ws, stp); break;
      default: return -1;
    }
    if (dt_trace) dt_trace[s] = dt;
  }
  if (stats) {
    stats[0] = st.solves;
    stats[1] = st.iterations;
    stats[2] = st.extra_guesses;
  }
  return 0;
}

double oracle_cfl_time_step(const oracle_params* p, const double* cells,
                            const int* dims, const double* dx) {
  Params P = to_params(p);
  Gas G = make_gas(P.gamma, P.kb_amu);
  BoxGeom g = make_geom(P.ndim, dims);
  switch (P.ndim) {
    case 1: return cfl_time_step<1>(G, P.courant, cells, g, dx);
    case 2: return cfl_time_step<2>(G, P.courant, cells, g, dx);
    case 3: return cfl_time_step<3>(G, P.courant, cells, g, dx);
  }
  return -1.0;
}

int oracle_set_boundaries(const oracle_params* p, double* cells,
                          const int* dims) {
  Params P = to_params(p);
  BoxGeom g = make_geom(P.ndim, dims);
  switch (P.ndim) {
    case 1: set_boundaries<1>(P, cells, g); return 0;
    case 2: set_boundaries<2>(P, cells, g); return 0;
    case 3: set_boundaries<3>(P, cells, g); return 0;
  }
  return -1;
}

int oracle_mh_solve(const oracle_params* p, double* cells, const int* dims,
                    const double* dx, double dt, int nthreads) {
  Params P = to_params(p);
  Gas G = make_gas(P.gamma, P.kb_amu);
  if (nthreads > 0) omp_set_num_threads(nthreads);
  BoxGeom g = make_geom(P.ndim, dims);
  Workspace ws;
  switch (P.ndim) {
    case 1:
      if (P.solver_type == kCpuIntensive) mh_solve_cpu_intensive<1>(P, G, cells, g, dx, dt);
      else mh_solve_memory_intensive<1>(P, G, cells, g, dx, dt, ws);
      return 0;
    case 2:
      if (P.solver_type == kCpuIntensive) mh_solve_cpu_intensive<2>(P, G, cells, g, dx, dt);
      else mh_solve_memory_intensive<2>(P, G, cells, g, dx, dt, ws);
      return 0;
    case 3:
      if (P.solver_type == kCpuIntensive) mh_solve_cpu_intensive<3>(P, G, cells, g, dx, dt);
      else mh_solve_memory_intensive<3>(P, G, cells, g, dx, dt, ws);
      return 0;
  }
  return -1;
}

// rhyme_riemann_problem_solve over n interface pairs.
int oracle_riemann_solve(const oracle_params* p, const double* l,
                         const double* r, long long n, double dx, double dt,
                         int axis, double* u) {
  Params P = to_params(p);
  Gas G = make_gas(P.gamma, P.kb_amu);
  const int W = P.ndim + 2;
  for (long long i = 0; i < n; ++i) {
    switch (P.ndim) {
      case 1: rp_solve<1>(G, P.vac_rho, P.vac_p, P.tol, P.n_iter, l + i * W, r + i * W, dx, dt, axis, u + i * W); break;
      case 2: rp_solve<2>(G, P.vac_rho, P.vac_p, P.tol, P.n_iter, l + i * W, r + i * W, dx, dt, axis, u + i * W); break;
      case 3: rp_solve<3>(G, P.vac_rho, P.vac_p, P.tol, P.n_iter, l + i * W, r + i * W, dx, dt, axis, u + i * W); break;
      default: return -1;
    }
  }
  return 0;
}

// rhyme_irs_exec over n state pairs. states[n][8] = (l_rho, l_v, l_p, l_cs,
// r_rho, r_v, r_p, r_cs) with v the normal velocity. out[n][3] = (p*, l_f,
// r_f).
int oracle_irs_exec(double gamma, double tol, int n_iter,
                    const double* states, long long n, double* out) {
  Gas G = make_gas(gamma, 1.0);
  for (long long i = 0; i < n; ++i) {
    const double* s = states + i * 8;
    double lf = 0.0, rf = 0.0;
    double ps = irs_exec(G, tol, n_iter, s[0], s[1], s[2], s[3], lf, s[4],
                         s[5], s[6], s[7], rf);
    out[i * 3 + 0] = ps;
    out[i * 3 + 1] = lf;
    out[i * 3 + 2] = rf;
  }
  return 0;
}

// rhyme_irs_guess_p_star over n state pairs (same layout as above).
int oracle_guess_p_star(double gamma, const double* states, long long n,
                        double* out6) {
  Gas G = make_gas(gamma, 1.0);
  for (long long i = 0; i < n; ++i) {
    const double* s = states + i * 8;
    guess_p_star(G, s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7],
                 out6 + i * 6);
  }
  return 0;
}

// rhyme_irs_nonlinear_wave_function: in[n][4] = (rho, p_k, cs, p); out[n][2].
int oracle_nonlinear_wave(double gamma, const double* in, long long n,
                          double* out) {
  Gas G = make_gas(gamma, 1.0);
  for (long long i = 0; i < n; ++i) {
    const double* s = in + i * 4;
    nonlinear_wave(G, s[0], s[1], s[2], s[3], out[i * 2], out[i * 2 + 1]);
  }
  return 0;
}

// rhyme_riemann_problem_star followed (optionally) by sampling at dx/dt,
// for 1-D states given as sides (rho, v, p, cs) the way the reference test
// factory fills them (rhyme_irs_tests_factory.f90:186-202).
// sides[8] = (l_rho, l_v, l_p, l_cs, r_rho, r_v, r_p, r_cs).
// star_out[10] = (p*, u*, l_is_shock, l_rho*, l_speed/speedH, l_speedT,
//                 r_is_shock, r_rho*, r_speed/speedH, r_speedT).
// If nsample > 0, samples[n] (x/t as dx with dt) fill u_out[n][3].
int oracle_star_and_sample(double gamma, double kb_amu, double vac_p,
                           double tol, int n_iter, const double* sides,
                           double* star_out, const double* sample_dx,
                           double sample_dt, long long nsample,
                           double* u_out) {
  Gas G = make_gas(gamma, kb_amu);
  Solution<1> s;
  s.left.rho = sides[0];
  s.left.v[0] = sides[1];
  s.left.p = sides[2];
  s.left.cs = sides[3];
  s.right.rho = sides[4];
  s.right.v[0] = sides[5];
  s.right.p = sides[6];
  s.right.cs = sides[7];
  rp_star<1>(G, vac_p, tol, n_iter, s, 0);
  star_out[0] = s.star_p;
  star_out[1] = s.star_u;
  star_out[2] = s.sl.is_shock ? 1.0 : 0.0;
  star_out[3] = s.sl.is_shock ? s.sl.shock_rho : s.sl.fan_rho;
  star_out[4] = s.sl.is_shock ? s.sl.shock_speed : s.sl.fan_speedH;
  star_out[5] = s.sl.is_shock ? s.sl.shock_speed : s.sl.fan_speedT;
  star_out[6] = s.sr.is_shock ? 1.0 : 0.0;
  star_out[7] = s.sr.is_shock ? s.sr.shock_rho : s.sr.fan_rho;
  star_out[8] = s.sr.is_shock ? s.sr.shock_speed : s.sr.fan_speedH;
  star_out[9] = s.sr.is_shock ? s.sr.shock_speed : s.sr.fan_speedT;
  for (long long i = 0; i < nsample; ++i)
    rp_sampling<1>(G, s, 0, sample_dx[i], sample_dt, u_out + i * 3);
  return 0;
}

// rhyme_slope_limiter_run over n triples; arrays [n][D+2].
int oracle_slope_limiter(int ndim, int type, double omega, const double* ul,
                         const double* u, const double* ur, long long n,
                         double* delta) {
  const int W = ndim + 2;
  for (long long i = 0; i < n * W; ++i)
    delta[i] = limited_slope(type, omega, ul[i], u[i], ur[i]);
  return 0;
}

// rhyme_muscl_hancock_half_step_extrapolation over n cells.
int oracle_half_step(int ndim, double gamma, const double* u,
                     const double* delta, long long n, int axis, double dx,
                     double dt, double* l, double* r) {
  Gas G = make_gas(gamma, 1.0);
  const int W = ndim + 2;
  for (long long i = 0; i < n; ++i) {
    switch (ndim) {
      case 1: half_step<1>(G, u + i * W, delta + i * W, axis, dx, dt, l + i * W, r + i * W); break;
      case 2: half_step<2>(G, u + i * W, delta + i * W, axis, dx, dt, l + i * W, r + i * W); break;
      case 3: half_step<3>(G, u + i * W, delta + i * W, axis, dx, dt, l + i * W, r + i * W); break;
      default: return -1;
    }
  }
  return 0;
}

// calc_flux / calc_p / calc_cs over n conserved states; out[n][D+2] fluxes,
// p_out[n], cs_out[n].
int oracle_eos(int ndim, double gamma, double kb_amu, const double* u,
               long long n, int axis, double* f, double* p_out,
               double* cs_out) {
  Gas G = make_gas(gamma, kb_amu);
  const int W = ndim + 2;
  for (long long i = 0; i < n; ++i) {
    const double* ui = u + i * W;
    switch (ndim) {
      case 1: flux<1>(G, ui, axis, f + i * W); p_out[i] = pressure<1>(G, ui); cs_out[i] = sound_speed<1>(G, ui); break;
      case 2: flux<2>(G, ui, axis, f + i * W); p_out[i] = pressure<2>(G, ui); cs_out[i] = sound_speed<2>(G, ui); break;
      case 3: flux<3>(G, ui, axis, f + i * W); p_out[i] = pressure<3>(G, ui); cs_out[i] = sound_speed<3>(G, ui); break;
      default: return -1;
    }
  }
  return 0;
}

}  // extern "C"
