// detmath.h -- a deterministic double-precision power function for host and
// device.
//
// Why: the hot path raises pressure ratios to fixed real powers (the
// Riemann solver's rarefaction and fan relations). CUDA's pow and the host
// libm pow may round a result differently in the last bit, and in unstable
// flows (a Kelvin-Helmholtz shear layer, say) one flipped bit grows to 1e-10
// .. 1e-7 relative after a few hundred steps. det_pow uses only IEEE
// additions, multiplications, divisions and explicit fma, in a fixed order,
// so the CUDA kernels and a host build (compiled without FMA contraction)
// return bit-identical results.
//
// Method (table-driven, tables in detmath_tables.h, written by
// detmath_tables.py with 200-bit mpmath):
//  - log: x = 2^k m, m in [1, 2); with ic = RN(1/c) for the centre c of m's
//    interval of width 1/128, r = m ic - 1 is formed exactly as a
//    double-double (TwoProduct, then p - 1 is exact) and |r| < 2^-8;
//    log x = k ln2 + log(1/ic) + log1p(r), the table holding log(1/ic) and
//    2^(j/64) as double-doubles, log1p by its Taylor series to r^8/8.
//  - the product y*log(x) is formed in double-double;
//  - exp: t = n ln2/64 + r, exp(t) = 2^(n div 64) 2^((n mod 64)/64) exp(r),
//    exp(r) = 1 + r + r^2 (1/2! + ... + r^5/7!), |r| <= ln2/128.
// Error before the final rounding about 2^-67 relative, so results are
// correctly rounded except in about 1 case in 10^4 (measured against
// 200-bit references: 99.99 %); the C library's pow is correctly rounded in
// 99.9 % of the same cases, and the two agree to the last bit as often.
// The error-free transforms are Knuth's TwoSum and Dekker's Fast2Sum, and
// TwoProduct with a fused multiply-add.
#pragma once

#include "detmath_tables.h"

#if defined(__CUDACC__)
#define RGPU_HD __host__ __device__ __forceinline__
#else
#define RGPU_HD inline
#include <cmath>
#endif

namespace detmath {

struct dd {
  double hi, lo;
};

#if defined(__CUDA_ARCH__)
RGPU_HD double d_fma(double a, double b, double c) { return fma(a, b, c); }
RGPU_HD double d_frexp(double x, int* e) { return frexp(x, e); }
RGPU_HD double d_ldexp(double x, int e) { return ldexp(x, e); }
RGPU_HD double d_rint(double x) { return rint(x); }
RGPU_HD bool d_isnan(double x) { return isnan(x); }
RGPU_HD bool d_isinf(double x) { return isinf(x); }
#else
RGPU_HD double d_fma(double a, double b, double c) { return std::fma(a, b, c); }
RGPU_HD double d_frexp(double x, int* e) { return std::frexp(x, e); }
RGPU_HD double d_ldexp(double x, int e) { return std::ldexp(x, e); }
RGPU_HD double d_rint(double x) { return std::rint(x); }
RGPU_HD bool d_isnan(double x) { return std::isnan(x); }
RGPU_HD bool d_isinf(double x) { return std::isinf(x); }
#endif

// Knuth's TwoSum: s + e == a + b exactly.
RGPU_HD dd two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
// Dekker's Fast2Sum, valid for |a| >= |b|.
RGPU_HD dd fast_two_sum(double a, double b) {
  double s = a + b;
  double e = b - (s - a);
  return {s, e};
}
// TwoProduct with a fused multiply-add: p + e == a * b exactly.
RGPU_HD dd two_prod(double a, double b) {
  double p = a * b;
  double e = d_fma(a, b, -p);
  return {p, e};
}
RGPU_HD dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  double e = s.lo + (a.lo + b.lo);
  return fast_two_sum(s.hi, e);
}

// ln 2 = LN2_HI + LN2_LO, LN2_HI with its low 21 bits zero (k*LN2_HI exact
// for |k| < 2^21).
constexpr double LN2_HI = 6.93147180369123816490e-01;
constexpr double LN2_LO = 1.90821492927058770002e-10;

// The tables of detmath_tables.h, one copy for host code and one in device
// memory (read through L1 by the lanes of a warp at different indices).
static const double kInvcHost[128] = DETMATH_INVC_TABLE;
static const double kLogcHost[256] = DETMATH_LOGC_TABLE;
static const double kExp2Host[128] = DETMATH_EXP2_TABLE;
#if defined(__CUDACC__)
static __device__ const double kInvcDev[128] = DETMATH_INVC_TABLE;
static __device__ const double kLogcDev[256] = DETMATH_LOGC_TABLE;
static __device__ const double kExp2Dev[128] = DETMATH_EXP2_TABLE;
#endif
RGPU_HD const double* invc_tab() {
#if defined(__CUDA_ARCH__)
  return kInvcDev;
#else
  return kInvcHost;
#endif
}
RGPU_HD const double* logc_tab() {
#if defined(__CUDA_ARCH__)
  return kLogcDev;
#else
  return kLogcHost;
#endif
}
RGPU_HD const double* exp2_tab() {
#if defined(__CUDA_ARCH__)
  return kExp2Dev;
#else
  return kExp2Host;
#endif
}

// log(x) as a double-double, x positive, finite and non-zero. x = m 2^k with
// m in [1, 2); with c the centre of m's interval of width 1/128 and
// ic = RN(1/c), r = m ic - 1 is formed exactly (|r| < 2^-8) and
// log x = k ln2 - log(ic) + log1p(r), log1p(r) = r - r^2/2 + ... - r^8/8
// (the next term is below 2^-72).
RGPU_HD dd log_dd(double x) {
  int k;
  double m = d_frexp(x, &k);  // x = m 2^k, m in [0.5, 1)
  m = m * 2.0;
  k = k - 1;
  const int i = (int)((m - 1.0) * 128.0);  // m - 1 and the scaling are exact
  const double ic = invc_tab()[i];
  const dd p = two_prod(m, ic);
  const dd r = two_sum(p.hi - 1.0, p.lo);  // p.hi - 1 is exact (p.hi near 1)
  const double x1 = r.hi;
  double P = -1.0 / 8.0;
  P = d_fma(P, x1, 1.0 / 7.0);
  P = d_fma(P, x1, -1.0 / 6.0);
  P = d_fma(P, x1, 1.0 / 5.0);
  P = d_fma(P, x1, -1.0 / 4.0);
  P = d_fma(P, x1, 1.0 / 3.0);
  P = d_fma(P, x1, -0.5);
  // log1p(r) - r.hi = r.lo (1 - r.hi) + r.hi^2 P
  const double low = r.lo + d_fma(-r.lo, x1, (x1 * x1) * P);
  const double kd = (double)k;
  const double* lc = logc_tab() + 2 * i;
  const dd s1 = two_sum(kd * LN2_HI, lc[0]);
  const dd s2 = two_sum(s1.hi, x1);
  const double lo = ((s1.lo + s2.lo) + (lc[1] + kd * LN2_LO)) + low;
  return fast_two_sum(s2.hi, lo);
}

// exp(t) for a double-double t: t = n ln2/64 + r, |r| <= ln2/128 (to the
// rounding of n), exp(t) = 2^(n div 64) 2^((n mod 64)/64) exp(r) with
// exp(r) = 1 + r + r^2 (1/2 + r/6 + ... + r^5/7!) (the next term is below
// 2^-74) and 2^(j/64) a double-double from the table.
RGPU_HD double exp_dd(dd t) {
  if (t.hi > 709.782712893384) return __builtin_huge_val();
  if (t.hi < -745.2) return 0.0;
  const double n = d_rint(t.hi * DETMATH_INV_LN2_64);  // |n| < 2^17
  const double a = d_fma(-n, DETMATH_LN2_64_HI, t.hi);  // exact: n*HI is exact and close to t.hi
  const double b = d_fma(-n, DETMATH_LN2_64_LO, t.lo);
  const dd r = two_sum(a, b);
  const double x = r.hi;
  double Q = 1.0 / 5040.0;
  Q = d_fma(Q, x, 1.0 / 720.0);
  Q = d_fma(Q, x, 1.0 / 120.0);
  Q = d_fma(Q, x, 1.0 / 24.0);
  Q = d_fma(Q, x, 1.0 / 6.0);
  Q = d_fma(Q, x, 0.5);
  // exp(r) = (1 + x) + [x^2 Q + r.lo (1 + x)]
  const double q = d_fma(x * x, Q, d_fma(r.lo, x, r.lo));
  const dd e1 = fast_two_sum(1.0, x);
  const double e_lo = e1.lo + q;
  const long long ni = (long long)n;
  const int j = (int)(ni & 63);          // n mod 64 in [0, 63]
  const int sc = (int)((ni - j) / 64);   // n div 64 (floor)
  const double* T = exp2_tab() + 2 * j;
  const dd pr = two_prod(T[0], e1.hi);
  const double lo = d_fma(T[0], e_lo, d_fma(T[1], e1.hi, pr.lo));
  const double res = pr.hi + lo;
  if (sc > -1000 && sc < 1000) return d_ldexp(res, sc);
  // scale in two steps near the range ends
  return d_ldexp(d_ldexp(res, sc / 2), sc - sc / 2);
}

// x**y for the exponents the hydro path uses (any finite y); special values
// follow the usual pow conventions for the cases that can occur there.
RGPU_HD double det_pow(double x, double y) {
  if (y == 0.0 || x == 1.0) return 1.0;
  if (d_isnan(x) || d_isnan(y)) return x + y;
  if (x == 0.0) return (y > 0.0) ? 0.0 : __builtin_huge_val();
  if (x < 0.0) {
    if (d_rint(y) != y) return (x - x) / (x - x);  // NaN
    const double r = det_pow(-x, y);
    const double half = 0.5 * y;
    return (d_rint(half) != half) ? -r : r;  // odd integer y
  }
  if (d_isinf(x)) return (y > 0.0) ? x : 0.0;
  const dd l = log_dd(x);
  const dd p = two_prod(y, l.hi);
  const dd t = fast_two_sum(p.hi, d_fma(y, l.lo, p.lo));
  return exp_dd(t);
}

// x**y1 and x**y2 sharing one logarithm (the rarefaction wave function and
// the fan relations raise one ratio to two powers).
RGPU_HD void det_pow2(double x, double y1, double y2, double* r1, double* r2) {
  if (!(x > 0.0) || d_isinf(x) || x == 1.0 || y1 == 0.0 || y2 == 0.0) {
    *r1 = det_pow(x, y1);
    *r2 = det_pow(x, y2);
    return;
  }
  const dd l = log_dd(x);
  dd p = two_prod(y1, l.hi);
  *r1 = exp_dd(fast_two_sum(p.hi, d_fma(y1, l.lo, p.lo)));
  p = two_prod(y2, l.hi);
  *r2 = exp_dd(fast_two_sum(p.hi, d_fma(y2, l.lo, p.lo)));
}

}  // namespace detmath
