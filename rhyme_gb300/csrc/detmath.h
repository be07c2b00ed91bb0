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
// Method (textbook, no tables):
//  - log: x = 2^k m with m in [sqrt(1/2), sqrt(2)); f = m - 1 (exact);
//    log(m) = 2 atanh(s), s = f / (2 + f), summed as 2s + 2s^3 (1/3 + s^2/5
//    + ... + s^22/25), with s and the leading term carried in double-double
//    (Dekker's and Knuth's error-free TwoProduct / TwoSum); then k ln2 added
//    with ln2 split into a 32-bit head and a tail so k*head is exact.
//  - the product y*log(x) is formed in double-double;
//  - exp: n = nearest integer to t/ln2, r = t - n ln2 (double-double),
//    exp(r) = 1 + r + r^2 (1/2! + r/3! + ... + r^14/16!) and 2^n applied
//    exactly.
// Relative error before the final rounding is about 2^-55 for |y log x| up
// to ~20, i.e. results are faithfully rounded (usually correctly rounded).
#pragma once

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
constexpr double INV_LN2 = 1.44269504088896338700e+00;
constexpr double SQRT1_2 = 7.07106781186547572737e-01;

// log(x) as a double-double, x positive, finite and non-zero.
RGPU_HD dd log_dd(double x) {
  int k;
  double m = d_frexp(x, &k);  // x = m 2^k, m in [0.5, 1)
  if (m < SQRT1_2) {
    m = m * 2.0;
    k = k - 1;
  }
  const double f = m - 1.0;       // exact for m in [0.5, 2]
  const dd den = two_sum(2.0, f);  // 2 + f
  const double s = f / den.hi;
  const double res = d_fma(-s, den.hi, f) - s * den.lo;  // f - s*(2+f)
  const double s_lo = res / den.hi;
  const double s2 = s * s;
  double P = 1.0 / 25.0;
  P = d_fma(P, s2, 1.0 / 23.0);
  P = d_fma(P, s2, 1.0 / 21.0);
  P = d_fma(P, s2, 1.0 / 19.0);
  P = d_fma(P, s2, 1.0 / 17.0);
  P = d_fma(P, s2, 1.0 / 15.0);
  P = d_fma(P, s2, 1.0 / 13.0);
  P = d_fma(P, s2, 1.0 / 11.0);
  P = d_fma(P, s2, 1.0 / 9.0);
  P = d_fma(P, s2, 1.0 / 7.0);
  P = d_fma(P, s2, 1.0 / 5.0);
  P = d_fma(P, s2, 1.0 / 3.0);
  const double tail = (2.0 * s) * (s2 * P);
  const dd lm = fast_two_sum(2.0 * s, d_fma(2.0, s_lo, tail));
  const double kd = (double)k;
  const dd kl = fast_two_sum(kd * LN2_HI, kd * LN2_LO);
  if (k == 0) return lm;
  return dd_add(kl, lm);
}

// exp(t) for a double-double t.
RGPU_HD double exp_dd(dd t) {
  if (t.hi > 709.782712893384) return __builtin_huge_val();
  if (t.hi < -745.2) return 0.0;
  const double n = d_rint(t.hi * INV_LN2);
  const double a = d_fma(-n, LN2_HI, t.hi);  // exact: n*LN2_HI is exact and close to t.hi
  const double b = d_fma(-n, LN2_LO, t.lo);
  const dd r = fast_two_sum(a, b);
  const double x = r.hi;
  double Q = 1.0 / 20922789888000.0;  // 1/16!
  Q = d_fma(Q, x, 1.0 / 1307674368000.0);
  Q = d_fma(Q, x, 1.0 / 87178291200.0);
  Q = d_fma(Q, x, 1.0 / 6227020800.0);
  Q = d_fma(Q, x, 1.0 / 479001600.0);
  Q = d_fma(Q, x, 1.0 / 39916800.0);
  Q = d_fma(Q, x, 1.0 / 3628800.0);
  Q = d_fma(Q, x, 1.0 / 362880.0);
  Q = d_fma(Q, x, 1.0 / 40320.0);
  Q = d_fma(Q, x, 1.0 / 5040.0);
  Q = d_fma(Q, x, 1.0 / 720.0);
  Q = d_fma(Q, x, 1.0 / 120.0);
  Q = d_fma(Q, x, 1.0 / 24.0);
  Q = d_fma(Q, x, 1.0 / 6.0);
  Q = d_fma(Q, x, 0.5);
  // exp(r) - 1 - r = r^2 Q(r) + r_lo*r (second order in the tail)
  const double q = d_fma(x * x, Q, r.lo * x);
  const dd one_r = fast_two_sum(1.0, x);
  const double lo = one_r.lo + (r.lo + q);
  const double res = one_r.hi + lo;
  const int ni = (int)n;
  if (ni > -1000 && ni < 1000) return d_ldexp(res, ni);
  // scale in two steps near the range ends
  return d_ldexp(d_ldexp(res, ni / 2), ni - ni / 2);
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
