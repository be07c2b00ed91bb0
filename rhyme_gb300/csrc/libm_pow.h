// libm_pow.h -- the C library's double-precision pow, restated for host and
// device so that the CUDA kernels return its bits.
//
// Why: Rhyme's Fortran raises pressure ratios to real powers
// (rhyme_irs_nonlinear_wave_function.f90:22-23, rhyme_irs_guess_p_star.f90:
// 28,32,53-55, rhyme_riemann_problem_star.f90:49-50,61-62,
// rhyme_riemann_problem_w_kfan.f90:22,29), and gfortran evaluates each real
// `a**b` by calling pow() from the C library. On Linux that is the GNU C
// Library's pow (glibc 2.28 and later: sysdeps/ieee754/dbl-64/e_pow.c), whose
// algorithm is Szabolcs Nagy's table-driven log and exp from Arm's
// optimized-routines. It is not correctly rounded (about one result in 10^3
// is off by one ulp), so any other pow differs from it somewhere, and flows
// that amplify one-ulp differences (a Kelvin-Helmholtz shear layer, shock
// interactions) then drift away from the reference by 1e-10 and more. This
// header performs the same operations in the same order, so that the FP64
// kernels and the reference agree to the last bit.
//
// The method, for x > 0 normal and finite y:
//  log: x = 2^k z with z in [OFF, 2 OFF), OFF = 0x1.69555p-1, the range cut
//   into 128 pieces by bits 45..51 of bits(z) - bits(OFF); with INVC, LOGC,
//   LOGCTAIL of z's piece, r = z INVC - 1 is exact (one fused multiply-add)
//   and log x = k ln2 + LOGC + LOGCTAIL + log1p(r), carried as hi + lo with
//   log1p(r) = r - r^2/2 + r^3 P(r), P of degree 5, the r^2 term split
//   exactly (Dekker) and every rounding error of the head collected in lo;
//  y log x is formed as ehi + elo with fused multiply-adds;
//  exp: ehi = k ln2/128 + r, |r| <= ln2/256, k rounded to nearest by the
//   2^52 + 2^51 shift; exp = 2^(k/128) (1 + TAIL) e^r with e^r - 1 - r of
//   degree 5, 2^(k/128) built from a table of 128 entries by integer
//   addition to the exponent field; near overflow and underflow the scaling
//   is split so no intermediate overflows and a subnormal result is rounded
//   once.
// glibc is built with GCC, which contracts a*b + c into a fused multiply-add
// where the product has no other use (in the same basic block); those places
// are written here as explicit fma() and every other operation is a separate
// IEEE operation (on the device through __dadd_rn/__dmul_rn, which nvcc never
// contracts; on the host this header must be compiled with
// -ffp-contract=off).
//
// Tables and constants: libm_pow_tables.h, written by libm_pow_tables.py,
// which derives every entry from its published definition and fits the two
// polynomials itself (Remez); the polynomial coefficients are then moved by a
// few ulps (offsets listed in that script) to the values at which this
// restatement agrees with the C library on every argument of the calibration
// sets. Checked: bit-identical to glibc 2.39's pow (x86-64 and AArch64) on
// 10^9 arguments drawn over the solver's exponents and over random
// exponents in [-30, 30] (tests/test_oracle_golden.py runs a smaller set).
#pragma once

#include <cstdint>
#include <cstring>

#ifdef LIBM_POW_TABLES_FILE  // another coefficient set (libm_pow_calibrate.py)
#include LIBM_POW_TABLES_FILE
#else
#include "libm_pow_tables.h"
#endif

#if defined(__CUDACC__)
#define LIBM_POW_HD __host__ __device__ __forceinline__
#else
#define LIBM_POW_HD inline
#include <cmath>
#endif

namespace libm_pow {

static const double kLogHost[4 * 128] = LIBM_POW_LOG_TABLE;
static const uint64_t kExpHost[2 * 128] = LIBM_POW_EXP_TABLE;
#if defined(__CUDACC__)
static __device__ const double kLogDev[4 * 128] = LIBM_POW_LOG_TABLE;
static __device__ const uint64_t kExpDev[2 * 128] = LIBM_POW_EXP_TABLE;
#endif

LIBM_POW_HD const double* log_tab() {
#if defined(__CUDA_ARCH__)
  return kLogDev;
#else
  return kLogHost;
#endif
}
LIBM_POW_HD const uint64_t* exp_tab() {
#if defined(__CUDA_ARCH__)
  return kExpDev;
#else
  return kExpHost;
#endif
}

// Single IEEE operations, never fused with a neighbour.
#if defined(__CUDA_ARCH__)
LIBM_POW_HD double add(double a, double b) { return __dadd_rn(a, b); }
LIBM_POW_HD double sub(double a, double b) { return __dsub_rn(a, b); }
LIBM_POW_HD double mul(double a, double b) { return __dmul_rn(a, b); }
LIBM_POW_HD double fma3(double a, double b, double c) { return __fma_rn(a, b, c); }
LIBM_POW_HD uint64_t bits(double d) { return (uint64_t)__double_as_longlong(d); }
LIBM_POW_HD double from_bits(uint64_t u) { return __longlong_as_double((long long)u); }
#else
LIBM_POW_HD double add(double a, double b) { return a + b; }
LIBM_POW_HD double sub(double a, double b) { return a - b; }
LIBM_POW_HD double mul(double a, double b) { return a * b; }
LIBM_POW_HD double fma3(double a, double b, double c) { return std::fma(a, b, c); }
LIBM_POW_HD uint64_t bits(double d) {
  uint64_t u;
  std::memcpy(&u, &d, sizeof u);
  return u;
}
LIBM_POW_HD double from_bits(uint64_t u) {
  double d;
  std::memcpy(&d, &u, sizeof d);
  return d;
}
#endif

constexpr uint64_t kOffBits = 0x3fe6955500000000ULL;  // bits of 0x1.69555p-1
constexpr uint64_t kOneBits = 0x3ff0000000000000ULL;
constexpr uint64_t kInfBits = 0x7ff0000000000000ULL;
constexpr uint64_t kSignBias = 0x800ULL << 7;  // lands on bit 63 after << 45
constexpr double kShift = 0x1.8p52;

// log of the positive normal number with bit pattern ix, as hi + *tail.
// lo_ulps (calibration only, 0 in the library) moves the low part by that
// many of its ulps before the final split.
LIBM_POW_HD double log_parts(uint64_t ix, double* tail, int lo_ulps = 0) {
  const uint64_t t = ix - kOffBits;
  const int i = (int)((t >> 45) & 127);
  const int k = (int)((int64_t)t >> 52);
  const double z = from_bits(ix - (t & (0xfffULL << 52)));
  const double kd = (double)k;
  const double* e = log_tab() + 4 * i;
  const double invc = e[0], logc = e[1], logctail = e[2];
  const double r = fma3(z, invc, -1.0);  // exact
  // k ln2 + log c + r, with the rounding errors gathered
  const double t1 = fma3(kd, LIBM_POW_LN2_HI, logc);  // exact
  const double t2 = add(t1, r);
  const double lo1 = fma3(kd, LIBM_POW_LN2_LO, logctail);
  const double lo2 = add(sub(t1, t2), r);
  // - r^2/2 split into ar2 + lo3 exactly
  const double ar = mul(-0.5, r);
  const double ar2 = mul(r, ar);
  const double ar3 = mul(r, ar2);
  const double hi = add(t2, ar2);
  const double lo3 = fma3(ar, r, -ar2);
  const double lo4 = add(sub(t2, hi), ar2);
  // log1p(r) - r + r^2/2 = ar3 (A1 + A2 r + ar2 (A3 + A4 r + ar2 (A5 + A6 r)))
  const double p56 = fma3(r, LIBM_POW_A6, LIBM_POW_A5);
  const double p34 = fma3(r, LIBM_POW_A4, LIBM_POW_A3);
  const double p12 = fma3(r, LIBM_POW_A2, LIBM_POW_A1);
  const double q = fma3(ar2, fma3(ar2, p56, p34), p12);
  double lo = fma3(ar3, q, add(add(add(lo1, lo2), lo3), lo4));
  if (lo_ulps) lo = from_bits(bits(lo) + (int64_t)lo_ulps * ((lo > 0.0) ? 1 : -1));
  const double y = add(hi, lo);
  *tail = add(sub(hi, y), lo);
  return y;
}

// Results whose exponent lies outside the normal scaling (|x| in [512, 1024)).
LIBM_POW_HD double exp_edge(double tmp, uint64_t sbits, uint64_t ki) {
  if ((ki & 0x80000000ULL) == 0) {
    // large result: scale by 2^1009 in two steps
    const double scale = from_bits(sbits - (1009ULL << 52));
    return mul(0x1p1009, fma3(scale, tmp, scale));
  }
  // small result: form it at 2^1022 times its size, round once, scale down
  sbits += 1022ULL << 52;  // now a signed scale within range
  const double scale = from_bits(sbits);
  const double st = mul(scale, tmp);
  double y = add(scale, st);
#if defined(__CUDA_ARCH__)
  const double ay = fabs(y);
#else
  const double ay = std::fabs(y);
#endif
  if (ay < 1.0) {
    const double one = (y < 0.0) ? -1.0 : 1.0;
    double lo = add(sub(scale, y), st);
    const double hi = add(one, y);
    lo = add(add(sub(one, hi), y), lo);
    y = sub(add(hi, lo), one);
    if (y == 0.0) y = from_bits(sbits & 0x8000000000000000ULL);
  }
  return mul(0x1p-1022, y);
}

// Intermediates of exp_parts for the calibration (not used by the library).
struct ExpTrace {
  double r, r4, u, tmp, scale;
};

// e^(x + xtail), negated when sign_bias is kSignBias.
LIBM_POW_HD double exp_parts(double x, double xtail, uint64_t sign_bias, ExpTrace* trace = nullptr) {
  uint32_t abstop = (uint32_t)(bits(x) >> 52) & 0x7ff;
  if (abstop - 0x3c9u >= 0x408u - 0x3c9u) {  // |x| < 2^-54 or |x| >= 512
    if ((int32_t)(abstop - 0x3c9u) < 0) {
      const double one = add(1.0, x);
      return sign_bias ? -one : one;
    }
    if (abstop >= 0x409u) {  // |x| >= 1024
      if (bits(x) >> 63) return sign_bias ? -0.0 : 0.0;
      return sign_bias ? -__builtin_huge_val() : __builtin_huge_val();
    }
    abstop = 0;  // 512 <= |x| < 1024: exp_edge below
  }
  const double kd0 = fma3(LIBM_POW_INV_LN2_N, x, kShift);
  const uint64_t ki = bits(kd0);
  const double kd = sub(kd0, kShift);
  double r = fma3(kd, LIBM_POW_NEG_LN2_LO_N, fma3(kd, LIBM_POW_NEG_LN2_HI_N, x));
  r = add(r, xtail);
  const uint64_t* e = exp_tab() + 2 * (ki & 127);
  const uint64_t top = (ki + sign_bias) << 45;
  const double tail = from_bits(e[0]);
  const uint64_t sbits = e[1] + top;
  const double r2 = mul(r, r);
  const double r4 = mul(r2, r2);
  const double u = fma3(r2, fma3(r, LIBM_POW_C3, LIBM_POW_C2), add(tail, r));
  const double tmp = fma3(r4, fma3(r, LIBM_POW_C5, LIBM_POW_C4), u);
  if (abstop == 0) return exp_edge(tmp, sbits, ki);
  const double scale = from_bits(sbits);
  if (trace) *trace = {r, r4, u, tmp, scale};
  return fma3(scale, tmp, scale);
}

// A NaN whose quiet bit (the top mantissa bit) is clear.
LIBM_POW_HD bool is_signalling(uint64_t u) {
  return 2 * (u ^ 0x0008000000000000ULL) > 2 * 0x7ff8000000000000ULL;
}

// 0: y is not an integer; 1: odd integer; 2: even integer (y finite, nonzero).
LIBM_POW_HD int integer_kind(uint64_t iy) {
  const int e = (int)((iy >> 52) & 0x7ff);
  if (e < 0x3ff) return 0;
  if (e > 0x3ff + 52) return 2;
  if (iy & ((1ULL << (0x3ff + 52 - e)) - 1)) return 0;
  if (iy & (1ULL << (0x3ff + 52 - e))) return 1;
  return 2;
}

// x**y with the C library's results, including the special values of C99
// Annex F (the hydro path only raises positive finite ratios).
LIBM_POW_HD double pow(double x, double y) {
  uint64_t ix = bits(x);
  const uint64_t iy = bits(y);
  uint32_t topx = (uint32_t)(ix >> 52);
  const uint32_t topy = (uint32_t)(iy >> 52);
  uint64_t sign_bias = 0;
  if (topx - 0x001u >= 0x7ff - 0x001u || (topy & 0x7ff) - 0x3beu >= 0x43e - 0x3beu) {
    // x is subnormal, zero, negative, infinite or NaN, or |y| < 2^-65,
    // |y| >= 2^63, or y is zero, infinite or NaN
    if (2 * iy - 1 >= 2 * kInfBits - 1) {  // y is +-0, +-inf or NaN
      // x**0 and 1**y are 1, except for a signalling NaN operand
      if (2 * iy == 0) return is_signalling(ix) ? add(x, y) : 1.0;
      if (ix == kOneBits) return is_signalling(iy) ? add(x, y) : 1.0;
      if (2 * ix > 2 * kInfBits || 2 * iy > 2 * kInfBits) return add(x, y);
      if (2 * ix == 2 * kOneBits) return 1.0;  // (-1)**(+-inf)
      if ((2 * ix < 2 * kOneBits) == !(iy >> 63)) return 0.0;
      return mul(y, y);  // +inf
    }
    if (2 * ix - 1 >= 2 * kInfBits - 1) {  // x is +-0, +-inf or NaN
      double x2 = mul(x, x);
      if ((ix >> 63) && integer_kind(iy) == 1) x2 = -x2;
      return (iy >> 63) ? 1.0 / x2 : x2;
    }
    if (ix >> 63) {  // x finite and negative
      const int kind = integer_kind(iy);
      if (kind == 0) return __builtin_nan("");
      if (kind == 1) sign_bias = kSignBias;
      ix &= 0x7fffffffffffffffULL;
      topx &= 0x7ff;
    }
    if ((topy & 0x7ff) - 0x3beu >= 0x43e - 0x3beu) {
      if (ix == kOneBits) return 1.0;
      if ((topy & 0x7ff) < 0x3be) return (ix > kOneBits) ? add(1.0, y) : sub(1.0, y);  // |y| tiny
      // |y| huge: overflow or underflow
      return ((ix > kOneBits) == (topy < 0x800)) ? __builtin_huge_val() : 0.0;
    }
    if (topx == 0) {  // subnormal x: normalise
      ix = bits(mul(x, 0x1p52));
      ix &= 0x7fffffffffffffffULL;
      ix -= 52ULL << 52;
    }
  }
  double lo;
  const double hi = log_parts(ix, &lo);
  const double ehi = mul(y, hi);
  const double elo = fma3(y, lo, fma3(y, hi, -ehi));
  return exp_parts(ehi, elo, sign_bias);
}

// x**y1 and x**y2 of one base sharing the logarithm: the same bits as two
// pow calls.
LIBM_POW_HD void pow2(double x, double y1, double y2, double* r1, double* r2) {
  const uint64_t ix = bits(x);
  const uint32_t topx = (uint32_t)(ix >> 52);
  const uint32_t t1 = (uint32_t)(bits(y1) >> 52) & 0x7ff, t2 = (uint32_t)(bits(y2) >> 52) & 0x7ff;
  if (topx - 0x001u >= 0x7ff - 0x001u || t1 - 0x3beu >= 0x43e - 0x3beu || t2 - 0x3beu >= 0x43e - 0x3beu) {
    *r1 = pow(x, y1);
    *r2 = pow(x, y2);
    return;
  }
  double lo;
  const double hi = log_parts(ix, &lo);
  double e = mul(y1, hi);
  *r1 = exp_parts(e, fma3(y1, lo, fma3(y1, hi, -e)), 0);
  e = mul(y2, hi);
  *r2 = exp_parts(e, fma3(y2, lo, fma3(y2, hi, -e)), 0);
}

}  // namespace libm_pow
