/* libm_pow_calibrate.cpp -- data for libm_pow_calibrate.py (build-time tool).
 *
 * Compiled against libm_pow.h with a candidate coefficient header
 * (-DLIBM_POW_TABLES_FILE=...), and run against this machine's C library
 * pow, which the restatement must reproduce.
 *
 *   log NB NE SEED   for NB bases x, the whole number k of ulps by which the
 *                    library's low part of log(x) differs from the
 *                    restatement's: the k in [-6, 6] for which the
 *                    restatement, its low part moved by k ulps, returns the
 *                    library's pow(x, y) for all NE exponents y (chosen so
 *                    that |y log x| is 300..500, where the last bits of the
 *                    logarithm reach the result). Prints "x k" for the bases
 *                    with exactly one such k.
 *   exp N THR SEED   N random (x, y); for those whose result lies within THR
 *                    ulp of a rounding boundary, the interval of
 *                    C4 + r*C5 (as an offset from the candidate's) for which
 *                    the final rounding gives the library's result. Prints
 *                    "r lo hi".
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <quadmath.h>

#include "libm_pow.h"

using libm_pow::bits;
using libm_pow::from_bits;

static unsigned long long g_s;
static unsigned long long next_u64() {
  g_s ^= g_s >> 12;
  g_s ^= g_s << 25;
  g_s ^= g_s >> 27;
  return g_s * 2685821657736338717ULL;
}
static double unit() { return (double)(next_u64() >> 11) * 0x1p-53; }

static double pow_shifted(double x, double y, int k) {
  double lo;
  const double hi = libm_pow::log_parts(bits(x), &lo, k);
  const double ehi = y * hi;
  const double elo = std::fma(y, lo, std::fma(y, hi, -ehi));
  return libm_pow::exp_parts(ehi, elo, 0);
}

static int run_log(long nb, long ne, unsigned long long seed) {
#pragma omp parallel for schedule(dynamic, 16)
  for (long i = 0; i < nb; ++i) {
    unsigned long long s = seed ^ ((unsigned long long)(i + 1) * 0x9E3779B97F4A7C15ULL);
    s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
    const unsigned long long b = s * 2685821657736338717ULL;
    const double u = (double)(b >> 11) * 0x1p-53;
    double x;
    if (i % 2 == 0) {  // the two pieces around 1 (largest |r|, logc = 0)
      const double d = 0.0004 + 0.0048 * u;
      x = (b & 1) ? 1.0 + d : 1.0 - d;
    } else {  // anywhere in [OFF, 2 OFF)
      x = 0.70573 + 0.7 * u;
    }
    const double L = std::log(x);
    long miss[13] = {0};
    for (long j = 0; j < ne; ++j) {
      double y = (300.0 + 200.0 * (j + 0.5) / ne) / L;
      if (j & 1) y = -y;
      const double R = std::pow(x, y);
      for (int k = -6; k <= 6; ++k)
        if (bits(pow_shifted(x, y, k)) != bits(R)) miss[k + 6]++;
    }
    int best = 0, nz = 0;
    for (int k = -6; k <= 6; ++k)
      if (miss[k + 6] == 0) {
        best = k;
        ++nz;
      }
    if (nz == 1) {
#pragma omp critical
      printf("%a %d\n", x, best);
    }
  }
  return 0;
}

static int run_exp(long n, double thr, unsigned long long seed) {
  g_s = seed;
  for (long i = 0; i < n; ++i) {
    const unsigned long long b = next_u64(), c = next_u64();
    const int e = -20 + (int)((b >> 52) % 41);
    const double x = from_bits(((unsigned long long)(1023 + e) << 52) | (c & ((1ULL << 52) - 1)));
    const double y = unit() * 16.0 - 8.0;
    double lo;
    const double hi = libm_pow::log_parts(bits(x), &lo);
    const double ehi = y * hi;
    const double elo = std::fma(y, lo, std::fma(y, hi, -ehi));
    const unsigned top = (unsigned)(bits(ehi) >> 52) & 0x7ff;
    if (top - 0x3c9u >= 0x408u - 0x3c9u) continue;  // tiny, or the edge scaling
    libm_pow::ExpTrace t;
    const double E = libm_pow::exp_parts(ehi, elo, 0, &t);
    const __float128 V = (__float128)t.scale * (__float128)t.tmp + (__float128)t.scale;
    const double ulp = from_bits(bits(E) + 1) - E;
    const double d = (double)((V - (__float128)E) / (__float128)ulp);
    if (std::fabs(std::fabs(d) - 0.5) > thr) continue;
    const double R = std::pow(x, y);
    // the doubles tmp with RN(scale (1 + tmp)) == R, then the pre-rounding
    // values of tmp that round to them, then C4 + r C5
    const double up = from_bits(bits(R) + 1) - R, dn = R - from_bits(bits(R) - 1);
    const __float128 Tlo = (((__float128)R - (__float128)dn / 2) - (__float128)t.scale) / (__float128)t.scale;
    const __float128 Thi = (((__float128)R + (__float128)up / 2) - (__float128)t.scale) / (__float128)t.scale;
    double tmin = (double)Tlo;
    if ((__float128)tmin < Tlo) tmin = std::nextafter(tmin, INFINITY);
    double tmax = (double)Thi;
    if ((__float128)tmax > Thi) tmax = std::nextafter(tmax, -INFINITY);
    if (tmin > tmax) continue;
    const __float128 Plo = (__float128)tmin - (__float128)(tmin - std::nextafter(tmin, -INFINITY)) / 2;
    const __float128 Phi = (__float128)tmax + (__float128)(std::nextafter(tmax, INFINITY) - tmax) / 2;
    const __float128 vb = (__float128)LIBM_POW_C4 + (__float128)t.r * (__float128)LIBM_POW_C5;
    const __float128 vlo = (Plo - (__float128)t.u) / (__float128)t.r4 - vb;
    const __float128 vhi = (Phi - (__float128)t.u) / (__float128)t.r4 - vb;
    printf("%a %a %a\n", t.r, (double)vlo, (double)vhi);
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 5 && !strcmp(argv[1], "log")) return run_log(atol(argv[2]), atol(argv[3]), strtoull(argv[4], 0, 10));
  if (argc == 5 && !strcmp(argv[1], "exp")) return run_exp(atol(argv[2]), atof(argv[3]), strtoull(argv[4], 0, 10));
  fprintf(stderr, "usage: %s log NBASES NEXPS SEED | exp N THRESHOLD SEED\n", argv[0]);
  return 2;
}
