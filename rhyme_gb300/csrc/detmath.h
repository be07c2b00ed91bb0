// detmath.h -- error-free transforms for double-double sums (host and
// device).
//
// The conservation totals (kernels_sanity.cu) accumulate in double-double so
// that their result is the exact sum rounded once, whatever the launch shape.
// Knuth's TwoSum and Dekker's Fast2Sum; the operations are plain IEEE
// additions in a fixed order (compiled without FMA contraction).
#pragma once

#if defined(__CUDACC__)
#define RGPU_HD __host__ __device__ __forceinline__
#else
#define RGPU_HD inline
#endif

namespace detmath {

struct dd {
  double hi, lo;
};

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

}  // namespace detmath
