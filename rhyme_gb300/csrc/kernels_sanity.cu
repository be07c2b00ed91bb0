// kernels_sanity.cu -- device sanity checks and conservation totals of a box.
//
// rhyme_samr_calc_total_mass.f90 / _total_energy.f90: sums over every cell of
// the box, ghosts included, of rho (e_tot) where it is > 0. Accumulated in
// double-double (error-free TwoSum per addition, then a tree of
// double-double sums) and rounded once at the end, so the result is the
// exact sum correctly rounded (but for ties at the 2^-104 level) whatever the
// launch shape; the reference's sequential sum differs from it by its own
// rounding errors.
//
// rhyme_sanity_check_perform.f90:34-90 (NaN per field, minimum of rho and
// e_tot with its first position) and rhyme_sanity_check_fill.f90:75-185 (per
// property: how many interior cells fall below / above a range, the most
// extreme such value with its first position in Fortran loop order, and the
// running extreme just before it) over the interior cells. Each block takes a
// contiguous run of cells in loop order, so a second pass over the block
// partials in block order reproduces the sequential loop's first-occurrence
// ties and its running extremes.
#include <cfloat>

#include "detmath.h"
#include "rgpu_internal.h"

namespace rgpu {

namespace {

constexpr int kSanThreads = 256;

using DD = detmath::dd;

// Double-double accumulation (Dekker/Knuth error-free sums): a running sum
// carried to about 2^-104 relative to the sum of magnitudes.
__device__ __forceinline__ DD dd_add1(DD a, double b) {
  const DD s = detmath::two_sum(a.hi, b);
  return detmath::fast_two_sum(s.hi, s.lo + a.lo);
}

__device__ __forceinline__ DD acc_add(DD a, DD b) {
  const DD s = detmath::two_sum(a.hi, b.hi);
  return detmath::fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

template <int D>
__device__ __forceinline__ double sc_value(int p, const double* u, const Gas<double>& G) {
  switch (p) {
    case SC_RHO: return u[0];
    case SC_VX: return u[1] / u[0];
    case SC_VY: return D > 1 ? u[2 % (D + 2)] / u[0] : 0.0;
    case SC_VZ: return D > 2 ? u[3 % (D + 2)] / u[0] : 0.0;
    case SC_E_TOT: return u[D + 1];
    default: {
      double ss = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) ss = ss + u[1 + a] * u[1 + a];
      const double v = sqrt(ss) / u[0];
      return (p == SC_ABS_V) ? v : v / sound_speed<D>(G, u);
    }
  }
}

// Sequential fold of one value into a partial (the loop body of the
// reference's update_info for one property).
__device__ __forceinline__ void fold(SanityPartial& s, int p, double v, long long idx, const double* rng) {
  if (v < rng[0]) {
    s.nbelow[p]++;
    if (v < s.vbelow[p]) {
      s.pbelow[p] = s.vbelow[p];
      s.vbelow[p] = v;
      s.ibelow[p] = idx;
    }
  }
  if (v > rng[1]) {
    s.nabove[p]++;
    if (v > s.vabove[p]) {
      s.pabove[p] = s.vabove[p];
      s.vabove[p] = v;
      s.iabove[p] = idx;
    }
  }
}

__device__ __forceinline__ void init_partial(SanityPartial& s) {
  for (int p = 0; p < SC_COUNT; ++p) {
    s.nbelow[p] = s.nabove[p] = 0;
    s.vbelow[p] = s.pbelow[p] = DBL_MAX;  // huge(0d0), as the reference initialises them
    s.vabove[p] = s.pabove[p] = -DBL_MAX;
    s.ibelow[p] = s.iabove[p] = -1;
  }
  for (int c = 0; c < 5; ++c) s.nan[c] = 0;
  s.rho_min = s.e_min = HUGE_VAL;
  s.irho_min = s.ie_min = -1;
}

// Interior cell t (Fortran order) -> its state.
template <int D>
__device__ __forceinline__ void load_cell(const double* __restrict__ U, const Geom& g, long long t, double* u) {
  const long long n0 = g.n[0], n1 = g.n[1];
  const int i = (int)(t % n0) + 1;
  const long long q = t / n0;
  const int j = (int)(q % n1) + 1;
  const int k = (int)(q / n1) + 1;
  const long long o = g.at(D, i, j, k);
#pragma unroll
  for (int c = 0; c < D + 2; ++c) u[c] = U[(long long)c * g.field + o];
}

// Pass 1: block b folds the contiguous run [b0, b1) of interior cells (in
// Fortran loop order). Each thread folds a contiguous sub-run of it, and
// thread 0 merges the sub-run partials in thread order, which is loop order.
template <int D>
__global__ void __launch_bounds__(kSanThreads)
    sanity_pass1(const double* __restrict__ U, Geom g, Gas<double> G, SanityRanges R,
                 SanityPartial* __restrict__ parts, long long per_block) {
  const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
  const long long b0 = (long long)blockIdx.x * per_block;
  const long long b1 = min(total, b0 + per_block);
  // each thread folds a contiguous sub-run; sub-runs are merged in order
  __shared__ SanityPartial sh[32];
  const long long len = (b1 > b0) ? b1 - b0 : 0;
  const long long per_t = (len + kSanThreads - 1) / kSanThreads;
  const long long t0 = b0 + (long long)threadIdx.x * per_t;
  const long long t1 = min(b1, t0 + per_t);
  SanityPartial s;
  init_partial(s);
  double u[D + 2];
  for (long long t = t0; t < t1; ++t) {
    load_cell<D>(U, g, t, u);
    for (int c = 0; c < D + 2; ++c)
      if (isnan(u[c])) s.nan[c] = 1;
    if (u[0] < s.rho_min) {
      s.rho_min = u[0];
      s.irho_min = t;
    }
    if (u[D + 1] < s.e_min) {
      s.e_min = u[D + 1];
      s.ie_min = t;
    }
#pragma unroll
    for (int p = 0; p < SC_COUNT; ++p)
      if (R.enabled[p]) fold(s, p, sc_value<D>(p, u, G), t, R.range[p]);
  }
  // ordered merge: 8 rounds of 32 threads; thread w of the warp holds
  // sub-run (round*32 + w); lane 0 merges them in order into the block total
  SanityPartial acc;
  if (threadIdx.x == 0) init_partial(acc);
  for (int round = 0; round < kSanThreads / 32; ++round) {
    __syncthreads();
    if ((int)threadIdx.x / 32 == round) sh[threadIdx.x % 32] = s;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 0; w < 32; ++w) merge_partial(acc, sh[w]);
  }
  if (threadIdx.x == 0) parts[blockIdx.x] = acc;
}

// Pass 2: one thread merges the block partials in block order.
__global__ void sanity_pass2(const SanityPartial* __restrict__ parts, int n, SanityPartial* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  SanityPartial acc;
  init_partial(acc);
  for (int b = 0; b < n; ++b) merge_partial(acc, parts[b]);
  *out = acc;
}

// Totals: double-double sums of rho > 0 and e_tot > 0 over all cells,
// ghosts included (the whole component blocks).
template <int D>
__global__ void __launch_bounds__(kSanThreads)
    totals_pass1(const double* __restrict__ U, long long field, DD* __restrict__ parts) {
  DD m = {0.0, 0.0}, e = {0.0, 0.0};
  const double* rho = U;
  const double* et = U + (long long)(D + 1) * field;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < field;
       t += (long long)gridDim.x * blockDim.x) {
    const double r = rho[t];
    const double x = et[t];
    if (r > 0.0) m = dd_add1(m, r);
    if (x > 0.0) e = dd_add1(e, x);
  }
  __shared__ DD sm[kSanThreads], se[kSanThreads];
  sm[threadIdx.x] = m;
  se[threadIdx.x] = e;
  __syncthreads();
  for (int w = kSanThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sm[threadIdx.x] = acc_add(sm[threadIdx.x], sm[threadIdx.x + w]);
      se[threadIdx.x] = acc_add(se[threadIdx.x], se[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    parts[2 * blockIdx.x] = sm[0];
    parts[2 * blockIdx.x + 1] = se[0];
  }
}

__global__ void totals_pass2(const DD* __restrict__ parts, int n, double* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  DD m = {0.0, 0.0}, e = {0.0, 0.0};
  for (int b = 0; b < n; ++b) {
    m = acc_add(m, parts[2 * b]);
    e = acc_add(e, parts[2 * b + 1]);
  }
  out[0] = m.hi + m.lo;
  out[1] = e.hi + e.lo;
}

}  // namespace

// Merge of the partial of a later run into an earlier one, as the
// sequential loop would continue: counts add; a later extreme replaces the
// earlier one only if strictly beyond it, and then the running extreme just
// before it is the better of the earlier extreme and the later run's own.
__host__ __device__ void merge_partial(SanityPartial& a, const SanityPartial& b) {
  for (int p = 0; p < SC_COUNT; ++p) {
    a.nbelow[p] += b.nbelow[p];
    a.nabove[p] += b.nabove[p];
    if (b.ibelow[p] >= 0 && b.vbelow[p] < a.vbelow[p]) {
      a.pbelow[p] = (b.pbelow[p] < a.vbelow[p]) ? b.pbelow[p] : a.vbelow[p];
      a.vbelow[p] = b.vbelow[p];
      a.ibelow[p] = b.ibelow[p];
    }
    if (b.iabove[p] >= 0 && b.vabove[p] > a.vabove[p]) {
      a.pabove[p] = (b.pabove[p] > a.vabove[p]) ? b.pabove[p] : a.vabove[p];
      a.vabove[p] = b.vabove[p];
      a.iabove[p] = b.iabove[p];
    }
  }
  for (int c = 0; c < 5; ++c) a.nan[c] |= b.nan[c];
  if (b.irho_min >= 0 && (a.irho_min < 0 || b.rho_min < a.rho_min)) {
    a.rho_min = b.rho_min;
    a.irho_min = b.irho_min;
  }
  if (b.ie_min >= 0 && (a.ie_min < 0 || b.e_min < a.e_min)) {
    a.e_min = b.e_min;
    a.ie_min = b.ie_min;
  }
}

cudaError_t launch_sanity(int ndim, const double* U, const Geom& g, const Gas<double>& G, const SanityRanges& R,
                          SanityPartial* parts, int nblocks, SanityPartial* out, cudaStream_t st) {
  const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
  const long long per_block = (total + nblocks - 1) / nblocks;
  switch (ndim) {
    case 1: sanity_pass1<1><<<nblocks, kSanThreads, 0, st>>>(U, g, G, R, parts, per_block); break;
    case 2: sanity_pass1<2><<<nblocks, kSanThreads, 0, st>>>(U, g, G, R, parts, per_block); break;
    case 3: sanity_pass1<3><<<nblocks, kSanThreads, 0, st>>>(U, g, G, R, parts, per_block); break;
    default: return cudaErrorInvalidValue;
  }
  sanity_pass2<<<1, 32, 0, st>>>(parts, nblocks, out);
  return cudaGetLastError();
}

cudaError_t launch_totals(int ndim, const double* U, long long field, void* parts, int nblocks, double* out,
                          cudaStream_t st) {
  DD* p = (DD*)parts;
  switch (ndim) {
    case 1: totals_pass1<1><<<nblocks, kSanThreads, 0, st>>>(U, field, p); break;
    case 2: totals_pass1<2><<<nblocks, kSanThreads, 0, st>>>(U, field, p); break;
    case 3: totals_pass1<3><<<nblocks, kSanThreads, 0, st>>>(U, field, p); break;
    default: return cudaErrorInvalidValue;
  }
  totals_pass2<<<1, 32, 0, st>>>(p, nblocks, out);
  return cudaGetLastError();
}

}  // namespace rgpu
