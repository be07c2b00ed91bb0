// sweeps.cu -- launchers of the mixed sweeps for every axis and tile shape of
// one dimensionality. Compiled three times (-DSWEEP_D=1, 2, 3) so the
// instantiations (axes x candidate shapes, single box and batched) build in
// parallel.
#include <cstring>

#include "sweep.cuh"

#ifndef SWEEP_D
#error "compile once per dimensionality with -DSWEEP_D=1, 2 or 3"
#endif

namespace rgpu {
namespace {

// The accumulation mode of an axis: the first axis starts the FP32 sum, the
// last one adds it to U^n in FP64.
template <int D, int A>
constexpr int mode_of() {
  return D == 1 ? ONLY : (A == 0 ? FIRST : (A == D - 1 ? LAST : MID));
}

// The tiles covering interior cells [lo, hi] of the outermost axis O = D-1
// (the whole box for lo = 1, hi = n[O]). A slab is swept as a box that
// starts at its first row: pointers shifted by lo - 1 rows, the extent along
// O cut to the rows from lo on (the rows before and after stay readable as
// the stencil's halo), queue entries shifted back. Where the tiles span O
// (O = A, or O = B across the pencils) the slab must start on a tile
// boundary and end on one or at the box's edge, so that every cell belongs
// to exactly one slab.
template <int D, int A, int S, int P>
cudaError_t launch_one(const MixedParams& M, const float* Uf, const double* U, const Geom& g, const Dx& dx,
                       const double* dtp, float* acc, double* Unew, const FallbackQueue& q, int lo, int hi,
                       cudaStream_t st, const SweepCarry& carry) {
  constexpr int B = Axes<D, A>::B, C = Axes<D, A>::C;
  constexpr int O = D - 1;
  const int NO = g.n[O];
  if (lo < 1 || hi > NO || lo > hi) return cudaErrorInvalidValue;
  if (O == A || O == B) {
    constexpr int T = (O == A) ? S : P;
    if ((lo - 1) % T != 0 || (hi != NO && (hi - lo + 1) % T != 0)) return cudaErrorInvalidValue;
  }
  Geom gs = g;
  FallbackQueue qs = q;
  const long long shift = (long long)(lo - 1) * g.s[O];
  gs.n[O] = NO - (lo - 1);
  qs.o_base = shift;
  qs.ga_base = (O == A) ? lo - 1 : 0;
  const int rows = hi - lo + 1;
  const int NA = (O == A) ? rows : g.n[A];
  const int NB = (B < D) ? ((O == B) ? rows : g.n[B]) : 1;
  const int NC = (C < D) ? ((O == C) ? rows : g.n[C]) : 1;
  const int tA = (NA + S - 1) / S, tB = (NB + P - 1) / P;
  if ((A == 0 ? tB : tA) > 65535 || NC > 65535) return cudaErrorInvalidConfiguration;
  const dim3 grid = (A == 0) ? dim3(tA, tB, NC) : dim3(tB, tA, NC);
  // the slab staged by one tensor copy of the whole box's mirror where
  // possible (its coordinates along O offset by the slab's first row)
  CUtensorMap map;
  memset(&map, 0, sizeof map);
  const int tma_on = encode_mirror_map(&map, Uf, g, D, A, S, P) ? 1 : 0;
  SweepCarry cs = carry;
  if (cs.Uf_next) cs.Uf_next += shift;
  sweep_kernel<D, A, S, P, mode_of<D, A>()><<<grid, TileCfg<S, P>::threads, 0, st>>>(
      M, Uf + shift, U + shift, gs, dx, dtp, acc + shift, Unew + shift, qs, map, tma_on, lo - 1, cs);
  return cudaGetLastError();
}

template <int D, int A, int S, int P>
cudaError_t launch_batch_one(const MixedParams& M, const BoxDesc* TB, const WorkItem* items, int n, int* head,
                             const FallbackQueue& q, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  constexpr int MODE = mode_of<D, A>();
  batch_sweep_kernel<D, A, S, P, MODE><<<152 * TileCfg<S, P>::template ctas<MODE>(), TileCfg<S, P>::threads, 0, st>>>(
      M, TB, items, n, head, q);
  return cudaGetLastError();
}

// shape index -> (S, P) as in sweep_shape()
template <int D, int A>
cudaError_t by_shape(int shape, const MixedParams& M, const float* Uf, const double* U, const Geom& g,
                     const Dx& dx, const double* dtp, float* acc, double* Unew,
                     const FallbackQueue& q, int lo, int hi, cudaStream_t st, const SweepCarry& carry) {
  if constexpr (D == 1) {
    switch (shape) {
      case 0: return launch_one<D, A, 64, 1>(M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
      case 1: return launch_one<D, A, 128, 1>(M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
      case 2: return launch_one<D, A, 256, 1>(M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
      case 3: return launch_one<D, A, 512, 1>(M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
    }
  } else {
    switch (shape) {
      case 0: return launch_one<D, A, 8, 32>(M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
      case 1: return launch_one<D, A, 16, 16>(M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
      case 2: return launch_one<D, A, 32, 8>(M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
      case 3: return launch_one<D, A, 64, 4>(M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
    }
  }
  return cudaErrorInvalidValue;
}

template <int D, int A>
cudaError_t batch_by_shape(int shape, const MixedParams& M, const BoxDesc* TB, const WorkItem* items, int n,
                           int* head, const FallbackQueue& q, cudaStream_t st) {
  if constexpr (D == 1) {
    switch (shape) {
      case 0: return launch_batch_one<D, A, 64, 1>(M, TB, items, n, head, q, st);
      case 1: return launch_batch_one<D, A, 128, 1>(M, TB, items, n, head, q, st);
      case 2: return launch_batch_one<D, A, 256, 1>(M, TB, items, n, head, q, st);
      case 3: return launch_batch_one<D, A, 512, 1>(M, TB, items, n, head, q, st);
    }
  } else {
    switch (shape) {
      case 0: return launch_batch_one<D, A, 8, 32>(M, TB, items, n, head, q, st);
      case 1: return launch_batch_one<D, A, 16, 16>(M, TB, items, n, head, q, st);
      case 2: return launch_batch_one<D, A, 32, 8>(M, TB, items, n, head, q, st);
      case 3: return launch_batch_one<D, A, 64, 4>(M, TB, items, n, head, q, st);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace

#define RGPU_CAT2(a, b) a##b
#define RGPU_CAT(a, b) RGPU_CAT2(a, b)

cudaError_t RGPU_CAT(launch_sweep_axis_, SWEEP_D)(int axis, int shape, const MixedParams& M, const float* Uf,
                                                 const double* U, const Geom& g, const Dx& dx,
                                                 const double* dtp, float* acc, double* Unew,
                                                 const FallbackQueue& q, int lo, int hi, cudaStream_t st,
                                                 const SweepCarry& carry) {
  constexpr int D = SWEEP_D;
  switch (axis) {
    case 0: return by_shape<D, 0>(shape, M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
    case 1:
      if constexpr (D > 1) return by_shape<D, 1>(shape, M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
      break;
    case 2:
      if constexpr (D > 2) return by_shape<D, 2>(shape, M, Uf, U, g, dx, dtp, acc, Unew, q, lo, hi, st, carry);
      break;
  }
  return cudaErrorInvalidValue;
}

cudaError_t RGPU_CAT(launch_batch_sweep_axis_, SWEEP_D)(int axis, int shape, const MixedParams& M,
                                                       const BoxDesc* TB, const WorkItem* items, int n,
                                                       int* head, const FallbackQueue& q, cudaStream_t st) {
  constexpr int D = SWEEP_D;
  switch (axis) {
    case 0: return batch_by_shape<D, 0>(shape, M, TB, items, n, head, q, st);
    case 1:
      if constexpr (D > 1) return batch_by_shape<D, 1>(shape, M, TB, items, n, head, q, st);
      break;
    case 2:
      if constexpr (D > 2) return batch_by_shape<D, 2>(shape, M, TB, items, n, head, q, st);
      break;
  }
  return cudaErrorInvalidValue;
}

#if SWEEP_D == 3
cudaError_t launch_sweep_xy_3(const MixedParams& M, const float* Uf, const Geom& g, const Dx& dx,
                              const double* dtp, float* acc, const FallbackQueue& q, cudaStream_t st) {
  constexpr int TX = 16, TY = 16;
  const unsigned gx = (unsigned)((g.n[0] + TX - 1) / TX), gy = (unsigned)((g.n[1] + TY - 1) / TY);
  if (gy > 65535 || g.n[2] > 65535) return cudaErrorNotSupported;
  CUtensorMap map;
  memset(&map, 0, sizeof map);
  if (!encode_xy_map(&map, Uf, g, TX, TY)) return cudaErrorNotSupported;
  sweep_xy_kernel<TX, TY><<<dim3(gx, gy, (unsigned)g.n[2]), XYCfg<TX, TY>::threads, 0, st>>>(M, g, dx, dtp, acc, q,
                                                                                             map, 0);
  return cudaGetLastError();
}
#endif

}  // namespace rgpu
