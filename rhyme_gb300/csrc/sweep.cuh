// sweep.cuh -- the fused per-axis sweep of the mixed-precision step.
//
// A CTA of TileCfg<S,P>::threads threads stages a slab of the FP32 mirror Uf (S
// cells along the sweep axis plus the 2-cell ghost/halo layer, for P
// pencils) in shared memory -- with one TMA tensor copy (cp.async.bulk.tensor
// over a 4-D map of the mirror, completion on an mbarrier) where the mirror's
// rows are 16-byte aligned, else with coalesced loads -- computes FP32 limited
// slopes and half-step face states for S+2 cells, solves the S+1 exact
// Riemann problems of the slab in FP32 (one thread per interface) and forms
// the flux difference of its S cells. The tile shape (S, P) is a template
// parameter; sweeps.cu instantiates every shape of the candidate set for
// the autotuner, once per dimensionality. sweep_xy_kernel (end of the file)
// runs the x and y sweeps of a 3-D box in one kernel.
#pragma once

#include <cuda.h>

#include "rgpu_internal.h"

namespace rgpu {
namespace {

// ---- TMA staging ------------------------------------------------------------
// Bounded waits: a copy that never completes sets a status bit instead of
// hanging the CTA.
constexpr long long kTmaWaitLimit = 1LL << 22;
constexpr int kStatusTmaTimeout = 8;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One elected thread: expect `bytes` on the barrier and start the copy of the
// box at coordinates (c0..c3) of `map` into dst (128-byte aligned).
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            unsigned long long* bar, unsigned bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];" ::"r"(smem_addr(dst)),
      "l"((unsigned long long)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
      : "memory");
}

// Wait for the barrier's phase `parity` to complete; false after the limit.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  for (long long i = 0; i < kTmaWaitLimit; ++i) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// TMA staging of one launch: the map of the whole box's mirror (unshifted)
// and the rows of the outermost axis that precede the launch's first row
// (a slab of the pipelined solve); on == 0: coalesced loads instead.
struct TmaStage {
  const CUtensorMap* map;
  int o_off;
  int on;
};

// Asynchronous 4- and 8-byte copies global -> shared (cp.async), completed
// per thread by cp_async_wait_all: the accumulator and the FP64 state a tile
// adds to at its end are fetched when the tile starts, behind the staging
// and the Riemann problems.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Sweep modes: the flux difference X of this axis becomes acc = X (FIRST),
// acc += X (MID), U^{n+1} = U + (acc + X) (LAST) or U^{n+1} = U + X (ONLY).
enum { FIRST = 0, MID = 1, LAST = 2, ONLY = 3 };

// Threads of a tile's CTA: one per interface of the tile ((S+1)·P, the
// costliest phase), rounded up to whole warps, so that no phase but the
// shared-memory staging needs a second, mostly idle round behind a barrier;
// at most 512. CTAs per SM (ctas<MODE>) such that a thread may keep up to
// 44 registers in the sweeps that only accumulate (5 CTAs of 288 threads;
// measured 4 % faster than 4 CTAs at 56) and 56 in the sweeps that form
// U^{n+1} (4 CTAs: at 44 registers these spill and lose 10 %).
template <int S, int P>
struct TileCfg {
  static constexpr int warps_ = ((S + 1) * P + 31) / 32;
  static constexpr int threads = warps_ * 32 > 512 ? 512 : warps_ * 32;
  template <int MODE>
  static constexpr int ctas() {
    constexpr int regs = (MODE == LAST || MODE == ONLY) ? 56 : 44;
    return 65536 / (threads * regs) > 0 ? 65536 / (threads * regs) : 1;
  }
};


// The flux difference dt/dx (F_left - F_right) of one component of one cell
// and its accumulation by mode, with explicit roundings (a fused
// multiply-add onto the running sum) so that every sweep variant performs
// exactly the same operations. a_prev / u_prev: the component's accumulator
// (MID, LAST) and U^n (LAST, ONLY), prefetched.
// Returns U^{n+1} of the component in the modes that form it (0 otherwise).
template <int MODE>
__device__ __forceinline__ double accumulate(float dtdx, float fl, float fr, float a_prev, double u_prev,
                                             long long oc, float* __restrict__ acc, double* __restrict__ Unew) {
  const float d = __fsub_rn(fl, fr);
  if (MODE == FIRST) {
    acc[oc] = __fmul_rn(dtdx, d);
  } else if (MODE == MID) {
    acc[oc] = __fmaf_rn(dtdx, d, a_prev);
  } else {
    const float tot = (MODE == LAST) ? __fmaf_rn(dtdx, d, a_prev) : __fmul_rn(dtdx, d);
    const double un = __dadd_rn(u_prev, widen_f32(tot));
    Unew[oc] = un;
    return un;
  }
  return 0.0;
}

// Block-wide maximum and or of (m, bad) of a CTA of NT threads (a multiple
// of 32), folded into *bits and *status by one thread.
template <int NT>
__device__ __forceinline__ void block_fold_max(float m, int bad, unsigned long long* bits, int* status) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float o = __shfl_down_sync(0xffffffffu, m, off);
    if (o > m) m = o;
    bad |= __shfl_down_sync(0xffffffffu, bad, off);
  }
  __shared__ float sm[NT / 32];
  __shared__ int sb[NT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sm[warp] = m;
    sb[warp] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < NT / 32; ++k) {
      if (sm[k] > m) m = sm[k];
      bad |= sb[k];
    }
    atomicMax(bits, (unsigned long long)__float_as_uint(m));
    if (bad) atomicOr(status, 1);
  }
}

// Slab geometry of axis A: pencils run along B (x unless A is x).
template <int D, int A>
struct Axes {
  static constexpr int B = (D == 1) ? 1 : (A == 0 ? 1 : 0);
  static constexpr int C = (D == 3) ? 3 - A - B : 2;
};

// The normal-first component order of axis A in the FP32 face states and
// interface fluxes: rho, the normal momentum, the other momenta in axis
// order, E. The FP32 face states and Riemann solve run on vectors in this
// order (face_states / rp_flux_f32 with axis 0), so every axis executes one
// copy of their code. nf_comp: the physical component at slot k;
// nf_slot: the slot of physical component c.
template <int D, int A>
__host__ __device__ constexpr int nf_comp(int k) {
  return (k == 0 || k == D + 1) ? k : (k == 1 ? 1 + A : 1 + ((k - 2) < A ? (k - 2) : (k - 1)));
}
template <int D, int A>
__host__ __device__ constexpr int nf_slot(int c) {
  return (c == 0 || c == D + 1) ? c : (c == 1 + A ? 1 : 2 + ((c - 1) < A ? (c - 1) : (c - 2)));
}

// Shared-memory slab; index (la along A, lb along the pencils) is stored
// with the x-fast index innermost so consecutive threads hit consecutive
// banks in both orientations. The state slab u is one component plane after
// another, each plane laid out as the tensor copy writes it: along x the
// S+4 staged cells of each of the P pencils; across x (sweeps along y or z,
// pencils along x) S+4 rows of P+4 cells, the pencils at columns 2..P+1 (a
// tensor copy must start at a 16-byte aligned x, 2 cells before the first
// interior pencil).
template <int D, int S, int P>
struct SweepSmem {
  alignas(128) float u[(D + 2) * (S + 4) * (P + 4)];  // FP32 state slab (ghost/halo layer included)
  float ul[D + 2][(S + 2) * P];  // face states (normal-first), left / right
  float ur[D + 2][(S + 2) * P];
  float f[D + 2][(S + 1) * P];   // interface fluxes (normal-first)
};

// One slab (tile tA along the sweep axis, tB across the pencils, plane cC)
// of a sweep. `box` tags queued FP64 interfaces (0 for a single box).
template <int D, int A, int S, int P, int MODE>
__device__ __forceinline__ void sweep_tile(const MixedParams& M, int limiter, float omega,
                                           const float* __restrict__ Uf, const double* __restrict__ U,
                                           const Geom& g, const Dx& dx, const double* __restrict__ dtp,
                                           float* __restrict__ acc, double* __restrict__ Unew,
                                           const FallbackQueue& q, int box,
                                           int tA, int tB, int cC, SweepSmem<D, S, P>& sh,
                                           const TmaStage& tma, unsigned long long* bar, unsigned& parity,
                                           const SweepCarry& carry = SweepCarry()) {
  constexpr int B = Axes<D, A>::B, C = Axes<D, A>::C;
  // component plane of the staged slab, and the index of (la, lb) in it
  constexpr int PLANE = (A == 0) ? (S + 4) * P : (S + 4) * (P + 4);
  auto ixu = [](int la, int lb) -> int { return (A == 0) ? lb * (S + 4) + la : la * (P + 4) + lb + 2; };
  float* su = sh.u;
  const int NA = g.n[A];
  const int NB = (B < D) ? g.n[B] : 1;
  const int a0 = tA * S + 1;  // first interior cell of the slab along A
  const int b0 = tB * P + 1;
  const long long F = g.field;
  // dt/dx and (0.5 dt)/dx once per CTA in FP32 (FP32(dt) times the FP32
  // inverse of dx: an FP64 division per CTA kept the FP64 pipe about 9 %
  // busy), formed by a thread outside the warp that issues and polls the
  // staging copy, while the copy is in flight
  __shared__ float s_dtdx[2];
  constexpr int kDtThread = TileCfg<S, P>::threads > 32 ? 32 : 0;
  // the accumulator (MID, LAST) and U^n (LAST, ONLY) of the tile's cells
  constexpr bool PRE_ACC = (MODE == MID || MODE == LAST);
  constexpr bool PRE_U = (MODE == LAST || MODE == ONLY);
  __shared__ float pre_acc[PRE_ACC ? (D + 2) * S * P : 1];
  __shared__ double pre_u[PRE_U ? (D + 2) * S * P : 1];
  __syncthreads();  // the previous tile of this CTA is done with the smem

  auto offset = [&](int ga, int gb) -> long long {
    int c3[3] = {1, 1, 1};
    c3[A] = ga;
    if (B < D) c3[B] = gb;
    if (C < D) c3[C] = cC;
    return g.at(D, c3[0], c3[1], c3[2]);
  };
  // thread item -> (la, lb), x-fast first; ix() the matching smem index
  auto split = [&](int it, int na, int& la, int& lb) {
    if (A == 0) {
      la = it % na;
      lb = it / na;
    } else {
      lb = it % P;
      la = it / P;
    }
  };
  auto ix = [&](int la, int lb, int na) -> int { return (A == 0) ? lb * na + la : la * P + lb; };

  // 0. start the copies of the accumulator and U^n of the tile's cells
  if (PRE_ACC || PRE_U) {
    for (int it = threadIdx.x; it < S * P; it += TileCfg<S, P>::threads) {
      int lu, lb;
      split(it, S, lu, lb);
      const int ga = a0 + lu, gb = b0 + lb;
      if (ga > NA || gb > NB) continue;
      const long long o = offset(ga, gb);
#pragma unroll
      for (int c = 0; c < D + 2; ++c) {
        if (PRE_ACC) cp_async4(&pre_acc[c * S * P + it], &acc[(long long)c * F + o]);
        if (PRE_U) cp_async8(&pre_u[c * S * P + it], &U[(long long)c * F + o]);
      }
    }
    cp_async_commit();
  }

  // 1. stage the FP32 slab: cells a0-2 .. a0+S+1 along A
  if (tma.on) {
    // one tensor copy of the whole slab (every component), zero-filled
    // beyond the array; coordinates are array indices (Fortran index + 1)
    if (threadIdx.x == 0) {
      int co[3] = {0, 0, 0};
      co[A] = a0 - 1;
      if (B < D) co[B] = (A == 0) ? b0 + 1 : b0 - 1;
      if (C < D) co[C] = cC + 1;
      co[D - 1] += tma.o_off;
      tma_load_4d(su, tma.map, co[0], co[1], co[2], 0, bar, (unsigned)((D + 2) * PLANE * sizeof(float)));
    }
    if (threadIdx.x == kDtThread) {
      const float dt = __double2float_rn(*dtp);
      s_dtdx[0] = dt * dx.inv_f[A];
      s_dtdx[1] = (0.5f * dt) * dx.inv_f[A];
    }
    // one warp polls the barrier; the others wait at the CTA barrier below,
    // off the issue slots the co-resident CTAs are computing with
    if (threadIdx.x < 32 && !mbar_wait(bar, parity)) {
      if (threadIdx.x == 0) atomicOr(q.status, kStatusTmaTimeout);
      mbar_wait(bar, parity);  // let a late copy land before the smem is reused
    }
    parity ^= 1u;
  } else {
    if (threadIdx.x == kDtThread) {
      const float dt = __double2float_rn(*dtp);
      s_dtdx[0] = dt * dx.inv_f[A];
      s_dtdx[1] = (0.5f * dt) * dx.inv_f[A];
    }
    for (int it = threadIdx.x; it < (S + 4) * P; it += TileCfg<S, P>::threads) {
      int la, lb;
      split(it, S + 4, la, lb);
      const int ga = a0 - 2 + la, gb = b0 + lb;
      const bool ok = ga <= NA + 2 && gb <= NB;
      const long long o = ok ? offset(ga, gb) : 0;
#pragma unroll
      for (int c = 0; c < D + 2; ++c) su[c * PLANE + ixu(la, lb)] = ok ? Uf[(long long)c * F + o] : 0.f;
    }
  }
  __syncthreads();
  const float dtdx = s_dtdx[0];
  const float hdtdx = s_dtdx[1];

  // 2. face states of cells a0-1 .. min(a0+S, NA+1)
  for (int it = threadIdx.x; it < (S + 2) * P; it += TileCfg<S, P>::threads) {
    int la, lb;
    split(it, S + 2, la, lb);
    if (a0 - 1 + la > NA + 1 || b0 + lb > NB) continue;
    // normal-first vectors (nf_comp); the face states stay in that order
    float um[D + 2], u0[D + 2], up[D + 2], l[D + 2], r[D + 2];
#pragma unroll
    for (int k = 0; k < D + 2; ++k) {
      const int c = nf_comp<D, A>(k);
      um[k] = su[c * PLANE + ixu(la, lb)];
      u0[k] = su[c * PLANE + ixu(la + 1, lb)];
      up[k] = su[c * PLANE + ixu(la + 2, lb)];
    }
    face_states<D, 0>(M.G, limiter, omega, um, u0, up, hdtdx, l, r);
#pragma unroll
    for (int k = 0; k < D + 2; ++k) {
      sh.ul[k][ix(la, lb, S + 2)] = l[k];
      sh.ur[k][ix(la, lb, S + 2)] = r[k];
    }
  }
  __syncthreads();

  // 3. FP32 Riemann problems at interfaces (a0-1+li | a0+li), li in [0, S]
  for (int it = threadIdx.x; it < (S + 1) * P; it += TileCfg<S, P>::threads) {
    int li, lb;
    split(it, S + 1, li, lb);
    if (a0 - 1 + li > NA || b0 + lb > NB) continue;
    float l[D + 2], r[D + 2], f[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      l[c] = sh.ur[c][ix(li, lb, S + 2)];
      r[c] = sh.ul[c][ix(li + 1, lb, S + 2)];
    }
    bool need64 = false;
    rp_flux_f32<D, 0>(M.G, M.rp, l, r, f, &need64);  // normal-first in and out
    if (!need64) {
#pragma unroll
      for (int c = 0; c < D + 2; ++c)
        if (!isfinite(f[c])) need64 = true;
    }
    if (need64) {
      // A non-finite cell in the interface's stencil (staged cells li .. li+3)
      // is non-finite in FP64 too, and the FP64 redo would give NaN: give it
      // here and queue nothing (a box the scheme has lost would otherwise
      // queue all its interfaces every step).
      bool finite = true;
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < D + 2; ++c) finite = finite && isfinite(su[c * PLANE + ixu(li + k, lb)]);
      // otherwise zero here; the FP64 correction is applied after the last
      // sweep. Each interface is queued once: by the tile whose left face it
      // is, or by the last tile for the box's right boundary.
      const int ga = a0 - 1 + li;
      if (finite && (li < S || ga == NA)) {
        const int slot = atomicAdd(q.n, 1);
        if (slot < q.cap) {
          FallbackEntry& e = q.e[slot];
          e.axis = A;
          e.ga = ga + q.ga_base;
          e.box = box;
          e.o = offset(ga, b0 + lb) + q.o_base;
        } else {
          atomicOr(q.status, 2);  // queue full: the interface keeps a zero flux
        }
      }
#pragma unroll
      for (int c = 0; c < D + 2; ++c) f[c] = finite ? 0.f : __int_as_float(0x7fffffff);
    }
#pragma unroll
    for (int c = 0; c < D + 2; ++c) sh.f[c][ix(li, lb, S + 1)] = f[c];
  }
  __syncthreads();

  // 4. flux differences of cells a0 .. a0+S-1 and the accumulation; with a
  // carry (last sweep), also the FP32 mirror of U^{n+1} and its signal speed
  constexpr bool FORMS = (MODE == LAST || MODE == ONLY);
  const bool carrying = FORMS && carry.bits != nullptr;
  float smax = 0.f;
  int sbad = 0;
  for (int it = threadIdx.x; it < S * P; it += TileCfg<S, P>::threads) {
    int lu, lb;
    split(it, S, lu, lb);
    const int ga = a0 + lu, gb = b0 + lb;
    if (ga > NA || gb > NB) continue;
    const long long o = offset(ga, gb);
    if (PRE_ACC || PRE_U) cp_async_wait_all();  // this thread's copies (same items as phase 0)
    double ud[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c)
      ud[c] = accumulate<MODE>(dtdx, sh.f[nf_slot<D, A>(c)][ix(lu, lb, S + 1)],
                               sh.f[nf_slot<D, A>(c)][ix(lu + 1, lb, S + 1)],
                               PRE_ACC ? pre_acc[c * S * P + it] : 0.f, PRE_U ? pre_u[c * S * P + it] : 0.0,
                               (long long)c * F + o, acc, Unew);
    if (carrying) {
      float un[D + 2];
#pragma unroll
      for (int c = 0; c < D + 2; ++c) {
        un[c] = narrow_mirror(ud[c]);
        carry.Uf_next[(long long)c * F + o] = un[c];
      }
      const float v = speed_f32<D>(M, un, sbad);
      if (v > smax) smax = v;
    }
  }
  if (carrying) block_fold_max<TileCfg<S, P>::threads>(smax, sbad, carry.bits, carry.status);
}

template <int D, int A, int S, int P, int MODE>
__global__ void __launch_bounds__(TileCfg<S, P>::threads, TileCfg<S, P>::template ctas<MODE>())
    sweep_kernel(MixedParams M, const float* __restrict__ Uf, const double* __restrict__ U, Geom g,
                 Dx dx, const double* __restrict__ dtp, float* __restrict__ acc,
                 double* __restrict__ Unew, FallbackQueue q, const __grid_constant__ CUtensorMap map,
                 int tma_on, int o_off, SweepCarry carry) {
  constexpr int C = Axes<D, A>::C;
  __shared__ SweepSmem<D, S, P> sh;
  __shared__ __align__(8) unsigned long long bar;
  if (tma_on && threadIdx.x == 0) mbar_init(&bar);  // ordered by the tile's first barrier
  unsigned parity = 0;
  const TmaStage tma{&map, o_off, tma_on};
  // tile origin: the fast grid axis runs along x
  const int tA = (A == 0) ? blockIdx.x : blockIdx.y;
  const int tB = (A == 0) ? blockIdx.y : blockIdx.x;
  const int cC = (C < D) ? (int)blockIdx.z + 1 : 1;
  sweep_tile<D, A, S, P, MODE>(M, M.limiter, M.omega, Uf, U, g, dx, dtp, acc, Unew, q, 0, tA, tB, cC,
                               sh, tma, &bar, parity, carry);
}

// The same sweep over the tiles of a batch of boxes, taken from a work queue
// (item.chunk = the tile's linear index tA + nA * (tB + nB * (cC - 1))).
template <int D, int A, int S, int P, int MODE>
__global__ void __launch_bounds__(TileCfg<S, P>::threads, TileCfg<S, P>::template ctas<MODE>())
    batch_sweep_kernel(MixedParams M, const BoxDesc* __restrict__ TB, const WorkItem* __restrict__ items,
                       int n, int* head, FallbackQueue q) {
  constexpr int B = Axes<D, A>::B;
  __shared__ SweepSmem<D, S, P> sh;
  __shared__ int s_item;
  unsigned parity = 0;
  const TmaStage tma{nullptr, 0, 0};
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= n) break;
    const WorkItem w = items[it];
    const BoxDesc& b = TB[w.box];
    const int nA = (b.g.n[A] + S - 1) / S;
    const int nB = ((B < D ? b.g.n[B] : 1) + P - 1) / P;
    const int tA = (int)(w.chunk % nA);
    const long long r = w.chunk / nA;
    const int tB = (int)(r % nB);
    const int cC = (int)(r / nB) + 1;
    sweep_tile<D, A, S, P, MODE>(M, b.limiter, b.omega_f, b.Uf, b.U, b.g, b.dx, b.ctl, b.acc, b.V,
                                 q, w.box, tA, tB, cC, sh, tma, nullptr, parity);
  }
}


// ---- the x and y sweeps of a 3-D box in one kernel ---------------------------
// A CTA takes a TX x TY tile of one z plane: one TMA copy stages the tile's
// FP32 state with a 2-cell halo along x and y ((TX+4) x (TY+4) cells, every
// component); then the face states of both axes (one loop over the x and y
// items), the interface fluxes of both axes (one loop), and the accumulator
// acc = dt/dx X + dt/dy Y, written once. The face states and fluxes run on
// normal-first vectors (nf_comp), so the loops hold one copy of the face
// state and Riemann code for both axes (two inlined copies cost the kernel
// as much in instruction-cache misses as the single staging saved). Every
// operation is the per-axis sweeps' (FIRST then MID, the same roundings):
// the result is bit-identical to sweep_kernel<3,0,...> then
// sweep_kernel<3,1,...>; it saves the second staging of the plane and the
// accumulator's round trip between the two sweeps.
template <int TX, int TY>
struct XYCfg {
  static constexpr int NXF = (TX + 2) * TY, NYF = TX * (TY + 2);  // face items
  static constexpr int NXI = (TX + 1) * TY, NYI = TX * (TY + 1);  // interfaces
  static constexpr int threads = ((NXF > NYF ? NXF : NYF) + 31) / 32 * 32;
  static constexpr int ctas = 65536 / (threads * 44) > 0 ? 65536 / (threads * 44) : 1;
};

template <int TX, int TY>
struct XYSmem {
  static constexpr int NF = XYCfg<TX, TY>::NXF > XYCfg<TX, TY>::NYF ? XYCfg<TX, TY>::NXF : XYCfg<TX, TY>::NYF;
  static constexpr int NI = XYCfg<TX, TY>::NXI > XYCfg<TX, TY>::NYI ? XYCfg<TX, TY>::NXI : XYCfg<TX, TY>::NYI;
  alignas(128) float u[5 * (TY + 4) * (TX + 4)];  // the staged plane (component after component)
  float fl[2][5][NF];                             // face states per axis (normal-first): left / right
  float fr[2][5][NF];
  float f[2][5][NI];                              // interface fluxes per axis (normal-first)
};

template <int TX, int TY>
__global__ void __launch_bounds__(XYCfg<TX, TY>::threads, XYCfg<TX, TY>::ctas)
    sweep_xy_kernel(MixedParams M, Geom g, Dx dx, const double* __restrict__ dtp, float* __restrict__ acc,
                    FallbackQueue q, const __grid_constant__ CUtensorMap map, int o_off) {
  using Cfg = XYCfg<TX, TY>;
  constexpr int NT = Cfg::threads;
  constexpr int PW = TX + 4;               // plane row
  constexpr int PL = (TX + 4) * (TY + 4);  // plane of one component
  __shared__ XYSmem<TX, TY> sh;
  __shared__ __align__(8) unsigned long long bar;
  __shared__ float s_dt[4];  // dt/dx, (0.5 dt)/dx, dt/dy, (0.5 dt)/dy
  const int NX = g.n[0], NY = g.n[1];
  const int x0 = blockIdx.x * TX + 1, y0 = blockIdx.y * TY + 1;
  const int cz = (int)blockIdx.z + 1;
  const long long F = g.field;
  float* su = sh.u;
  if (threadIdx.x == 0) mbar_init(&bar);
  __syncthreads();
  // 1. stage the plane: cells x0-2 .. x0+TX+1, y0-2 .. y0+TY+1 of plane cz
  if (threadIdx.x == 0)
    tma_load_4d(su, &map, x0 - 1, y0 - 1, cz + 1 + o_off, 0, &bar, (unsigned)(5 * PL * sizeof(float)));
  if (threadIdx.x == 32) {
    const float dt = __double2float_rn(*dtp);
    s_dt[0] = dt * dx.inv_f[0];
    s_dt[1] = (0.5f * dt) * dx.inv_f[0];
    s_dt[2] = dt * dx.inv_f[1];
    s_dt[3] = (0.5f * dt) * dx.inv_f[1];
  }
  if (threadIdx.x < 32 && !mbar_wait(&bar, 0)) {
    if (threadIdx.x == 0) atomicOr(q.status, kStatusTmaTimeout);
    mbar_wait(&bar, 0);
  }
  __syncthreads();

  // 2. face states: x of cells x0-1 .. x0+TX (rows y0 ..), then y of cells
  // y0-1 .. y0+TY (columns x0 ..); one loop, the axis only in the indices
  for (int it = threadIdx.x; it < Cfg::NXF + Cfg::NYF; it += NT) {
    const int ax = it >= Cfg::NXF;
    const int t = ax ? it - Cfg::NXF : it;
    int base, stride, slot;
    if (!ax) {
      const int la = t % (TX + 2), lb = t / (TX + 2);
      if (x0 - 1 + la > NX + 1 || y0 + lb > NY) continue;
      base = (lb + 2) * PW + la;
      stride = 1;
      slot = lb * (TX + 2) + la;
    } else {
      const int lb = t % TX, la = t / TX;
      if (y0 - 1 + la > NY + 1 || x0 + lb > NX) continue;
      base = la * PW + lb + 2;
      stride = PW;
      slot = la * TX + lb;
    }
    const int c1 = ax ? 2 : 1, c2 = ax ? 1 : 2;  // normal-first: the normal momentum first
    const int comp[5] = {0, c1, c2, 3, 4};
    float um[5], u0[5], up[5], l[5], r[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int b = comp[k] * PL + base;
      um[k] = su[b];
      u0[k] = su[b + stride];
      up[k] = su[b + 2 * stride];
    }
    face_states<3, 0>(M.G, M.limiter, M.omega, um, u0, up, s_dt[ax ? 3 : 1], l, r);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      sh.fl[ax][k][slot] = l[k];
      sh.fr[ax][k][slot] = r[k];
    }
  }
  __syncthreads();
  // 3. interfaces: x0-1+li | x0+li (rows y0 ..), then y0-1+lj | y0+lj
  for (int it = threadIdx.x; it < Cfg::NXI + Cfg::NYI; it += NT) {
    const int ax = it >= Cfg::NXI;
    const int t = ax ? it - Cfg::NXI : it;
    int li, lb, N, T, ga, px, py, sl, sr, sf;
    if (!ax) {
      li = t % (TX + 1);
      lb = t / (TX + 1);
      if (x0 - 1 + li > NX || y0 + lb > NY) continue;
      N = NX, T = TX, ga = x0 - 1 + li, px = li, py = lb + 2;
      sl = lb * (TX + 2) + li, sr = sl + 1, sf = lb * (TX + 1) + li;
    } else {
      lb = t % TX;
      li = t / TX;
      if (y0 - 1 + li > NY || x0 + lb > NX) continue;
      N = NY, T = TY, ga = y0 - 1 + li, px = lb + 2, py = li;
      sl = li * TX + lb, sr = sl + TX, sf = li * TX + lb;
    }
    float l[5], r[5], f[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      l[k] = sh.fr[ax][k][sl];
      r[k] = sh.fl[ax][k][sr];
    }
    bool need64 = false;
    rp_flux_f32<3, 0>(M.G, M.rp, l, r, f, &need64);
    if (!need64) {
#pragma unroll
      for (int k = 0; k < 5; ++k)
        if (!isfinite(f[k])) need64 = true;
    }
    if (need64) {
      // as the per-axis sweeps: queued once (by the tile whose left face it
      // is, or by the last tile at the box's right boundary) unless a cell
      // of its stencil is non-finite (then the flux is NaN)
      const int step = ax ? PW : 1;
      bool finite = true;
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 5; ++c) finite = finite && isfinite(su[c * PL + py * PW + px + k * step]);
      if (finite && (li < T || ga == N)) {
        const int slot = atomicAdd(q.n, 1);
        if (slot < q.cap) {
          FallbackEntry& e = q.e[slot];
          e.axis = ax;
          e.ga = ga;
          e.box = 0;
          e.o = (ax ? g.at(3, x0 + lb, ga, cz) : g.at(3, ga, y0 + lb, cz)) + q.o_base;
        } else {
          atomicOr(q.status, 2);
        }
      }
#pragma unroll
      for (int k = 0; k < 5; ++k) f[k] = finite ? 0.f : __int_as_float(0x7fffffff);
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) sh.f[ax][k][sf] = f[k];
  }
  __syncthreads();
  // 4. acc = dt/dx X + dt/dy Y (the per-axis FIRST and MID roundings); the
  // y fluxes hold m_y in slot 1 and m_x in slot 2
  for (int it = threadIdx.x; it < TX * TY; it += NT) {
    const int lu = it % TX, lv = it / TX;
    if (x0 + lu > NX || y0 + lv > NY) continue;
    const long long o = g.at(3, x0 + lu, y0 + lv, cz);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      const int ky = (c == 1) ? 2 : (c == 2 ? 1 : c);
      const float ax_ = __fmul_rn(s_dt[0], __fsub_rn(sh.f[0][c][lv * (TX + 1) + lu], sh.f[0][c][lv * (TX + 1) + lu + 1]));
      acc[(long long)c * F + o] =
          __fmaf_rn(s_dt[2], __fsub_rn(sh.f[1][ky][lv * TX + lu], sh.f[1][ky][(lv + 1) * TX + lu]), ax_);
    }
  }
}

}  // namespace
}  // namespace rgpu
