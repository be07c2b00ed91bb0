// kernels_mixed.cu -- mixed-precision MUSCL-Hancock step.
//
// The conserved state stays FP64 in HBM (U) and is mirrored once per step as
// FP32 (Uf). Each axis is one fused sweep kernel: a CTA stages a slab of
// Uf (S cells along the sweep axis plus the 2-cell ghost/halo layer, for P
// pencils) in shared memory with coalesced loads, computes FP32 limited
// slopes and half-step face states for S+2 cells, solves the S+1 exact
// Riemann problems of the slab in FP32 and forms the flux difference of its
// S cells. The flux differences of the axes are summed in FP32 in the
// reference's association ((X + Y) + Z), and the last sweep adds the sum to
// U in FP64 and writes U^{n+1} and its FP32 mirror: one FP64 add per
// conserved component and cell, since on GB300 even FP64 adds are scarce.
//
// Interfaces that near vacuum, or whose FP32 Newton iteration misses the
// tolerance on its first guess, get a zero flux in the sweep and are appended
// (once, by the tile that owns them) to a device queue with their FP32 face
// states. After the last sweep one kernel solves the queued interfaces with
// the FP64 Riemann solver (same device code, double) and applies
// -+ dt/dx * F to the two adjacent interior cells of U^{n+1}; a second one
// refreshes their FP32 mirror. Keeping the FP64 code out of the sweeps keeps
// them at ~64 registers (it tripled their register count inline).
//
// The CFL maximum of the mixed path is taken in FP32 over Uf; dt itself is
// formed in FP64.
#include "rgpu_internal.h"

namespace rgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 152 * 32;

inline int grid_for(long long total, int block) {
  long long b = (total + block - 1) / block;
  if (b < 1) b = 1;
  if (b > kMaxBlocks) b = kMaxBlocks;
  return (int)b;
}

// U (FP64) -> Uf (FP32) over whole component blocks (ghosts included).
__global__ void __launch_bounds__(kThreads) to_f32_kernel(const double* __restrict__ U,
                                                          float* __restrict__ Uf, long long n) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    Uf[t] = (float)U[t];
}

// |v| + cs of interior cell t of Uf in FP32; bad marks non-positive density
// or a non-finite value.
template <int D>
__device__ __forceinline__ float signal_speed_f32(const MixedParams& M, const float* __restrict__ Uf,
                                                  const Geom& g, long long t, int& bad) {
  const long long n0 = g.n[0], n1 = g.n[1];
  const int i = (int)(t % n0) + 1;
  const long long q = t / n0;
  const int j = (int)(q % n1) + 1;
  const int k = (int)(q / n1) + 1;
  const long long o = g.at(D, i, j, k);
  float u[D + 2];
#pragma unroll
  for (int c = 0; c < D + 2; ++c) u[c] = Uf[(long long)c * g.field + o];
  float ss = 0.f;
#pragma unroll
  for (int a = 0; a < D; ++a) ss = ss + u[1 + a] * u[1 + a];
  const float v = sqrtf(ss) / u[0] + sound_speed<D>(M.G, u);
  if (!(u[0] > 0.f) || !isfinite(v)) bad = 1;
  return v;
}

// FP32 signal-speed maximum over the interior of Uf; the last block forms
// dt = courant * min(dx) / max in FP64 and resets the accumulators.
template <int D>
__global__ void __launch_bounds__(kThreads)
    cfl_f32_kernel(MixedParams M, const float* __restrict__ Uf, Geom g, double courant, double mdx,
                   StepScratch s) {
  const long long total = (long long)g.n[0] * g.n[1] * (long long)g.n[2];
  float m = 0.f;
  int bad = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const float v = signal_speed_f32<D>(M, Uf, g, t, bad);
    if (v > m) m = v;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float o = __shfl_down_sync(0xffffffffu, m, off);
    if (o > m) m = o;
    bad |= __shfl_down_sync(0xffffffffu, bad, off);
  }
  __shared__ float sm[kThreads / 32];
  __shared__ int sb[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sm[warp] = m;
    sb[warp] = bad;
  }
  __syncthreads();
  if (warp == 0) {
    m = (lane < kThreads / 32) ? sm[lane] : 0.f;
    bad = (lane < kThreads / 32) ? sb[lane] : 0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float o = __shfl_down_sync(0xffffffffu, m, off);
      if (o > m) m = o;
      bad |= __shfl_down_sync(0xffffffffu, bad, off);
    }
    if (lane == 0) {
      // non-negative floats order like their bit patterns
      atomicMax(s.max_bits, (unsigned long long)__float_as_uint(m));
      if (bad) atomicOr(s.status, 1);
      __threadfence();
      const unsigned int prev = atomicAdd(s.counter, 1u);
      if (prev == gridDim.x - 1) {
        __threadfence();
        const float mu = __uint_as_float((unsigned int)atomicAdd(s.max_bits, 0ull));
        const double dt = courant * mdx / (double)mu;
        *s.dt = dt;
        if (s.dt_trace) {
          const int pos = *s.trace_pos;
          if (pos >= 0 && pos < s.trace_cap) s.dt_trace[pos] = dt;
          *s.trace_pos = pos + 1;
        }
        atomicExch(s.max_bits, 0ull);
        atomicExch(s.counter, 0u);
      }
    }
  }
}

// Sweep modes: the flux difference X of this axis becomes acc = X (FIRST),
// acc += X (MID), U^{n+1} = U + (acc + X) (LAST) or U^{n+1} = U + X (ONLY).
enum { FIRST = 0, MID = 1, LAST = 2, ONLY = 3 };

// Slab geometry of axis A: pencils run along B (x unless A is x).
template <int D, int A>
struct Axes {
  static constexpr int B = (D == 1) ? 1 : (A == 0 ? 1 : 0);
  static constexpr int C = (D == 3) ? 3 - A - B : 2;
};

// Shared-memory slab; index (la along A, lb along the pencils) is stored
// with the x-fast index innermost so consecutive threads hit consecutive
// banks in both orientations.
template <int D, int S, int P>
struct SweepSmem {
  float u[D + 2][(S + 4) * P];   // FP32 state slab (ghost/halo layer included)
  float ul[D + 2][(S + 2) * P];  // face states, left / right
  float ur[D + 2][(S + 2) * P];
  float f[D + 2][(S + 1) * P];   // interface fluxes
};

// One slab (tile tA along the sweep axis, tB across the pencils, plane cC)
// of a sweep. `box` tags queued FP64 interfaces (0 for a single box).
template <int D, int A, int S, int P, int MODE>
__device__ __forceinline__ void sweep_tile(const MixedParams& M, int limiter, float omega,
                                           const float* __restrict__ Uf, const double* __restrict__ U,
                                           const Geom& g, const Dx& dx, const double* __restrict__ dtp,
                                           float* __restrict__ acc, double* __restrict__ Unew,
                                           float* __restrict__ Ufnew, const FallbackQueue& q, int box,
                                           int tA, int tB, int cC, SweepSmem<D, S, P>& sh) {
  constexpr int B = Axes<D, A>::B, C = Axes<D, A>::C;
  const int NA = g.n[A];
  const int NB = (B < D) ? g.n[B] : 1;
  const int a0 = tA * S + 1;  // first interior cell of the slab along A
  const int b0 = tB * P + 1;
  const long long F = g.field;
  // dt/dx and (0.5 dt)/dx once per CTA (FP64 divisions are scarce on GB300)
  __shared__ float s_dtdx[2];
  __syncthreads();  // the previous tile of this CTA is done with the smem
  if (threadIdx.x == 0) {
    const double dt = *dtp;
    s_dtdx[0] = (float)(dt / dx.v[A]);
    s_dtdx[1] = (float)(0.5 * dt / dx.v[A]);
  }

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

  // 1. stage the FP32 slab: cells a0-2 .. a0+S+1 along A
  for (int it = threadIdx.x; it < (S + 4) * P; it += kThreads) {
    int la, lb;
    split(it, S + 4, la, lb);
    const int ga = a0 - 2 + la, gb = b0 + lb;
    const bool ok = ga <= NA + 2 && gb <= NB;
    const long long o = ok ? offset(ga, gb) : 0;
#pragma unroll
    for (int c = 0; c < D + 2; ++c) sh.u[c][ix(la, lb, S + 4)] = ok ? Uf[(long long)c * F + o] : 0.f;
  }
  __syncthreads();
  const float dtdx = s_dtdx[0];
  const float hdtdx = s_dtdx[1];

  // 2. face states of cells a0-1 .. min(a0+S, NA+1)
  for (int it = threadIdx.x; it < (S + 2) * P; it += kThreads) {
    int la, lb;
    split(it, S + 2, la, lb);
    if (a0 - 1 + la > NA + 1 || b0 + lb > NB) continue;
    float um[D + 2], u0[D + 2], up[D + 2], l[D + 2], r[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      um[c] = sh.u[c][ix(la, lb, S + 4)];
      u0[c] = sh.u[c][ix(la + 1, lb, S + 4)];
      up[c] = sh.u[c][ix(la + 2, lb, S + 4)];
    }
    face_states<D, A>(M.G, limiter, omega, um, u0, up, hdtdx, l, r);
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      sh.ul[c][ix(la, lb, S + 2)] = l[c];
      sh.ur[c][ix(la, lb, S + 2)] = r[c];
    }
  }
  __syncthreads();

  // 3. FP32 Riemann problems at interfaces (a0-1+li | a0+li), li in [0, S]
  for (int it = threadIdx.x; it < (S + 1) * P; it += kThreads) {
    int li, lb;
    split(it, S + 1, li, lb);
    if (a0 - 1 + li > NA || b0 + lb > NB) continue;
    float l[D + 2], r[D + 2], u[D + 2], f[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      l[c] = sh.ur[c][ix(li, lb, S + 2)];
      r[c] = sh.ul[c][ix(li + 1, lb, S + 2)];
    }
    bool need64 = false;
    rp_solve<D, A, float, true>(M.G, M.rp, l, r, 0.f, u, &need64);
    if (!need64) {
      flux<D, A>(M.G, u, f);
#pragma unroll
      for (int c = 0; c < D + 2; ++c)
        if (!isfinite(f[c])) need64 = true;
    }
    if (need64) {
      // zero here; the FP64 correction is applied after the last sweep.
      // Each interface is queued once: by the tile whose left face it is,
      // or by the last tile for the box's right boundary.
      const int ga = a0 - 1 + li;
      if (li < S || ga == NA) {
        const int slot = atomicAdd(q.n, 1);
        if (slot < q.cap) {
          FallbackEntry& e = q.e[slot];
          e.axis = A;
          e.ga = ga;
          e.box = box;
          e.o = offset(ga, b0 + lb);
#pragma unroll
          for (int c = 0; c < D + 2; ++c) {
            e.l[c] = l[c];
            e.r[c] = r[c];
          }
        } else {
          atomicOr(q.status, 2);  // queue full: the interface keeps a zero flux
        }
      }
#pragma unroll
      for (int c = 0; c < D + 2; ++c) f[c] = 0.f;
    }
#pragma unroll
    for (int c = 0; c < D + 2; ++c) sh.f[c][ix(li, lb, S + 1)] = f[c];
  }
  __syncthreads();

  // 4. flux differences of cells a0 .. a0+S-1 and the accumulation
  for (int it = threadIdx.x; it < S * P; it += kThreads) {
    int lu, lb;
    split(it, S, lu, lb);
    const int ga = a0 + lu, gb = b0 + lb;
    if (ga > NA || gb > NB) continue;
    const long long o = offset(ga, gb);
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      const float x = dtdx * (sh.f[c][ix(lu, lb, S + 1)] - sh.f[c][ix(lu + 1, lb, S + 1)]);
      const long long oc = (long long)c * F + o;
      if (MODE == FIRST) {
        acc[oc] = x;
      } else if (MODE == MID) {
        acc[oc] = acc[oc] + x;
      } else {
        const float tot = (MODE == LAST) ? acc[oc] + x : x;
        const double un = U[oc] + (double)tot;
        Unew[oc] = un;
        Ufnew[oc] = (float)un;
      }
    }
  }
}

template <int D, int A, int S, int P, int MODE>
__global__ void __launch_bounds__(kThreads, 4)
    sweep_kernel(MixedParams M, const float* __restrict__ Uf, const double* __restrict__ U, Geom g,
                 Dx dx, const double* __restrict__ dtp, float* __restrict__ acc,
                 double* __restrict__ Unew, float* __restrict__ Ufnew, FallbackQueue q) {
  constexpr int C = Axes<D, A>::C;
  __shared__ SweepSmem<D, S, P> sh;
  // tile origin: the fast grid axis runs along x
  const int tA = (A == 0) ? blockIdx.x : blockIdx.y;
  const int tB = (A == 0) ? blockIdx.y : blockIdx.x;
  const int cC = (C < D) ? (int)blockIdx.z + 1 : 1;
  sweep_tile<D, A, S, P, MODE>(M, M.limiter, M.omega, Uf, U, g, dx, dtp, acc, Unew, Ufnew, q, 0, tA, tB, cC,
                               sh);
}

// The same sweep over the tiles of a batch of boxes, taken from a work queue
// (item.chunk = the tile's linear index tA + nA * (tB + nB * (cC - 1))).
template <int D, int A, int S, int P, int MODE>
__global__ void __launch_bounds__(kThreads, 4)
    batch_sweep_kernel(MixedParams M, const BoxDesc* __restrict__ TB, const WorkItem* __restrict__ items,
                       int n, int* head, FallbackQueue q) {
  constexpr int B = Axes<D, A>::B;
  __shared__ SweepSmem<D, S, P> sh;
  __shared__ int s_item;
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
    sweep_tile<D, A, S, P, MODE>(M, b.limiter, b.omega_f, b.Uf, b.U, b.g, b.dx, b.ctl, b.acc, b.V, b.Vf,
                                 q, w.box, tA, tB, cC, sh);
  }
}

template <int D, int A, int S, int P, int MODE>
cudaError_t launch_sweep(const MixedParams& M, const float* Uf, const double* U, const Geom& g,
                         const Dx& dx, const double* dtp, float* acc, double* Unew, float* Ufnew,
                         const FallbackQueue& q, cudaStream_t st) {
  constexpr int B = Axes<D, A>::B, C = Axes<D, A>::C;
  const int NA = g.n[A];
  const int NB = (B < D) ? g.n[B] : 1;
  const int NC = (C < D) ? g.n[C] : 1;
  dim3 grid;
  if (A == 0) {
    grid = dim3((NA + S - 1) / S, (NB + P - 1) / P, NC);
  } else {
    grid = dim3((NB + P - 1) / P, (NA + S - 1) / S, NC);
  }
  sweep_kernel<D, A, S, P, MODE><<<grid, kThreads, 0, st>>>(M, Uf, U, g, dx, dtp, acc, Unew, Ufnew, q);
  return cudaGetLastError();
}

// FP64 Riemann problems of the queued interfaces; -+ dt/dx * F applied to
// the adjacent interior cells of U^{n+1} (atomically: a cell can border two
// queued interfaces).
template <int D>
__global__ void __launch_bounds__(128)
    fallback_fix_kernel(MixedParams M, FallbackQueue q, Geom g, Dx dx, const double* __restrict__ dtp,
                        double* __restrict__ Unew) {
  const int n = min(*q.n, q.cap);
  if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0) atomicAdd(q.total, n);
  const double dt = *dtp;
  const long long F = g.field;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const FallbackEntry e = q.e[i];
    double l[D + 2], r[D + 2], f[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      l[c] = (double)e.l[c];
      r[c] = (double)e.r[c];
    }
    if (e.axis == 0) interface_flux<D, 0>(M.G64, M.rp64, l, r, f);
    if constexpr (D > 1) {
      if (e.axis == 1) interface_flux<D, 1>(M.G64, M.rp64, l, r, f);
    }
    if constexpr (D > 2) {
      if (e.axis == 2) interface_flux<D, 2>(M.G64, M.rp64, l, r, f);
    }
    const double dtdx = dt / dx.v[e.axis];
    const long long sa = g.s[e.axis];
    const int NA = g.n[e.axis];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      const double corr = dtdx * f[c];
      if (e.ga >= 1) atomicAdd(&Unew[(long long)c * F + e.o], -corr);
      if (e.ga + 1 <= NA) atomicAdd(&Unew[(long long)c * F + e.o + sa], corr);
    }
  }
}

// FP32 mirror of the cells the fix-up touched.
template <int D>
__global__ void __launch_bounds__(256)
    fallback_refresh_kernel(FallbackQueue q, Geom g, const double* __restrict__ Unew,
                            float* __restrict__ Ufnew) {
  const int n = min(*q.n, q.cap);
  const long long F = g.field;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const FallbackEntry e = q.e[i];
    const long long sa = g.s[e.axis];
    const int NA = g.n[e.axis];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      const long long oc = (long long)c * F + e.o;
      if (e.ga >= 1) Ufnew[oc] = (float)Unew[oc];
      if (e.ga + 1 <= NA) Ufnew[oc + sa] = (float)Unew[oc + sa];
    }
  }
}

template <int D>
cudaError_t launch_fallback(const MixedParams& M, const FallbackQueue& q, const Geom& g, const Dx& dx,
                            const double* dtp, double* Unew, float* Ufnew, cudaStream_t st) {
  fallback_fix_kernel<D><<<152, 128, 0, st>>>(M, q, g, dx, dtp, Unew);
  fallback_refresh_kernel<D><<<152, 256, 0, st>>>(q, g, Unew, Ufnew);
  return cudaGetLastError();
}

// Batched FP32 CFL over work items (chunks of 256 cells of a box): per-box
// maximum through atomics, the last item of a box forms its dt in FP64.
template <int D>
__global__ void __launch_bounds__(256)
    batch_cfl_f32_kernel(MixedParams M, double courant, const BoxDesc* __restrict__ TB,
                         const WorkItem* __restrict__ items, int n, int* head) {
  __shared__ float sm[8];
  __shared__ int sb[8];
  __shared__ int s_item;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= n) break;
    const WorkItem w = items[it];
    const BoxDesc& b = TB[w.box];
    const long long total = (long long)b.g.n[0] * b.g.n[1] * b.g.n[2];
    const long long t = w.chunk * kBatchChunk + threadIdx.x;
    float m = 0.f;
    int bad = 0;
    if (t < total) {
      const float v = signal_speed_f32<D>(M, b.Uf, b.g, t, bad);
      if (v > m) m = v;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float o = __shfl_down_sync(0xffffffffu, m, off);
      if (o > m) m = o;
      bad |= __shfl_down_sync(0xffffffffu, bad, off);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
      sm[warp] = m;
      sb[warp] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 1; k < 8; ++k) {
        if (sm[k] > m) m = sm[k];
        bad |= sb[k];
      }
      unsigned long long* max_bits = (unsigned long long*)(b.ctl + 1);
      unsigned int* counter = (unsigned int*)(b.ctl + 2);
      int* status = (int*)(b.ctl + 2) + 1;
      atomicMax(max_bits, (unsigned long long)__float_as_uint(m));
      if (bad) atomicOr(status, 1);
      __threadfence();
      if (atomicAdd(counter, 1u) == (unsigned int)(b.cfl_items - 1)) {
        __threadfence();
        const float mu = __uint_as_float((unsigned int)atomicAdd(max_bits, 0ull));
        b.ctl[0] = courant * b.dx.min / (double)mu;
        atomicExch(max_bits, 0ull);
        atomicExch(counter, 0u);
      }
    }
  }
}

// Batched FP64 fix-up: as fallback_fix_kernel, with the box of each entry.
template <int D>
__global__ void __launch_bounds__(128)
    batch_fallback_fix_kernel(MixedParams M, FallbackQueue q, const BoxDesc* __restrict__ TB) {
  const int n = min(*q.n, q.cap);
  if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0) atomicAdd(q.total, n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const FallbackEntry e = q.e[i];
    const BoxDesc& b = TB[e.box];
    double l[D + 2], r[D + 2], f[D + 2];
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      l[c] = (double)e.l[c];
      r[c] = (double)e.r[c];
    }
    if (e.axis == 0) interface_flux<D, 0>(M.G64, M.rp64, l, r, f);
    if constexpr (D > 1) {
      if (e.axis == 1) interface_flux<D, 1>(M.G64, M.rp64, l, r, f);
    }
    if constexpr (D > 2) {
      if (e.axis == 2) interface_flux<D, 2>(M.G64, M.rp64, l, r, f);
    }
    const double dtdx = b.ctl[0] / b.dx.v[e.axis];
    const long long sa = b.g.s[e.axis];
    const int NA = b.g.n[e.axis];
    const long long F = b.g.field;
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      const double corr = dtdx * f[c];
      if (e.ga >= 1) atomicAdd(&b.V[(long long)c * F + e.o], -corr);
      if (e.ga + 1 <= NA) atomicAdd(&b.V[(long long)c * F + e.o + sa], corr);
    }
  }
}

template <int D>
__global__ void __launch_bounds__(256)
    batch_fallback_refresh_kernel(FallbackQueue q, const BoxDesc* __restrict__ TB) {
  const int n = min(*q.n, q.cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const FallbackEntry e = q.e[i];
    const BoxDesc& b = TB[e.box];
    const long long sa = b.g.s[e.axis];
    const int NA = b.g.n[e.axis];
    const long long F = b.g.field;
#pragma unroll
    for (int c = 0; c < D + 2; ++c) {
      const long long oc = (long long)c * F + e.o;
      if (e.ga >= 1) b.Vf[oc] = (float)b.V[oc];
      if (e.ga + 1 <= NA) b.Vf[oc + sa] = (float)b.V[oc + sa];
    }
  }
}

template <int D, int A, int S, int P, int MODE>
cudaError_t launch_batch_sweep(const MixedParams& M, const BoxDesc* TB, const BatchLists& L,
                               const FallbackQueue& q, int slot, cudaStream_t st) {
  if (L.n_sweep[A] == 0) return cudaSuccess;
  batch_sweep_kernel<D, A, S, P, MODE><<<152 * 4, kThreads, 0, st>>>(M, TB, L.sweep[A], L.n_sweep[A],
                                                                     L.heads + slot, q);
  return cudaGetLastError();
}

template <int D>
cudaError_t launch_batch_fallback(const MixedParams& M, const BoxDesc* TB, const FallbackQueue& q,
                                  cudaStream_t st) {
  batch_fallback_fix_kernel<D><<<152, 128, 0, st>>>(M, q, TB);
  batch_fallback_refresh_kernel<D><<<152, 256, 0, st>>>(q, TB);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_to_f32(const double* U, float* Uf, long long n, cudaStream_t st) {
  to_f32_kernel<<<grid_for(n, kThreads), kThreads, 0, st>>>(U, Uf, n);
  return cudaGetLastError();
}

cudaError_t launch_cfl_mixed(const MixedParams& M, const float* Uf, const Geom& g, double courant,
                             const Dx& dx, const StepScratch& s, cudaStream_t st) {
  const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
  int grid = grid_for(total, kThreads);
  if (grid > 152 * 4) grid = 152 * 4;
  switch (M.ndim) {
    case 1: cfl_f32_kernel<1><<<grid, kThreads, 0, st>>>(M, Uf, g, courant, dx.min, s); break;
    case 2: cfl_f32_kernel<2><<<grid, kThreads, 0, st>>>(M, Uf, g, courant, dx.min, s); break;
    case 3: cfl_f32_kernel<3><<<grid, kThreads, 0, st>>>(M, Uf, g, courant, dx.min, s); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_mh_solve_mixed(const MixedParams& M, const double* U, const float* Uf,
                                  double* Unew, float* Ufnew, float* acc, const Geom& g,
                                  const Dx& dx, const StepScratch& s, const FallbackQueue& q,
                                  cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(q.n, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  switch (M.ndim) {
    case 1:
      e = launch_sweep<1, 0, 256, 1, ONLY>(M, Uf, U, g, dx, s.dt, acc, Unew, Ufnew, q, st);
      if (e == cudaSuccess) e = launch_fallback<1>(M, q, g, dx, s.dt, Unew, Ufnew, st);
      break;
    case 2:
      e = launch_sweep<2, 0, 32, 8, FIRST>(M, Uf, U, g, dx, s.dt, acc, Unew, Ufnew, q, st);
      if (e == cudaSuccess)
        e = launch_sweep<2, 1, 16, 16, LAST>(M, Uf, U, g, dx, s.dt, acc, Unew, Ufnew, q, st);
      if (e == cudaSuccess) e = launch_fallback<2>(M, q, g, dx, s.dt, Unew, Ufnew, st);
      break;
    case 3:
      e = launch_sweep<3, 0, 32, 8, FIRST>(M, Uf, U, g, dx, s.dt, acc, Unew, Ufnew, q, st);
      if (e == cudaSuccess)
        e = launch_sweep<3, 1, 16, 16, MID>(M, Uf, U, g, dx, s.dt, acc, Unew, Ufnew, q, st);
      if (e == cudaSuccess)
        e = launch_sweep<3, 2, 16, 16, LAST>(M, Uf, U, g, dx, s.dt, acc, Unew, Ufnew, q, st);
      if (e == cudaSuccess) e = launch_fallback<3>(M, q, g, dx, s.dt, Unew, Ufnew, st);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return e;
}

// Tile counts of a sweep of box dims along axis A (the item lists of a batch
// enumerate these); must match the tile shapes the sweeps are launched with.
void sweep_tiles(int ndim, int axis, const int* n, int* tS, int* tP) {
  if (ndim == 1) {
    *tS = 256;
    *tP = 1;
  } else if (axis == 0) {
    *tS = 32;
    *tP = 8;
  } else {
    *tS = 16;
    *tP = 16;
  }
  (void)n;
}

cudaError_t launch_batch_cfl_mixed(const MixedParams& M, double courant, const BoxDesc* TB,
                                   const BatchLists& L, cudaStream_t st) {
  if (!L.n_cfl) return cudaSuccess;
  switch (M.ndim) {
    case 1: batch_cfl_f32_kernel<1><<<152 * 4, 256, 0, st>>>(M, courant, TB, L.cfl, L.n_cfl, L.heads + 0); break;
    case 2: batch_cfl_f32_kernel<2><<<152 * 4, 256, 0, st>>>(M, courant, TB, L.cfl, L.n_cfl, L.heads + 0); break;
    case 3: batch_cfl_f32_kernel<3><<<152 * 4, 256, 0, st>>>(M, courant, TB, L.cfl, L.n_cfl, L.heads + 0); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// The mixed passes of one batch step after the CFL and ghost passes: the
// sweeps of every box (slot 5 + axis of the queue heads), then the FP64
// fix-up of the queued interfaces.
cudaError_t launch_batch_sweeps(const MixedParams& M, const BoxDesc* TB, const BatchLists& L,
                                const FallbackQueue& q, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(q.n, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  switch (M.ndim) {
    case 1:
      e = launch_batch_sweep<1, 0, 256, 1, ONLY>(M, TB, L, q, 5, st);
      if (e == cudaSuccess) e = launch_batch_fallback<1>(M, TB, q, st);
      break;
    case 2:
      e = launch_batch_sweep<2, 0, 32, 8, FIRST>(M, TB, L, q, 5, st);
      if (e == cudaSuccess) e = launch_batch_sweep<2, 1, 16, 16, LAST>(M, TB, L, q, 6, st);
      if (e == cudaSuccess) e = launch_batch_fallback<2>(M, TB, q, st);
      break;
    case 3:
      e = launch_batch_sweep<3, 0, 32, 8, FIRST>(M, TB, L, q, 5, st);
      if (e == cudaSuccess) e = launch_batch_sweep<3, 1, 16, 16, MID>(M, TB, L, q, 6, st);
      if (e == cudaSuccess) e = launch_batch_sweep<3, 2, 16, 16, LAST>(M, TB, L, q, 7, st);
      if (e == cudaSuccess) e = launch_batch_fallback<3>(M, TB, q, st);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return e;
}

}  // namespace rgpu
