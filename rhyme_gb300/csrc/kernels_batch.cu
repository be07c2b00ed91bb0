// kernels_batch.cu -- one step of a batch of independent boxes of uneven
// sizes, each with its own dt, boundary types, limiter and cell size.
//
// Every pass is one persistent kernel (a few CTAs per SM) fed by a work
// queue: the host lists, per box, the chunks of that pass's index space
// (largest boxes first), and each CTA repeatedly takes the next chunk with an
// atomic increment of the pass's queue head. The per-element arithmetic is
// the single-box code (box_elems.cuh, the mixed sweep body), so a box gives
// the same result alone and inside a batch. A step is captured once per
// buffer parity in a CUDA graph by the host.
//
// Compiled with --fmad=false (the FP64 passes must match the oracle).
#include "box_elems.cuh"

namespace rgpu {

namespace {

// Next work item of a pass for this CTA (-1 when the queue is empty).
__device__ __forceinline__ int next_item(int* head, int n) {
  __shared__ int s_item;
  __syncthreads();
  if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
  __syncthreads();
  const int it = s_item;
  return it < n ? it : -1;
}

template <int D>
__global__ void __launch_bounds__(256)
    batch_cfl_kernel(Gas<double> G, double courant, const BoxDesc* __restrict__ T,
                     const WorkItem* __restrict__ items, int n, int* head) {
  __shared__ double sm[8];
  __shared__ int sb[8];
  for (int it = next_item(head, n); it >= 0; it = next_item(head, n)) {
    const WorkItem w = items[it];
    const BoxDesc& b = T[w.box];
    const long long total = (long long)b.g.n[0] * b.g.n[1] * b.g.n[2];
    const long long t = w.chunk * kBatchChunk + threadIdx.x;
    double m = 0.0;
    int bad = 0;
    if (t < total) {
      const double v = signal_speed_elem<D>(G, b.U, b.g, t, bad);
      if (v > m) m = v;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double o = __shfl_down_sync(0xffffffffu, m, off);
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
      atomicMax(max_bits, (unsigned long long)__double_as_longlong(m));
      if (bad) atomicOr(status, 1);
      __threadfence();
      if (atomicAdd(counter, 1u) == (unsigned int)(b.cfl_items - 1)) {
        __threadfence();
        const double mu = __longlong_as_double((long long)atomicAdd(max_bits, 0ull));
        b.ctl[0] = courant * b.dx.min / mu;
        atomicExch(max_bits, 0ull);
        atomicExch(counter, 0u);
      }
    }
  }
}

template <int D, typename T>
__global__ void __launch_bounds__(256)
    batch_ghost_kernel(const BoxDesc* __restrict__ TB, const WorkItem* __restrict__ items, int n,
                       int* head, bool f32) {
  for (int it = next_item(head, n); it >= 0; it = next_item(head, n)) {
    const WorkItem w = items[it];
    const BoxDesc& b = TB[w.box];
    long long off1, off2, total;
    ghost_offsets<D>(b.g, off1, off2, total);
    const long long t = w.chunk * kBatchChunk + threadIdx.x;
    if (t >= total) continue;
    BoxRules R;
    for (int i = 0; i < 6; ++i) {
      R.bc[i] = b.bc[i];
      for (int c = 0; c < 5; ++c) R.inflow[i][c] = b.inflow[i][c];
    }
    if (f32)
      ghost_elem<D, T>(R, (T*)b.Uf, (T*)nullptr, b.g, off1, off2, t);
    else
      ghost_elem<D, T>(R, (T*)b.U, (T*)b.V, b.g, off1, off2, t);
  }
}

template <int D>
__device__ __forceinline__ BoxRules rules_of_box(const BoxDesc& b) {
  BoxRules R;
  for (int i = 0; i < 6; ++i) R.bc[i] = b.bc[i];
  R.limiter = b.limiter;
  R.omega = b.omega;
  R.solver_type = b.solver_type;
  return R;
}

template <int D>
__global__ void __launch_bounds__(128)
    batch_faces_kernel(Gas<double> G, const BoxDesc* __restrict__ TB, const WorkItem* __restrict__ items,
                       int n, int* head) {
  for (int it = next_item(head, n); it >= 0; it = next_item(head, n)) {
    const WorkItem w = items[it];
    const BoxDesc& b = TB[w.box];
    const BoxRules R = rules_of_box<D>(b);
    const long long t = w.chunk * kBatchFluxChunk + threadIdx.x;
    const double dt = b.ctl[0];
    if (w.axis == 0) {
      if (t < face_count<0>(b.g)) faces_elem<D, 0>(G, R, b.U, b.g, 0.5 * dt / b.dx.v[0], b.faces, t);
    }
    if constexpr (D > 1) {
      if (w.axis == 1 && t < face_count<1>(b.g)) faces_elem<D, 1>(G, R, b.U, b.g, 0.5 * dt / b.dx.v[1], b.faces, t);
    }
    if constexpr (D > 2) {
      if (w.axis == 2 && t < face_count<2>(b.g)) faces_elem<D, 2>(G, R, b.U, b.g, 0.5 * dt / b.dx.v[2], b.faces, t);
    }
  }
}

// At least 3 CTAs per SM: the persistent grid is 152 x 3 CTAs (and in 3-D
// the FP64 solver would otherwise take 216 registers, 2 CTAs per SM).
template <int D>
__global__ void __launch_bounds__(128, 3)
    batch_flux_kernel(Gas<double> G, Rp<double> rp, const BoxDesc* __restrict__ TB,
                      const WorkItem* __restrict__ items, int n, int* head) {
  for (int it = next_item(head, n); it >= 0; it = next_item(head, n)) {
    const WorkItem w = items[it];
    const BoxDesc& b = TB[w.box];
    const long long t = w.chunk * kBatchFluxChunk + threadIdx.x;
    if (w.axis == 0) {
      if (t < iface_count<0>(b.g)) flux_elem<D, 0>(G, rp, b.faces, b.g, b.fluxes, t);
    }
    if constexpr (D > 1) {
      if (w.axis == 1 && t < iface_count<1>(b.g)) flux_elem<D, 1>(G, rp, b.faces, b.g, b.fluxes, t);
    }
    if constexpr (D > 2) {
      if (w.axis == 2 && t < iface_count<2>(b.g)) flux_elem<D, 2>(G, rp, b.faces, b.g, b.fluxes, t);
    }
  }
}

template <int D>
__global__ void __launch_bounds__(256)
    batch_update_kernel(const BoxDesc* __restrict__ TB, const WorkItem* __restrict__ items, int n,
                        int* head) {
  for (int it = next_item(head, n); it >= 0; it = next_item(head, n)) {
    const WorkItem w = items[it];
    const BoxDesc& b = TB[w.box];
    const long long total = (long long)b.g.n[0] * b.g.n[1] * b.g.n[2];
    const long long t = w.chunk * kBatchChunk + threadIdx.x;
    if (t >= total) continue;
    const double dt = b.ctl[0];
    double dtdx[3];
#pragma unroll
    for (int a = 0; a < D; ++a) dtdx[a] = dt / b.dx.v[a];
    update_elem<D>(b.solver_type, b.U, b.fluxes, b.g, dtdx, b.V, t);
  }
}

template <int D>
cudaError_t batch_step_d(const DevParams& P, const MixedParams& M, bool mixed, const BoxDesc* TB,
                         const BatchLists& L, FallbackQueue q, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(L.heads, 0, kBatchHeads * sizeof(int), st);
  if (e != cudaSuccess) return e;
  if (mixed) {
    e = launch_batch_cfl_mixed(M, P.courant, TB, L, st);
    if (e != cudaSuccess) return e;
  } else if (L.n_cfl) {
    batch_cfl_kernel<D><<<152 * 4, 256, 0, st>>>(P.G, P.courant, TB, L.cfl, L.n_cfl, L.heads + 0);
  }
  if (L.n_ghost) {
    batch_ghost_kernel<D, double><<<152 * 4, 256, 0, st>>>(TB, L.ghost, L.n_ghost, L.heads + 1, false);
    if (mixed) batch_ghost_kernel<D, float><<<152 * 4, 256, 0, st>>>(TB, L.ghost, L.n_ghost, L.heads + kHeadGhostF32, true);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (mixed) return launch_batch_sweeps(M, TB, L, q, st);
  if (L.n_faces) batch_faces_kernel<D><<<152 * 4, 128, 0, st>>>(P.G, TB, L.faces, L.n_faces, L.heads + 2);
  if (L.n_flux) batch_flux_kernel<D><<<152 * 3, 128, 0, st>>>(P.G, P.rp, TB, L.flux, L.n_flux, L.heads + 3);
  if (L.n_update) batch_update_kernel<D><<<152 * 4, 256, 0, st>>>(TB, L.update, L.n_update, L.heads + 4);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_batch_step(const DevParams& P, const MixedParams& M, bool mixed, int ndim,
                              const BoxDesc* table, const BatchLists& L, FallbackQueue q,
                              cudaStream_t st) {
  switch (ndim) {
    case 1: return batch_step_d<1>(P, M, mixed, table, L, q, st);
    case 2: return batch_step_d<2>(P, M, mixed, table, L, q, st);
    case 3: return batch_step_d<3>(P, M, mixed, table, L, q, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace rgpu
