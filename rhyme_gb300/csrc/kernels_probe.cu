// kernels_probe.cu -- arithmetic rate probe of the GPU (instrumentation).
//
// The roofline of this path is set by arithmetic, not by HBM: the plain FP64
// step is bound by the FP64 pipe (divisions, square roots and the powers of
// the exact Riemann solver), the mixed form by FP32 issue. This probe
// measures the rates those bounds are quoted against, with the same
// operations the solver uses: FP64 fused multiply-add, division, square
// root and libm_pow::pow; FP32 fused multiply-add, the sweeps' approximate
// division (this unit is built with -prec-div=false like the sweeps) and
// their power exp2f(y log2f(x)); and the two FP64 operations of the mixed
// form's state update, the FP64 add and the FP64 <-> FP32 conversions. Every thread runs kProbeChains independent
// dependency chains, so the pipes, not latencies, set the rate; each chain's
// result is written out so nothing is optimised away.
#include <cmath>

#include "../../include/rhyme_gpu.h"
#include "libm_pow.h"
#include "rgpu_internal.h"

namespace {

constexpr int kProbeChains = 8;
constexpr int kProbeThreads = 256;

template <int KIND>
__global__ void __launch_bounds__(kProbeThreads) probe_kernel(int iters, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (KIND < 4 || KIND >= 7) {
    double v[kProbeChains];
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) v[c] = 1.0 + 1e-3 * (t % 97) + 1e-4 * c;
    const double a = 0.999999, b = 1e-7, y = 0.2;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < kProbeChains; ++c) {
        if (KIND == 0) v[c] = fma(v[c], a, b);         // FP64 FMA
        if (KIND == 1) v[c] = __ddiv_rn(1.25, v[c]);   // FP64 division (x -> 1.25/x stays near 1.1)
        if (KIND == 2) v[c] = __dsqrt_rn(v[c] + 0.5);  // FP64 square root (converges to ~1.2)
        if (KIND == 3) v[c] = libm_pow::pow(v[c] + 0.25, y);  // the restated C-library pow
        if (KIND == 7) v[c] = __dadd_rn(v[c], b);               // FP64 add
        // FP64 -> FP32 -> FP64 (two conversions; the FP32 multiply keeps
        // the chain from folding)
        if (KIND == 8) v[c] = (double)__fmul_rn(__double2float_rn(v[c]), 0.9999999f);
      }
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) s += v[c];
    out[t] = s;
  } else {
    float v[kProbeChains];
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) v[c] = 1.0f + 1e-3f * (t % 97) + 1e-4f * c;
    const float a = 0.999999f, b = 1e-7f, y = 0.2f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < kProbeChains; ++c) {
        if (KIND == 4) v[c] = fmaf(v[c], a, b);                 // FP32 FMA
        if (KIND == 5) v[c] = 1.25f / v[c];                      // FP32 division (approximate)
        if (KIND == 6) v[c] = exp2f(y * log2f(v[c] + 0.25f));   // FP32 power as in the sweeps
      }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) s += v[c];
    out[t] = s;
  }
}

template <int KIND>
cudaError_t launch_probe(int blocks, int iters, double* out, cudaStream_t st) {
  probe_kernel<KIND><<<blocks, kProbeThreads, 0, st>>>(iters, out);
  return cudaGetLastError();
}

cudaError_t launch_kind(int kind, int blocks, int iters, double* out, cudaStream_t st) {
  switch (kind) {
    case 0: return launch_probe<0>(blocks, iters, out, st);
    case 1: return launch_probe<1>(blocks, iters, out, st);
    case 2: return launch_probe<2>(blocks, iters, out, st);
    case 3: return launch_probe<3>(blocks, iters, out, st);
    case 4: return launch_probe<4>(blocks, iters, out, st);
    case 5: return launch_probe<5>(blocks, iters, out, st);
    case 6: return launch_probe<6>(blocks, iters, out, st);
    case 7: return launch_probe<7>(blocks, iters, out, st);
    case 8: return launch_probe<8>(blocks, iters, out, st);
  }
  return cudaErrorInvalidValue;
}

// Self-check of the integer conversions of the mixed state update
// (rgpu_internal.h widen_f32, narrow_mirror) against the hardware ones, on
// n pseudo-random bit patterns per thread family (splitmix64): doubles of
// every exponent, doubles near the FP32 rounding boundaries, ties, the
// limits of the FP32 range, and FP32 values (subnormals excluded: the FP32
// units flush them).
__device__ __forceinline__ unsigned long long splitmix(unsigned long long& s) {
  unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void conversion_check_kernel(long long n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long local = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    unsigned long long s = seed ^ (unsigned long long)t * 0xD1B54A32D192ED03ull;
    const unsigned long long r = splitmix(s);
    unsigned long long bits;
    switch (t & 3) {
      case 0: bits = r; break;  // any double
      case 1: {                 // FP32 exponent range, low bits at or next to a tie
        const unsigned long long e = 896 + (r >> 56) % 256;
        const unsigned long long low = (r >> 8) & 3;
        bits = (r & 0x8000000000000000ull) | (e << 52) | (r & 0x000fffffe0000000ull) |
               (low == 0 ? 0x10000000ull : low == 1 ? 0x0fffffffull : low == 2 ? 0x10000001ull : (r & 0x1fffffffull));
        break;
      }
      case 2: {                 // the edges: around FLT_MIN and FLT_MAX, zeros
        const unsigned long long e = ((r >> 60) & 1) ? 896 + 254 + ((r >> 56) & 3) : 894 + ((r >> 56) & 3);
        bits = (r & 0x8000000000000000ull) | (e << 52) | (((r >> 61) & 1) ? 0x000fffffffffffffull : (r & 0x000fffffffffffffull));
        if (((r >> 50) & 15) == 0) bits &= 0x8000000000000000ull;
        break;
      }
      default: bits = 0; break;
    }
    if ((t & 3) != 3) {
      const double x = __longlong_as_double((long long)bits);
      const float a = rgpu::narrow_mirror(x), b = rgpu::mirror_of(x);
      if (__float_as_uint(a) != __float_as_uint(b) && !(isnan(a) && isnan(b))) ++local;
    } else {
      const unsigned f = (unsigned)r;
      const unsigned mag = f & 0x7fffffffu;
      if (mag != 0 && mag < 0x00800000u) continue;  // FP32 subnormal
      const float y = __uint_as_float(f);
      const double a = rgpu::widen_f32(y), b = (double)y;
      if (__double_as_longlong(a) != __double_as_longlong(b) && !(isnan(a) && isnan(b))) ++local;
    }
  }
  if (local) atomicAdd(bad, local);
}

}  // namespace

extern "C" int rhyme_gpu_check_conversions(long long n, unsigned long long seed, unsigned long long* mismatches) {
  if (n < 0 || !mismatches) return RHYME_GPU_EINVAL;
  unsigned long long* d = nullptr;
  cudaError_t e = cudaMalloc((void**)&d, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(unsigned long long));
  if (e == cudaSuccess && n > 0) {
    conversion_check_kernel<<<1024, 256>>>(n, seed, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(mismatches, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  return e == cudaSuccess ? RHYME_GPU_OK : RHYME_GPU_ECUDA;
}

extern "C" int rhyme_gpu_rate_probe(int kind, int iters, double* ops_per_second, double* ms) {
  if (kind < 0 || kind > 8 || iters < 1 || !ops_per_second) return RHYME_GPU_EINVAL;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return RHYME_GPU_ECUDA;
  const int blocks = sms * 8;  // 8 CTAs of 256 threads per SM
  const long long threads = (long long)blocks * kProbeThreads;
  double* out = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaStream_t st = nullptr;
  cudaError_t e = cudaMalloc((void**)&out, threads * sizeof(double));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  float best = 0.f;
  // one warm-up launch, then the fastest of three timed launches
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
    e = cudaEventRecord(ev[0], st);
    if (e == cudaSuccess) e = launch_kind(kind, blocks, iters, out, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
    if (e == cudaSuccess && rep > 0 && (best == 0.f || t < best)) best = t;
  }
  if (ev[0]) cudaEventDestroy(ev[0]);
  if (ev[1]) cudaEventDestroy(ev[1]);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  if (e != cudaSuccess || best <= 0.f) return RHYME_GPU_ECUDA;
  // operations: one per chain step (an FMA counts as two floating-point
  // operations for the FMA kinds, the conversion kind two conversions)
  const double ops =
      (double)threads * iters * kProbeChains * ((kind == 0 || kind == 4 || kind == 8) ? 2.0 : 1.0);
  *ops_per_second = ops / (best * 1e-3);
  if (ms) *ms = best;
  return RHYME_GPU_OK;
}
