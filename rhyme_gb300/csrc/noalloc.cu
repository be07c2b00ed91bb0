// noalloc.cu -- the one entry point that allocates nothing on the device.
//
// Some callers cannot allocate device memory themselves or through this
// library: a host code whose device arrays come from its own pool (for
// example a Fortran driver whose boxes live in CUDA Fortran or OpenACC
// device arrays) and that must keep every device allocation under its own
// accounting, or a run under a fixed device-memory budget where a
// cudaMalloc in the middle of a step could fail, fragment the pool or
// synchronize the device. rhyme_gpu_mh_solve_noalloc serves them: the caller
// passes device pointers to the state before and after the step, and the
// solver's scratch (face states, interface fluxes and dt) lives in the
// file-scope array below, of fixed size, which every GPU that loads this
// library holds until the process exits.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/rhyme_gpu.h"
#include "rgpu_internal.h"

using namespace rgpu;

namespace {

constexpr long long kScratchDoubles = RHYME_GPU_NOALLOC_SCRATCH_DOUBLES;
constexpr int kMaxDevices = 64;

// Scratch shared by every call on a device: dt at [0], face states from
// [32], then the interface fluxes.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

double* g_scratch_addr[kMaxDevices] = {};
std::once_flag g_scratch_once[kMaxDevices];
cudaError_t g_scratch_err[kMaxDevices] = {};

// Device address of the scratch array on `dev` (the current device), looked
// up once per device.
cudaError_t scratch_on(int dev, double** out) {
  std::call_once(g_scratch_once[dev], [dev] {
    void* p = nullptr;
    g_scratch_err[dev] = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    g_scratch_addr[dev] = (double*)p;
  });
  *out = g_scratch_addr[dev];
  return g_scratch_err[dev];
}

int bad(const char* fmt, long long a = 0, long long b = 0) {
  fprintf(stderr, "rhyme_gpu_mh_solve_noalloc: ");
  fprintf(stderr, fmt, a, b);
  fprintf(stderr, "\n");
  return RHYME_GPU_EINVAL;
}

}  // namespace

extern "C" int rhyme_gpu_mh_solve_noalloc(const rhyme_gpu_params* params, const double* d_cells_in,
                                          double* d_cells_out, const int dims[3], const double dx[3],
                                          double dt, void* stream) {
  if (!params || !d_cells_in || !d_cells_out || !dims || !dx) return bad("null argument");
  const int D = params->ndim;
  if (D < 1 || D > 3) return bad("ndim must be 1, 2 or 3 (got %lld)", D);
  if (params->limiter < 1 || params->limiter > 4) return bad("unknown slope limiter %lld", params->limiter);
  if (params->solver_type != RHYME_GPU_CPU_INTENSIVE && params->solver_type != RHYME_GPU_MEMORY_INTENSIVE)
    return bad("unknown solver type %lld", params->solver_type);
  if (params->precision != RHYME_GPU_FP64) return bad("only the FP64 solver runs without allocation");
  if (!(params->gamma > 1.0) || !(params->kb_amu > 0.0) || params->n_iteration < 0)
    return bad("bad gas or Riemann parameters");
  if (!(dt > 0.0) || !std::isfinite(dt)) return bad("dt must be positive and finite");
  for (int a = 0; a < 3; ++a) {
    if (a < D && dims[a] < 1) return bad("dims(%lld) must be >= 1", a + 1);
    if (a >= D && dims[a] != 1) return bad("dims(%lld) must be 1 beyond NDIM", a + 1);
  }
  const Geom g = make_geom(D, dims);
  const long long need = 32 + 3LL * D * (D + 2) * g.field;
  if (need > kScratchDoubles)
    return bad("box too large: needs %lld scratch doubles, the fixed scratch holds %lld", need,
               kScratchDoubles);

  // The update reads U^n and writes U^{n+1} through restrict-qualified
  // pointers, so the two state arrays must not share memory.
  const long long bytes = (long long)(D + 2) * g.field * (long long)sizeof(double);
  const char* in_lo = (const char*)d_cells_in;
  const char* out_lo = (const char*)d_cells_out;
  if (in_lo < out_lo + bytes && out_lo < in_lo + bytes)
    return bad("d_cells_in and d_cells_out overlap; pass two separate state arrays");

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) return RHYME_GPU_ECUDA;
  double* base = nullptr;
  e = scratch_on(dev, &base);
  if (e != cudaSuccess || !base) {
    fprintf(stderr, "rhyme_gpu_mh_solve_noalloc: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
    return RHYME_GPU_ECUDA;
  }

  DevParams P;
  make_dev_params(params, &P);

  Dx d;
  memset(&d, 0, sizeof d);
  for (int a = 0; a < 3; ++a) d.v[a] = (a < D) ? dx[a] : 1.0;
  d.min = d.v[0];
  for (int a = 1; a < D; ++a)
    if (d.v[a] < d.min) d.min = d.v[a];
  for (int a = 0; a < 3; ++a) d.inv_f[a] = (float)(1.0 / d.v[a]);

  StepScratch s;
  s.dt = base;
  s.faces = base + 32;
  s.fluxes = s.faces + 2LL * D * (D + 2) * g.field;
  cudaStream_t st = (cudaStream_t)stream;
  e = launch_set_double(s.dt, dt, st);
  if (e == cudaSuccess) e = launch_mh_solve(P, d_cells_in, d_cells_out, g, d, s, st);
  if (e != cudaSuccess) {
    fprintf(stderr, "rhyme_gpu_mh_solve_noalloc: %s\n", cudaGetErrorString(e));
    return RHYME_GPU_ECUDA;
  }
  return RHYME_GPU_OK;
}
