// rhyme_gpu.cu -- host side of the C-ABI (include/rhyme_gpu.h).
//
// A context holds the run parameters (the values of Rhyme's solver modules),
// one CUDA stream, a copy stream (made on first use) and a registry of
// boxes. Each box owns two device state buffers (ping-pong: the unsplit
// update reads U^n and writes U^{n+1}), the solver scratch, and up to two
// captured CUDA graphs of one driver step (one per buffer parity) that
// rhyme_gpu_run replays. Large 2-/3-D mixed boxes with a page-locked host
// array move in slabs of rows on the copy stream, overlapped with the
// kernels (upload_slabs, solve_slabs_write_back). Below the single-box
// entry points: the autotuner, level output, sanity checks and painting,
// batches, and the server.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <map>
#include <vector>

#include "../../include/rhyme_gpu.h"
#include "rgpu_internal.h"

using namespace rgpu;

namespace {

// Slabs of an overlapped upload or solve, and the smallest box (hydro bytes)
// worth it.
constexpr int kPipeSlabs = 16;
constexpr size_t kPipeMinBytes = size_t(16) << 20;

struct Box {
  int level = 0, number = 0;
  double* host = nullptr;
  int dims[3] = {1, 1, 1};
  int ncmp = 0;
  Geom g{};
  size_t hydro_bytes = 0;  // (NDIM+2) component blocks
  double* state[2] = {nullptr, nullptr};
  int cur = 0;
  StepScratch s{};
  float* Uf[2] = {nullptr, nullptr};  // FP32 mirrors of the state (mixed mode)
  float* acc = nullptr;               // FP32 flux-difference accumulator (mixed mode)
  int* fb_count = nullptr;            // interfaces redone in FP64 (mixed mode)
  FallbackQueue fbq{};                // FP64 fallback queue (mixed mode)
  double* trace_buf = nullptr;
  int* trace_pos = nullptr;
  bool registered_host = false;
  bool host_pinned = false;  // host array is page-locked (no wait after upload)
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  Dx graph_dx{};
  bool graph_valid = false;
  DevParams dp{};   // the context's parameters with this box's overrides
  MixedParams mp{};
  Dx dx{};          // cell size for batched steps (rhyme_gpu_batch_create)
  SweepPlan plan{};  // tile shape per axis of the mixed sweeps
  bool plan_valid = false;
  // Copies overlapped with kernels (2-/3-D mixed boxes with a page-locked
  // host array): an upload writes the FP32 mirror of the arriving rows
  // (mirror_valid: Uf[cur] is the FP32 image of the current state, as long
  // as ghost fills keep the two in step) and folds their CFL maximum into
  // *ingest_bits (maxu_valid: it is the current state's), and with
  // write-back on (wb) a solve copies the rows of the new state to the host
  // array as they are finished (wb_pending: the host array receives the
  // current state).
  unsigned long long* ingest_bits = nullptr;
  int* fb_done = nullptr;  // fix-up entries done by the slabs solved so far
  bool mirror_valid = false;
  bool maxu_valid = false;
  // the resident run's carry (mixed): the last sweep of each captured step
  // writes the next state's FP32 mirror and folds its signal speeds into
  // *carry_bits; *carry_ok (device) lets the next CFL pass use them;
  // carry_valid: nothing changed the state since the last resident run
  unsigned long long* carry_bits = nullptr;
  int* carry_ok = nullptr;
  bool carry_valid = false;
  bool wb = false;
  bool wb_pending = false;
};

}  // namespace

struct rhyme_gpu_ctx {
  rhyme_gpu_params params{};
  DevParams dp{};
  MixedParams mp{};
  bool mixed = false;
  bool fuse_xy = true;  // 3-D mixed: the x and y sweeps as one kernel (RHYME_GPU_XY=0: two)
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<Box*> boxes;
  double* pinned_dt = nullptr;   // pinned host scalars read back synchronously (dt, status, totals)
  void* elem_buf = nullptr;      // growable device buffer for element calls
  size_t elem_cap = 0;
  double timeout_s = 600.0;
  std::map<int, int> tuned;  // box-size class -> tile shape (mixed sweeps)
  // level output drain (rhyme_gpu_output_level)
  cudaStream_t copy = nullptr;
  cudaEvent_t out_packed = nullptr, out_done = nullptr;
  float* out_dev = nullptr;
  size_t out_cap = 0;  // floats
  PackDesc* out_desc = nullptr;
  size_t desc_cap = 0;  // descriptors
  bool out_pending = false;
  // slab pipelines of uploads and write-backs (on the copy stream)
  cudaEvent_t pipe_ev[kPipeSlabs + 1] = {};
  cudaEvent_t wb_done = nullptr;
};

namespace {

constexpr int kTraceCap = 4096;

int fail(rhyme_gpu_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? RHYME_GPU_ENOMEM : RHYME_GPU_ECUDA, \
                  "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);   \
  } while (0)

// Bounded wait on the context stream: polls an event until the deadline.
int wait_stream(rhyme_gpu_ctx* ctx) {
  cudaEvent_t ev;
  CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev, ctx->stream);
  if (e != cudaSuccess) {
    cudaEventDestroy(ev);
    return fail(ctx, RHYME_GPU_ECUDA, "cudaEventRecord: %s", cudaGetErrorString(e));
  }
  auto t0 = std::chrono::steady_clock::now();
  int spins = 0;
  for (;;) {
    e = cudaEventQuery(ev);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) {
      cudaEventDestroy(ev);
      return fail(ctx, RHYME_GPU_ECUDA, "stream wait: %s", cudaGetErrorString(e));
    }
    double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el > ctx->timeout_s) {
      cudaEventDestroy(ev);
      return fail(ctx, RHYME_GPU_ETIMEDOUT, "stream wait exceeded %.0f s", ctx->timeout_s);
    }
    if (++spins > 64) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  cudaEventDestroy(ev);
  return RHYME_GPU_OK;
}

Box* find_box(rhyme_gpu_ctx* ctx, int handle) {
  if (handle < 0 || handle >= (int)ctx->boxes.size()) return nullptr;
  return ctx->boxes[handle];
}

int validate(rhyme_gpu_ctx* ctx, const rhyme_gpu_params* p) {
  if (p->ndim < 1 || p->ndim > 3) return fail(ctx, RHYME_GPU_EINVAL, "ndim must be 1, 2 or 3 (got %d)", p->ndim);
  if (p->limiter < 1 || p->limiter > 4) return fail(ctx, RHYME_GPU_EINVAL, "unknown slope limiter %d", p->limiter);
  if (p->solver_type != RHYME_GPU_CPU_INTENSIVE && p->solver_type != RHYME_GPU_MEMORY_INTENSIVE)
    return fail(ctx, RHYME_GPU_EINVAL, "Unknown solver type %d", p->solver_type);
  if (p->precision != RHYME_GPU_FP64 && p->precision != RHYME_GPU_MIXED)
    return fail(ctx, RHYME_GPU_EINVAL, "unknown precision mode %d", p->precision);
  if (p->sweep_tuning != RHYME_GPU_TUNE_AUTO && p->sweep_tuning != RHYME_GPU_TUNE_FIXED)
    return fail(ctx, RHYME_GPU_EINVAL, "unknown sweep tuning mode %d", p->sweep_tuning);
  if (p->n_iteration < 0) return fail(ctx, RHYME_GPU_EINVAL, "n_iteration must be >= 0");
  if (!(p->gamma > 1.0)) return fail(ctx, RHYME_GPU_EINVAL, "gamma must exceed 1");
  if (!(p->kb_amu > 0.0)) return fail(ctx, RHYME_GPU_EINVAL, "kb_amu must be positive");
  if (!(p->courant > 0.0)) return fail(ctx, RHYME_GPU_EINVAL, "courant number must be positive");
  for (int i = 0; i < 2 * p->ndim; ++i)
    if (p->bc[i] < 1 || p->bc[i] > 5) return fail(ctx, RHYME_GPU_EINVAL, "unknown boundary type %d on side %d", p->bc[i], i + 1);
  return RHYME_GPU_OK;
}

}  // namespace

// Declared in rgpu_internal.h: the allocation-free entry point builds its
// kernel parameters with the same function.
void rgpu::make_dev_params(const rhyme_gpu_params* p, DevParams* d) {
  memset(d, 0, sizeof(*d));
  const double g = p->gamma;
  Gas<double>& G = d->G;
  G.g = g;
  G.gm1 = g - 1.0;
  G.gp1 = g + 1.0;
  G.gm1_gp1 = G.gm1 / G.gp1;
  G.gm1_2g = G.gm1 / (2.0 * g);
  G.gp1_2g = G.gp1 / (2.0 * g);
  G.g_inv = 1.0 / g;
  G.kb_amu = p->kb_amu;
  G.two_gp1 = 2.0 / G.gp1;
  G.two_gm1 = 2.0 / G.gm1;
  G.inv_gm1_2g = 1.0 / G.gm1_2g;
  G.gm1_half = 0.5 * G.gm1;
  G.half_gm1 = G.gm1 / 2.0;
  G.g_kb_amu = g * p->kb_amu;
  d->rp.vac_rho = p->vacuum_density;
  d->rp.vac_p = p->vacuum_pressure;
  d->rp.vac_rho_next = std::nextafter(p->vacuum_density, 1.0);
  d->rp.tol = p->tolerance;
  d->rp.n_iter = p->n_iteration;
  d->ndim = p->ndim;
  d->limiter = p->limiter;
  d->omega = p->omega;
  d->solver_type = p->solver_type;
  for (int i = 0; i < 6; ++i) {
    d->bc[i] = (i < 2 * p->ndim) ? p->bc[i] : 0;
    for (int c = 0; c < 5; ++c) d->inflow[i][c] = p->inflow[i][c];
  }
  d->courant = p->courant;
}

namespace {

void make_mixed_params(const DevParams& d, MixedParams* m) {
  memset(m, 0, sizeof(*m));
  const Gas<double>& G = d.G;
  Gas<float>& F = m->G;
  F.g = (float)G.g;
  F.gm1 = (float)G.gm1;
  F.gp1 = (float)G.gp1;
  F.gm1_gp1 = (float)G.gm1_gp1;
  F.gm1_2g = (float)G.gm1_2g;
  F.gp1_2g = (float)G.gp1_2g;
  F.g_inv = (float)G.g_inv;
  F.kb_amu = (float)G.kb_amu;
  F.two_gp1 = (float)G.two_gp1;
  F.two_gm1 = (float)G.two_gm1;
  F.inv_gm1_2g = (float)G.inv_gm1_2g;
  F.gm1_half = (float)G.gm1_half;
  F.half_gm1 = (float)G.half_gm1;
  F.g_kb_amu = (float)G.g_kb_amu;
  m->rp.vac_rho = (float)d.rp.vac_rho;
  m->rp.vac_p = (float)d.rp.vac_p;
  m->rp.vac_rho_next = std::nextafter((float)d.rp.vac_rho, 1.0f);
  m->rp.tol = (float)d.rp.tol;
  m->rp.n_iter = d.rp.n_iter;
  m->G64 = d.G;
  m->rp64 = d.rp;
  m->ndim = d.ndim;
  m->limiter = d.limiter;
  m->omega = (float)d.omega;
  m->omega64 = d.omega;
}

// Frees a box's device memory in stream order on `st` (after the work
// already queued there) and unpins the caller's array.
void destroy_box(Box* b, cudaStream_t st) {
  if (!b) return;
  for (int i = 0; i < 2; ++i) {
    if (b->graph[i]) cudaGraphExecDestroy(b->graph[i]);
    if (b->state[i]) cudaFreeAsync(b->state[i], st);
    if (b->Uf[i]) cudaFreeAsync(b->Uf[i], st);
  }
  if (b->acc) cudaFreeAsync(b->acc, st);
  if (b->fbq.e) cudaFreeAsync(b->fbq.e, st);
  if (b->s.faces) cudaFreeAsync(b->s.faces, st);
  if (b->s.fluxes) cudaFreeAsync(b->s.fluxes, st);
  if (b->s.dt) cudaFreeAsync(b->s.dt, st);
  if (b->registered_host) cudaHostUnregister(b->host);
  delete b;
}

Dx make_dx(int D, const double dx[3]) {
  Dx d;
  memset(&d, 0, sizeof d);  // padding too: steps compare Dx values bytewise
  for (int a = 0; a < 3; ++a) d.v[a] = (a < D) ? dx[a] : 1.0;
  // minval(samr%levels(0)%dx), rhyme_cfl_time_step.f90:74
  d.min = d.v[0];
  for (int a = 1; a < D; ++a)
    if (d.v[a] < d.min) d.min = d.v[a];
  for (int a = 0; a < 3; ++a) d.inv_f[a] = (float)(1.0 / d.v[a]);
  return d;
}

}  // namespace

extern "C" {

int rhyme_gpu_abi_version(void) { return RHYME_GPU_ABI_VERSION; }

int rhyme_gpu_create(rhyme_gpu_ctx** out, const rhyme_gpu_params* params) {
  if (!out || !params) return RHYME_GPU_EINVAL;
  *out = nullptr;
  rhyme_gpu_ctx* ctx = new rhyme_gpu_ctx();
  int rc = validate(ctx, params);
  if (rc != RHYME_GPU_OK) {
    fprintf(stderr, "rhyme_gpu_create: %s\n", ctx->err.c_str());
    delete ctx;
    return rc;
  }
  ctx->params = *params;
  make_dev_params(params, &ctx->dp);
  make_mixed_params(ctx->dp, &ctx->mp);
  ctx->mixed = (params->precision == RHYME_GPU_MIXED);
  const char* xy = getenv("RHYME_GPU_XY");
  if (xy && atoi(xy) == 0) ctx->fuse_xy = false;
  const char* to = getenv("RHYME_GPU_TIMEOUT_S");
  if (to && atof(to) > 0) ctx->timeout_s = atof(to);
  cudaError_t e = cudaGetDevice(&ctx->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->pinned_dt, sizeof(double) * 8);
  if (e != cudaSuccess) {
    fprintf(stderr, "rhyme_gpu_create: %s\n", cudaGetErrorString(e));
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return RHYME_GPU_ECUDA;
  }
  *out = ctx;
  return RHYME_GPU_OK;
}

int rhyme_gpu_destroy(rhyme_gpu_ctx* ctx) {
  if (!ctx) return RHYME_GPU_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (Box* b : ctx->boxes) destroy_box(b, ctx->stream);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->copy) cudaStreamSynchronize(ctx->copy);
  cudaFree(ctx->elem_buf);
  cudaFree(ctx->out_dev);
  cudaFree(ctx->out_desc);
  if (ctx->out_packed) cudaEventDestroy(ctx->out_packed);
  if (ctx->out_done) cudaEventDestroy(ctx->out_done);
  for (cudaEvent_t ev : ctx->pipe_ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->wb_done) cudaEventDestroy(ctx->wb_done);
  if (ctx->copy) cudaStreamDestroy(ctx->copy);
  cudaFreeHost(ctx->pinned_dt);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return RHYME_GPU_OK;
}

const char* rhyme_gpu_last_error(const rhyme_gpu_ctx* ctx) { return ctx ? ctx->err.c_str() : ""; }

int rhyme_gpu_get_stream(rhyme_gpu_ctx* ctx, void** stream) {
  if (!ctx || !stream) return RHYME_GPU_EINVAL;
  *stream = (void*)ctx->stream;
  return RHYME_GPU_OK;
}

int rhyme_gpu_synchronize(rhyme_gpu_ctx* ctx) {
  if (!ctx) return RHYME_GPU_EINVAL;
  return wait_stream(ctx);
}

}  // extern "C"

namespace {

// Device bytes a box of these dims takes (state buffers and scratch).
long long box_device_bytes(int D, bool mixed, const int* dims) {
  const Geom g = make_geom(D, dims);
  const long long F = g.field;
  long long bytes = 2LL * (D + 2) * F * 8 + 64 + 8 * kTraceCap;
  if (mixed) {
    const long long cells = (long long)g.n[0] * g.n[1] * g.n[2];
    bytes += 2LL * (D + 2) * F * 4 + (D > 1 ? (D + 2) * F * 4 : 0);
    bytes += std::max<long long>(4096, D * cells / 16) * (long long)sizeof(FallbackEntry);
  } else {
    bytes += 3LL * D * (D + 2) * F * 8;
  }
  return bytes;
}

// The copy stream and its events, made on first use.
int ensure_copy_stream(rhyme_gpu_ctx* ctx) {
  if (ctx->copy) return RHYME_GPU_OK;
  CK(cudaStreamCreateWithFlags(&ctx->copy, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->out_packed, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->out_done, cudaEventDisableTiming));
  for (cudaEvent_t& ev : ctx->pipe_ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->wb_done, cudaEventDisableTiming));
  return RHYME_GPU_OK;
}

// The state of the box changed on the device: the upload's CFL maximum and
// the write-back no longer describe it.
void state_changed(Box* b) {
  b->mirror_valid = false;
  b->maxu_valid = false;
  b->carry_valid = false;
  b->wb_pending = false;
}

// Whether the box's copies overlap its kernels: mixed precision, 2-D or 3-D,
// a host array the library page-locked, and enough rows of the outermost
// axis to split.
bool pipelined(const rhyme_gpu_ctx* ctx, const Box* b) {
  const int D = ctx->params.ndim;
  return ctx->mixed && D >= 2 && b->registered_host && b->hydro_bytes >= kPipeMinBytes &&
         b->g.n[D - 1] >= 2 * kPipeSlabs;
}

// Upload in slabs of rows of the outermost axis (copy stream); each slab,
// once arrived, has its ghost cells copied to the other buffer and the CFL
// maximum of its interior folded into *ingest_bits (context stream), while
// the next slab is in flight.
int upload_slabs(rhyme_gpu_ctx* ctx, Box* b) {
  int rc = ensure_copy_stream(ctx);
  if (rc != RHYME_GPU_OK) return rc;
  const int D = ctx->params.ndim, O = D - 1;
  const long long row = b->g.s[O];
  const int rows = b->g.n[O] + 4;
  const size_t pitch = (size_t)b->g.field * sizeof(double);
  double* U = b->state[b->cur];
  double* V = b->state[1 - b->cur];
  state_changed(b);
  // the copies follow the context stream's earlier work on these buffers
  CK(cudaEventRecord(ctx->pipe_ev[kPipeSlabs], ctx->stream));
  CK(cudaStreamWaitEvent(ctx->copy, ctx->pipe_ev[kPipeSlabs], 0));
  CK(cudaMemsetAsync(b->ingest_bits, 0, sizeof(unsigned long long), ctx->stream));
  const int per = (rows + kPipeSlabs - 1) / kPipeSlabs;
  for (int j = 0; j < kPipeSlabs; ++j) {
    const int r0 = j * per, r1 = std::min(rows, r0 + per);
    if (r0 >= r1) break;
    const size_t off = (size_t)r0 * row;
    CK(cudaMemcpy2DAsync(U + off, pitch, b->host + off, pitch, (size_t)(r1 - r0) * row * sizeof(double), D + 2,
                         cudaMemcpyHostToDevice, ctx->copy));
    CK(cudaEventRecord(ctx->pipe_ev[j], ctx->copy));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->pipe_ev[j], 0));
    CK(launch_ingest_mixed(b->mp, U, V, b->Uf[b->cur], b->g, (long long)off, (long long)r1 * row, b->ingest_bits,
                           b->s.status, ctx->stream));
  }
  b->mirror_valid = true;
  b->maxu_valid = true;
  return RHYME_GPU_OK;
}

int register_box_impl(rhyme_gpu_ctx* ctx, int level, int number, double* cells, const int dims[3], int ghost,
                      int ncmp, bool pin, bool upload, int* handle, bool host_pinned = false) {
  if (!ctx || !cells || !dims || !handle) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  const int D = ctx->params.ndim;
  if (ghost != 2) return fail(ctx, RHYME_GPU_EINVAL, "ghost width must be 2 (got %d)", ghost);
  if (ncmp < D + 2) return fail(ctx, RHYME_GPU_EINVAL, "ncmp %d < NDIM+2", ncmp);
  for (int a = 0; a < 3; ++a) {
    if (a < D && dims[a] < 1) return fail(ctx, RHYME_GPU_EINVAL, "dims(%d) must be >= 1", a + 1);
    if (a >= D && dims[a] != 1) return fail(ctx, RHYME_GPU_EINVAL, "dims(%d) must be 1 beyond NDIM", a + 1);
  }
  Box* b = new Box();
  b->dp = ctx->dp;
  b->mp = ctx->mp;
  b->level = level;
  b->number = number;
  b->host = cells;
  b->host_pinned = host_pinned;
  b->ncmp = ncmp;
  for (int a = 0; a < 3; ++a) b->dims[a] = dims[a];
  b->g = make_geom(D, dims);
  const long long F = b->g.field;
  b->hydro_bytes = (size_t)(D + 2) * F * sizeof(double);
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaMallocAsync((void**)&b->state[i], b->hydro_bytes, st);
  if (ctx->mixed) {
    for (int i = 0; i < 2 && e == cudaSuccess; ++i)
      e = cudaMallocAsync((void**)&b->Uf[i], (size_t)(D + 2) * F * sizeof(float), st);
    if (e == cudaSuccess && D > 1) e = cudaMallocAsync((void**)&b->acc, (size_t)(D + 2) * F * sizeof(float), st);
    long long cells_n = (long long)b->g.n[0] * b->g.n[1] * b->g.n[2];
    b->fbq.cap = (int)std::min<long long>(std::max<long long>(4096, D * cells_n / 16), 1LL << 30);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->fbq.e, (size_t)b->fbq.cap * sizeof(FallbackEntry), st);
  } else {
    if (e == cudaSuccess)
      e = cudaMallocAsync((void**)&b->s.faces, (size_t)2 * D * (D + 2) * F * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->s.fluxes, (size_t)D * (D + 2) * F * sizeof(double), st);
  }
  // small block: dt, max_bits, counter, status, trace_pos, then the trace
  const size_t small = 64 + sizeof(double) * kTraceCap;
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->s.dt, small, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->s.dt, 0, small, st);
  if (e != cudaSuccess) {
    destroy_box(b, st);
    return fail(ctx, e == cudaErrorMemoryAllocation ? RHYME_GPU_ENOMEM : RHYME_GPU_ECUDA,
                "box allocation: %s", cudaGetErrorString(e));
  }
  char* base = (char*)b->s.dt;
  b->s.max_bits = (unsigned long long*)(base + 8);
  b->s.counter = (unsigned int*)(base + 16);
  b->s.status = (int*)(base + 20);
  b->trace_pos = (int*)(base + 24);
  b->fb_count = (int*)(base + 28);
  b->fbq.n = (int*)(base + 32);
  b->fb_done = (int*)(base + 36);
  b->ingest_bits = (unsigned long long*)(base + 40);
  b->carry_bits = (unsigned long long*)(base + 48);
  b->carry_ok = (int*)(base + 56);
  b->fbq.status = b->s.status;
  b->fbq.total = b->fb_count;
  b->trace_buf = (double*)(base + 64);
  // Pin the caller's array for asynchronous copies when asked and possible;
  // a failure here only costs copy speed.
  if (pin) {
    if (cudaHostRegister(cells, (size_t)ncmp * F * sizeof(double), cudaHostRegisterDefault) == cudaSuccess)
      b->registered_host = true;
    else
      cudaGetLastError();
  }
  // set up before the upload (the server passes page-locked staging)
  // reuse a free slot
  int h = -1;
  for (int i = 0; i < (int)ctx->boxes.size(); ++i)
    if (!ctx->boxes[i]) {
      h = i;
      break;
    }
  if (h < 0) {
    ctx->boxes.push_back(b);
    h = (int)ctx->boxes.size() - 1;
  } else {
    ctx->boxes[h] = b;
  }
  *handle = h;
  if (!upload) return RHYME_GPU_OK;
  return rhyme_gpu_sync_to_device(ctx, h);
}

}  // namespace

extern "C" {

int rhyme_gpu_register_box(rhyme_gpu_ctx* ctx, int level, int number, double* cells, const int dims[3],
                           int ghost, int ncmp, int* handle) {
  return register_box_impl(ctx, level, number, cells, dims, ghost, ncmp, true, true, handle);
}

int rhyme_gpu_unregister_box(rhyme_gpu_ctx* ctx, int handle) {
  if (!ctx) return RHYME_GPU_EINVAL;
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  // copies to or from the host array may be in flight (the context stream
  // waits for them)
  if (b->registered_host) {
    int rc = wait_stream(ctx);
    if (rc != RHYME_GPU_OK) return rc;
  }
  destroy_box(b, ctx->stream);
  ctx->boxes[handle] = nullptr;
  return RHYME_GPU_OK;
}

int rhyme_gpu_sync_to_device(rhyme_gpu_ctx* ctx, int handle) {
  if (!ctx) return RHYME_GPU_EINVAL;
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  if (pipelined(ctx, b)) return upload_slabs(ctx, b);
  state_changed(b);
  // Both buffers receive the full hydro blocks (ghosts and corners included).
  CK(cudaMemcpyAsync(b->state[b->cur], b->host, b->hydro_bytes, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(b->state[1 - b->cur], b->state[b->cur], b->hydro_bytes, cudaMemcpyDeviceToDevice,
                     ctx->stream));
  if (ctx->mixed) {
    const long long n = (long long)(ctx->params.ndim + 2) * b->g.field;
    CK(launch_to_f32(b->state[b->cur], b->Uf[b->cur], n, ctx->stream));
    CK(launch_to_f32(b->state[b->cur], b->Uf[1 - b->cur], n, ctx->stream));
  }
  if (!b->registered_host && !b->host_pinned) return wait_stream(ctx);
  return RHYME_GPU_OK;
}

int rhyme_gpu_sync_to_host(rhyme_gpu_ctx* ctx, int handle) {
  if (!ctx) return RHYME_GPU_EINVAL;
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  // with write-back the solve's copies are in flight (the stream waits for them)
  if (!b->wb_pending)
    CK(cudaMemcpyAsync(b->host, b->state[b->cur], b->hydro_bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return wait_stream(ctx);
}

namespace {

// Checks a row range of the box's outermost axis; the copy's geometry.
int rows_geometry(rhyme_gpu_ctx* ctx, Box* b, int row0, int nrows, long long* row, size_t* pitch) {
  const int D = ctx->params.ndim;
  const int rows = b->g.n[D - 1] + 4;
  if (row0 < 0 || nrows < 1 || row0 + nrows > rows)
    return fail(ctx, RHYME_GPU_EINVAL, "rows [%d, %d) outside 0..%d", row0, row0 + nrows, rows);
  *row = b->g.s[D - 1];
  *pitch = (size_t)b->g.field * sizeof(double);
  return RHYME_GPU_OK;
}

}  // namespace

int rhyme_gpu_get_rows(rhyme_gpu_ctx* ctx, int handle, int row0, int nrows, double* out) {
  if (!ctx || !out) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  long long row;
  size_t pitch;
  int rc = rows_geometry(ctx, b, row0, nrows, &row, &pitch);
  if (rc != RHYME_GPU_OK) return rc;
  const size_t width = (size_t)nrows * row * sizeof(double);
  // out may be host memory or device memory (this GPU's or a peer's): the
  // copy kind follows the pointers
  CK(cudaMemcpy2DAsync(out, width, b->state[b->cur] + (size_t)row0 * row, pitch, width, ctx->params.ndim + 2,
                       cudaMemcpyDefault, ctx->stream));
  return wait_stream(ctx);
}

int rhyme_gpu_set_rows(rhyme_gpu_ctx* ctx, int handle, int row0, int nrows, const double* in) {
  if (!ctx || !in) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  long long row;
  size_t pitch;
  int rc = rows_geometry(ctx, b, row0, nrows, &row, &pitch);
  if (rc != RHYME_GPU_OK) return rc;
  const size_t width = (size_t)nrows * row * sizeof(double);
  const size_t off = (size_t)row0 * row;
  state_changed(b);
  CK(cudaMemcpy2DAsync(b->state[b->cur] + off, pitch, in, width, width, ctx->params.ndim + 2,
                       cudaMemcpyDefault, ctx->stream));
  CK(cudaMemcpy2DAsync(b->state[1 - b->cur] + off, pitch, b->state[b->cur] + off, pitch, width,
                       ctx->params.ndim + 2, cudaMemcpyDeviceToDevice, ctx->stream));
  // the caller's buffer may be reused on return
  return wait_stream(ctx);
}

int rhyme_gpu_set_host_writeback(rhyme_gpu_ctx* ctx, int handle, int on) {
  if (!ctx) return RHYME_GPU_EINVAL;
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  b->wb = on != 0;
  return RHYME_GPU_OK;
}

int rhyme_gpu_box_status(rhyme_gpu_ctx* ctx, int handle, int* flags) {
  if (!ctx || !flags) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  int* st = (int*)(ctx->pinned_dt + 1);
  CK(cudaMemcpyAsync(st, b->s.status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemsetAsync(b->s.status, 0, sizeof(int), ctx->stream));
  int rc = wait_stream(ctx);
  if (rc != RHYME_GPU_OK) return rc;
  *flags = *st;
  if (*st & 1)
    return fail(ctx, RHYME_GPU_ENANSTATE,
                "box (level %d, number %d) met non-positive density or a non-finite signal speed",
                b->level, b->number);
  return RHYME_GPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Step entry points
// ---------------------------------------------------------------------------
namespace {

StepScratch scratch_of(Box* b, bool trace) {
  StepScratch s = b->s;
  s.dt_trace = trace ? b->trace_buf : nullptr;
  s.trace_pos = b->trace_pos;
  s.trace_cap = trace ? kTraceCap : 0;
  return s;
}

// One driver step on the device: dt (into s.dt), ghost fill of U (mirrored
// into the other buffer), solve U -> other buffer.
// ---- autotuner of the mixed sweeps ------------------------------------------
//
// A box-size class is (NDIM, axis, ceil(log2) of the box's extent along the
// axis and along the pencil axis, each clamped to [3, 10]). The first box of
// a class met by a context has its sweep along that axis timed with every
// candidate tile shape (one warm-up and three timed launches each, CUDA
// events on the context's stream) on its current state; the fastest shape is
// kept for the class. A sweep only reads U^n and its FP32 mirror, so the
// timing launches leave the state alone (they write the next-step buffers,
// which the step itself overwrites).

int size_bucket(int n) {
  int b = 3;
  while (b < 10 && (1 << b) < n) ++b;
  return b;
}

int class_key(int D, int axis, const Geom& g) {
  const int bax = (D == 1) ? 1 : (axis == 0 ? 1 : 0);
  const int nB = (bax < D) ? g.n[bax] : 1;
  return D | (axis << 2) | (size_bucket(g.n[axis]) << 4) | (size_bucket(nB) << 8);
}

int tune_axis(rhyme_gpu_ctx* ctx, Box* b, const Dx& dx, int axis, int* best) {
  const int D = ctx->params.ndim;
  const int c = b->cur;
  StepScratch sc = scratch_of(b, false);
  *best = default_sweep_shape(D, axis, b->g.n[axis]);
  CK(launch_cfl_mixed(b->mp, b->state[c], b->Uf[c], b->g, b->dp.courant, dx, sc, ctx->stream));
  CK(launch_ghost_fill_f32(b->dp, b->Uf[c], b->g, ctx->stream));
  b->mirror_valid = false;  // the FP32 ghosts were filled without the FP64 ones
  cudaEvent_t ev[2];
  CK(cudaEventCreate(&ev[0]));
  if (cudaEventCreate(&ev[1]) != cudaSuccess) {
    cudaEventDestroy(ev[0]);
    return fail(ctx, RHYME_GPU_ECUDA, "event create failed");
  }
  int rc = RHYME_GPU_OK;
  float best_ms = 0.f;
  bool have = false;
  for (int k = 0; k < kSweepShapes && rc == RHYME_GPU_OK; ++k) {
    float total = 0.f;
    bool ok = true;
    for (int rep = 0; rep < 4 && ok; ++rep) {
      cudaError_t e = cudaMemsetAsync(b->fbq.n, 0, sizeof(int), ctx->stream);
      if (e == cudaSuccess) e = cudaEventRecord(ev[0], ctx->stream);
      if (e == cudaSuccess)
        e = launch_sweep_axis(D, axis, k, b->mp, b->Uf[c], b->state[c], b->g, dx, sc.dt, b->acc,
                              b->state[1 - c], b->fbq, ctx->stream);
      if (e == cudaErrorInvalidConfiguration) {  // grid too large for this shape
        ok = false;
        break;
      }
      if (e == cudaSuccess) e = cudaEventRecord(ev[1], ctx->stream);
      if (e != cudaSuccess) {
        rc = fail(ctx, RHYME_GPU_ECUDA, "autotune launch: %s", cudaGetErrorString(e));
        break;
      }
      rc = wait_stream(ctx);
      if (rc != RHYME_GPU_OK) break;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[0], ev[1]);
      if (rep > 0) total += ms;
    }
    if (rc == RHYME_GPU_OK && ok && (!have || total < best_ms)) {
      have = true;
      best_ms = total;
      *best = k;
    }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (rc == RHYME_GPU_OK) CK(cudaMemsetAsync(b->fbq.n, 0, sizeof(int), ctx->stream));
  return rc;
}

// The box's tile shapes (mixed mode): from the class table, tuning the
// classes not seen yet (RHYME_GPU_TUNE_AUTO), or by the size rule. Must run
// outside stream capture.
int box_plan(rhyme_gpu_ctx* ctx, Box* b, const Dx& dx) {
  if (!ctx->mixed || b->plan_valid) return RHYME_GPU_OK;
  const int D = ctx->params.ndim;
  for (int a = 0; a < 3; ++a) b->plan.shape[a] = default_sweep_shape(D, a < D ? a : 0, b->g.n[a < D ? a : 0]);
  if (ctx->params.sweep_tuning == RHYME_GPU_TUNE_AUTO) {
    for (int a = 0; a < D; ++a) {
      const int key = class_key(D, a, b->g);
      auto it = ctx->tuned.find(key);
      if (it == ctx->tuned.end()) {
        int best = 0;
        int rc = tune_axis(ctx, b, dx, a, &best);
        if (rc != RHYME_GPU_OK) return rc;
        it = ctx->tuned.emplace(key, best).first;
      }
      b->plan.shape[a] = it->second;
    }
  }
  b->plan.fuse_xy = (D == 3 && ctx->fuse_xy) ? 1 : 0;
  b->plan_valid = true;
  return RHYME_GPU_OK;
}

// One captured step: CFL pass (dt; in mixed precision also the FP32
// mirror's interior), ghost fill (the FP64 state, the other buffer and the
// mirror's ghosts), solve. Running the ghost fill on a second stream beside
// the CFL pass made the captured step 2.8 % slower at 256^3.
// The mixed step's carry: the last sweep writes U^{n+1}'s FP32 mirror into
// the other buffer's mirror and folds its signal speeds.
SweepCarry carry_of(Box* b, int cur) {
  SweepCarry c;
  c.Uf_next = b->Uf[1 - cur];
  c.bits = b->carry_bits;
  c.status = b->s.status;
  return c;
}

// In mixed precision the step carries its CFL pass into the next one: the
// next step's CFL pass only forms dt from the carried maximum (unless the
// FP64 fix-up changed cells after the sweep; launch_cfl_carry).
cudaError_t enqueue_step(rhyme_gpu_ctx* ctx, Box* b, int cur, const Dx& dx, bool trace) {
  StepScratch s = scratch_of(b, trace);
  double* U = b->state[cur];
  double* V = b->state[1 - cur];
  cudaError_t e = ctx->mixed ? launch_cfl_carry(b->mp, U, b->Uf[cur], b->g, b->dp.courant, dx, s, b->carry_bits,
                                                b->carry_ok, b->fbq.n, ctx->stream)
                             : launch_cfl(b->dp, U, b->g, dx, s, ctx->stream);
  if (e == cudaSuccess) e = launch_ghost_fill(b->dp, U, V, b->g, ctx->stream, ctx->mixed ? b->Uf[cur] : nullptr);
  if (e != cudaSuccess) return e;
  if (ctx->mixed)
    return launch_mh_solve_mixed(b->mp, U, b->Uf[cur], V, b->acc, b->g, dx, s, b->fbq, b->plan, ctx->stream,
                                 nullptr, carry_of(b, cur));
  return launch_mh_solve(b->dp, U, V, b->g, dx, s, ctx->stream);
}

int ensure_graphs(rhyme_gpu_ctx* ctx, Box* b, const Dx& dx) {
  if (b->graph_valid && memcmp(&b->graph_dx, &dx, sizeof(Dx)) == 0) return RHYME_GPU_OK;
  int prc = box_plan(ctx, b, dx);
  if (prc != RHYME_GPU_OK) return prc;
  for (int i = 0; i < 2; ++i) {
    if (b->graph[i]) {
      cudaGraphExecDestroy(b->graph[i]);
      b->graph[i] = nullptr;
    }
  }
  for (int parity = 0; parity < 2; ++parity) {
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_step(ctx, b, parity, dx, true);
    cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (e2 == cudaSuccess) cudaGraphDestroy(graph);
      return fail(ctx, RHYME_GPU_ECUDA, "graph capture: %s",
                  cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    cudaError_t e3 = cudaGraphInstantiate(&b->graph[parity], graph, 0);
    cudaGraphDestroy(graph);
    if (e3 != cudaSuccess) return fail(ctx, RHYME_GPU_ECUDA, "graph instantiate: %s", cudaGetErrorString(e3));
  }
  b->graph_dx = dx;
  b->graph_valid = true;
  return RHYME_GPU_OK;
}

// The mixed solve in slabs of rows of the outermost axis (a multiple of
// every sweep's tile extent along it), each slab's finished rows copied to
// the host array on the copy stream while the next slab is solved. A slab's
// last row waits for the next slab, which may queue the FP64 fix-up of the
// interface between them. The context stream waits for the copies.
int solve_slabs_write_back(rhyme_gpu_ctx* ctx, Box* b, const Dx& d) {
  int rc = ensure_copy_stream(ctx);
  if (rc != RHYME_GPU_OK) return rc;
  const int D = ctx->params.ndim, O = D - 1;
  const int N = b->g.n[O];
  int align = 1;
  for (int a = 0; a < D; ++a) {
    int S = 1, P = 1;
    sweep_shape(D, b->plan.shape[a], &S, &P);
    const int bax = (a == 0) ? 1 : 0;
    const int t = (a == O) ? S : (bax == O ? P : 1);
    if (t > align) align = t;
  }
  int rows = (N + kPipeSlabs - 1) / kPipeSlabs;
  rows = (rows + align - 1) / align * align;
  const long long row = b->g.s[O];
  const size_t pitch = (size_t)b->g.field * sizeof(double);
  const double* U = b->state[b->cur];
  double* V = b->state[1 - b->cur];
  const StepScratch sc = scratch_of(b, false);
  CK(cudaMemsetAsync(b->fbq.n, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(b->fb_done, 0, sizeof(int), ctx->stream));
  long long copied = 0;  // array rows of V already sent
  int j = 0;
  for (int lo = 1; lo <= N; lo += rows, ++j) {
    const int hi = std::min(N, lo + rows - 1);
    CK(launch_mh_solve_mixed_slab(b->mp, U, b->Uf[b->cur], V, b->acc, b->g, d, sc, b->fbq, b->fb_done, b->plan,
                                  lo, hi, ctx->stream));
    // final: array rows up to the one of cell hi - 1 (cell i is array row
    // i + 1), or all of them after the last slab
    const long long end = (hi == N) ? (long long)N + 4 : (long long)hi + 1;
    CK(cudaEventRecord(ctx->pipe_ev[j], ctx->stream));
    CK(cudaStreamWaitEvent(ctx->copy, ctx->pipe_ev[j], 0));
    CK(cudaMemcpy2DAsync(b->host + copied * row, pitch, V + copied * row, pitch,
                         (size_t)((end - copied) * row) * sizeof(double), D + 2, cudaMemcpyDeviceToHost, ctx->copy));
    copied = end;
  }
  CK(cudaEventRecord(ctx->wb_done, ctx->copy));
  CK(cudaStreamWaitEvent(ctx->stream, ctx->wb_done, 0));
  return RHYME_GPU_OK;
}

}  // namespace

extern "C" {

int rhyme_gpu_cfl_time_step(rhyme_gpu_ctx* ctx, int handle, const double dx[3], double* dt) {
  if (!ctx || !dx || !dt) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  Dx d = make_dx(ctx->params.ndim, dx);
  if (ctx->mixed && b->maxu_valid)
    CK(launch_cfl_finish(b->ingest_bits, b->dp.courant, d, scratch_of(b, false), ctx->stream));
  else if (ctx->mixed)
    CK(launch_cfl_mixed(b->mp, b->state[b->cur], b->Uf[b->cur], b->g, b->dp.courant, d, scratch_of(b, false),
                        ctx->stream));
  else
    CK(launch_cfl(b->dp, b->state[b->cur], b->g, d, scratch_of(b, false), ctx->stream));
  CK(cudaMemcpyAsync(ctx->pinned_dt, b->s.dt, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  int rc = wait_stream(ctx);
  if (rc != RHYME_GPU_OK) return rc;
  *dt = ctx->pinned_dt[0];
  return RHYME_GPU_OK;
}

double rhyme_gpu_cfl_dt(rhyme_gpu_ctx* ctx, int handle, const double dx[3]) {
  double dt = -1.0;
  if (rhyme_gpu_cfl_time_step(ctx, handle, dx, &dt) != RHYME_GPU_OK) return -1.0;
  return dt;
}

int rhyme_gpu_set_boundaries(rhyme_gpu_ctx* ctx, int handle) {
  if (!ctx) return RHYME_GPU_EINVAL;
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  CK(launch_ghost_fill(b->dp, b->state[b->cur], b->state[1 - b->cur], b->g, ctx->stream,
                       ctx->mixed ? b->Uf[b->cur] : nullptr));
  return RHYME_GPU_OK;
}

int rhyme_gpu_mh_solve(rhyme_gpu_ctx* ctx, int handle, const double dx[3], double dt) {
  if (!ctx || !dx) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(ctx, RHYME_GPU_EINVAL, "dt must be positive and finite");
  Dx d = make_dx(ctx->params.ndim, dx);
  int rc = box_plan(ctx, b, d);
  if (rc != RHYME_GPU_OK) return rc;
  // dt by value through a one-thread kernel: no host staging buffer, so no
  // wait for the stream (the host enqueues the solve while the ghost fill
  // or an upload still runs)
  CK(launch_set_double(b->s.dt, dt, ctx->stream));
  bool written_back = false;
  if (ctx->mixed) {
    // the FP32 mirror of the whole box (ghosts included) from the state this
    // solve reads, unless an upload wrote it since the state last changed
    // (the ghost fill keeps it in step): a driver may call the solve without
    // the CFL pass that otherwise writes the mirror
    if (!b->mirror_valid)
      CK(launch_to_f32(b->state[b->cur], b->Uf[b->cur], (long long)(ctx->params.ndim + 2) * b->g.field,
                       ctx->stream));
    if (b->wb && pipelined(ctx, b)) {
      rc = solve_slabs_write_back(ctx, b, d);
      if (rc != RHYME_GPU_OK) return rc;
      written_back = true;
    } else {
      CK(launch_mh_solve_mixed(b->mp, b->state[b->cur], b->Uf[b->cur], b->state[1 - b->cur], b->acc, b->g, d,
                               scratch_of(b, false), b->fbq, b->plan, ctx->stream));
    }
  }
  else
    CK(launch_mh_solve(b->dp, b->state[b->cur], b->state[1 - b->cur], b->g, d, scratch_of(b, false),
                       ctx->stream));
  b->cur = 1 - b->cur;
  state_changed(b);
  if (b->wb) {
    if (!written_back)
      CK(cudaMemcpyAsync(b->host, b->state[b->cur], b->hydro_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    b->wb_pending = true;
  }
  return RHYME_GPU_OK;
}

int rhyme_gpu_run(rhyme_gpu_ctx* ctx, int handle, const double dx[3], int nsteps, double* dt_trace) {
  if (!ctx || !dx) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  if (nsteps < 0) return fail(ctx, RHYME_GPU_EINVAL, "nsteps must be >= 0");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  Dx d = make_dx(ctx->params.ndim, dx);
  int rc = ensure_graphs(ctx, b, d);
  if (rc != RHYME_GPU_OK) return rc;
  if (nsteps == 0) return RHYME_GPU_OK;
  // a state changed since the last resident run: its first CFL pass is whole
  if (ctx->mixed && !b->carry_valid) CK(cudaMemsetAsync(b->carry_ok, 0, sizeof(int), ctx->stream));
  state_changed(b);
  b->carry_valid = true;
  int done = 0;
  while (done < nsteps) {
    const int chunk = (nsteps - done < kTraceCap) ? nsteps - done : kTraceCap;
    CK(cudaMemsetAsync(b->trace_pos, 0, sizeof(int), ctx->stream));
    for (int s = 0; s < chunk; ++s) {
      CK(cudaGraphLaunch(b->graph[b->cur], ctx->stream));
      b->cur = 1 - b->cur;
    }
    if (dt_trace) {
      CK(cudaMemcpyAsync(dt_trace + done, b->trace_buf, sizeof(double) * chunk, cudaMemcpyDeviceToHost,
                         ctx->stream));
      rc = wait_stream(ctx);
      if (rc != RHYME_GPU_OK) return rc;
    }
    done += chunk;
  }
  return RHYME_GPU_OK;
}

// ---------------------------------------------------------------------------
// Element-level entry points
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

int elem_reserve(rhyme_gpu_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->elem_cap) return RHYME_GPU_OK;
  int rc = wait_stream(ctx);
  if (rc != RHYME_GPU_OK) return rc;
  cudaFree(ctx->elem_buf);
  ctx->elem_buf = nullptr;
  ctx->elem_cap = 0;
  CK(cudaMalloc(&ctx->elem_buf, bytes));
  ctx->elem_cap = bytes;
  return RHYME_GPU_OK;
}

// Copies `nin` host arrays of in_sz[i] bytes to the device, runs `launch`
// with the device pointers, copies `nout` results back and waits.
template <typename F>
int elem_call(rhyme_gpu_ctx* ctx, int nin, const void* const* in, const size_t* in_sz, int nout,
              void* const* out, const size_t* out_sz, F launch) {
  size_t total = 0;
  size_t off[8];
  for (int i = 0; i < nin + nout; ++i) {
    off[i] = total;
    total += ((i < nin ? in_sz[i] : out_sz[i - nin]) + 255) & ~(size_t)255;
  }
  int rc = elem_reserve(ctx, total > 0 ? total : 256);
  if (rc != RHYME_GPU_OK) return rc;
  char* base = (char*)ctx->elem_buf;
  for (int i = 0; i < nin; ++i)
    CK(cudaMemcpyAsync(base + off[i], in[i], in_sz[i], cudaMemcpyHostToDevice, ctx->stream));
  CK(launch(base, off));
  for (int i = 0; i < nout; ++i)
    CK(cudaMemcpyAsync(out[i], base + off[nin + i], out_sz[i], cudaMemcpyDeviceToHost, ctx->stream));
  return wait_stream(ctx);
}

}  // namespace

extern "C" {

int rhyme_gpu_riemann_solve(rhyme_gpu_ctx* ctx, const double* l, const double* r, long long n,
                            double dx, double dt, int axis, double* u) {
  if (!ctx || n < 0 || (n > 0 && (!l || !r || !u))) return fail(ctx, RHYME_GPU_EINVAL, "bad argument");
  if (axis < 0 || axis >= ctx->params.ndim) return fail(ctx, RHYME_GPU_EINVAL, "axis %d out of range", axis);
  if (n == 0) return RHYME_GPU_OK;
  const size_t sz = (size_t)n * (ctx->params.ndim + 2) * sizeof(double);
  const void* in[2] = {l, r};
  size_t isz[2] = {sz, sz};
  void* out[1] = {u};
  size_t osz[1] = {sz};
  const double dxdt = dx / dt;  // rhyme_riemann_problem_solve.f90:17
  DevParams P = ctx->dp;
  return elem_call(ctx, 2, in, isz, 1, out, osz, [&](char* base, const size_t* off) {
    return launch_riemann_solve(P, (const double*)(base + off[0]), (const double*)(base + off[1]), n, dxdt,
                                axis, (double*)(base + off[2]), ctx->stream);
  });
}

int rhyme_gpu_irs_exec(rhyme_gpu_ctx* ctx, const double* states, long long n, double* out3) {
  if (!ctx || n < 0 || (n > 0 && (!states || !out3))) return fail(ctx, RHYME_GPU_EINVAL, "bad argument");
  if (n == 0) return RHYME_GPU_OK;
  const void* in[1] = {states};
  size_t isz[1] = {(size_t)n * 8 * sizeof(double)};
  void* out[1] = {out3};
  size_t osz[1] = {(size_t)n * 3 * sizeof(double)};
  DevParams P = ctx->dp;
  return elem_call(ctx, 1, in, isz, 1, out, osz, [&](char* base, const size_t* off) {
    return launch_irs_exec(P, (const double*)(base + off[0]), n, (double*)(base + off[1]), ctx->stream);
  });
}

int rhyme_gpu_slope_limiter(rhyme_gpu_ctx* ctx, const double* ul, const double* u, const double* ur,
                            long long n, double* delta) {
  if (!ctx || n < 0 || (n > 0 && (!ul || !u || !ur || !delta))) return fail(ctx, RHYME_GPU_EINVAL, "bad argument");
  if (n == 0) return RHYME_GPU_OK;
  const long long m = n * (ctx->params.ndim + 2);
  const size_t sz = (size_t)m * sizeof(double);
  const void* in[3] = {ul, u, ur};
  size_t isz[3] = {sz, sz, sz};
  void* out[1] = {delta};
  size_t osz[1] = {sz};
  DevParams P = ctx->dp;
  return elem_call(ctx, 3, in, isz, 1, out, osz, [&](char* base, const size_t* off) {
    return launch_slope_limiter(P, (const double*)(base + off[0]), (const double*)(base + off[1]),
                                (const double*)(base + off[2]), m, (double*)(base + off[3]), ctx->stream);
  });
}

int rhyme_gpu_half_step(rhyme_gpu_ctx* ctx, const double* u, const double* delta, long long n, int axis,
                        double dx, double dt, double* l, double* r) {
  if (!ctx || n < 0 || (n > 0 && (!u || !delta || !l || !r))) return fail(ctx, RHYME_GPU_EINVAL, "bad argument");
  if (axis < 0 || axis >= ctx->params.ndim) return fail(ctx, RHYME_GPU_EINVAL, "axis %d out of range", axis);
  if (n == 0) return RHYME_GPU_OK;
  const size_t sz = (size_t)n * (ctx->params.ndim + 2) * sizeof(double);
  const void* in[2] = {u, delta};
  size_t isz[2] = {sz, sz};
  void* out[2] = {l, r};
  size_t osz[2] = {sz, sz};
  const double hdtdx = 0.5 * dt / dx;  // .5d0*dt/dx, half_step_extrapolation.f90:20
  DevParams P = ctx->dp;
  return elem_call(ctx, 2, in, isz, 2, out, osz, [&](char* base, const size_t* off) {
    return launch_half_step(P, (const double*)(base + off[0]), (const double*)(base + off[1]), n, axis, hdtdx,
                            (double*)(base + off[2]), (double*)(base + off[3]), ctx->stream);
  });
}

}  // extern "C"

extern "C" int rhyme_gpu_profile_steps(rhyme_gpu_ctx* ctx, int handle, const double dx[3], int nsteps,
                                       double ms[5]) {
  if (!ctx || !dx || !ms || nsteps < 1) return fail(ctx, RHYME_GPU_EINVAL, "bad argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  Dx d = make_dx(ctx->params.ndim, dx);
  int prc = box_plan(ctx, b, d);
  if (prc != RHYME_GPU_OK) return prc;
  // the step as the resident run takes it (mixed: with the carried CFL)
  if (ctx->mixed && !b->carry_valid) CK(cudaMemsetAsync(b->carry_ok, 0, sizeof(int), ctx->stream));
  state_changed(b);
  cudaEvent_t ev[6];
  for (int i = 0; i < 6; ++i) CK(cudaEventCreate(&ev[i]));
  double acc[5] = {0, 0, 0, 0, 0};
  int rc = RHYME_GPU_OK;
  int fused = 0;
  for (int s = 0; s < nsteps && rc == RHYME_GPU_OK; ++s) {
    StepScratch sc = scratch_of(b, false);
    double* U = b->state[b->cur];
    double* V = b->state[1 - b->cur];
    cudaError_t e = cudaEventRecord(ev[0], ctx->stream);
    if (ctx->mixed) {
      // mixed: ms[2..4] are the x, y and z sweeps (the last one with the
      // FP64 fix-up of the queued interfaces and the carried CFL pass)
      if (e == cudaSuccess)
        e = launch_cfl_carry(b->mp, U, b->Uf[b->cur], b->g, b->dp.courant, d, sc, b->carry_bits, b->carry_ok,
                             b->fbq.n, ctx->stream);
      if (e == cudaSuccess) e = cudaEventRecord(ev[1], ctx->stream);
      if (e == cudaSuccess) e = launch_ghost_fill(b->dp, U, V, b->g, ctx->stream, b->Uf[b->cur]);
      if (e == cudaSuccess) e = cudaEventRecord(ev[2], ctx->stream);
      if (e == cudaSuccess)
        e = launch_mh_solve_mixed(b->mp, U, b->Uf[b->cur], V, b->acc, b->g, d, sc,
                                  b->fbq, b->plan, ctx->stream, ev + 3, carry_of(b, b->cur), &fused);
    } else {
      if (e == cudaSuccess) e = launch_cfl(b->dp, U, b->g, d, sc, ctx->stream);
      if (e == cudaSuccess) e = cudaEventRecord(ev[1], ctx->stream);
      if (e == cudaSuccess) e = launch_ghost_fill(b->dp, U, V, b->g, ctx->stream);
      if (e == cudaSuccess) e = launch_mh_solve(b->dp, U, V, b->g, d, sc, ctx->stream, ev + 2);
    }
    if (e != cudaSuccess) {
      rc = fail(ctx, RHYME_GPU_ECUDA, "profile launch: %s", cudaGetErrorString(e));
      break;
    }
    b->cur = 1 - b->cur;
    rc = wait_stream(ctx);
    if (rc != RHYME_GPU_OK) break;
    for (int k = 0; k < 5; ++k) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      acc[k] += t;
    }
  }
  for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
  for (int k = 0; k < 5; ++k) ms[k] = acc[k] / nsteps;
  if (fused) ms[3] = -1.0;  // ms[2]: the x and y sweeps as one kernel
  b->carry_valid = ctx->mixed && rc == RHYME_GPU_OK;
  return rc;
}

// ---- level output drain -----------------------------------------------------

namespace {

// Polls an event against the context's deadline.
int wait_event(rhyme_gpu_ctx* ctx, cudaEvent_t ev) {
  auto t0 = std::chrono::steady_clock::now();
  int spins = 0;
  for (;;) {
    cudaError_t e = cudaEventQuery(ev);
    if (e == cudaSuccess) return RHYME_GPU_OK;
    if (e != cudaErrorNotReady) return fail(ctx, RHYME_GPU_ECUDA, "event wait: %s", cudaGetErrorString(e));
    double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el > ctx->timeout_s) return fail(ctx, RHYME_GPU_ETIMEDOUT, "event wait exceeded %.0f s", ctx->timeout_s);
    if (++spins > 64) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

}  // namespace

extern "C" int rhyme_gpu_output_level(rhyme_gpu_ctx* ctx, const int* handles, int n, int ncmp, float* data,
                                      long long capacity) {
  if (!ctx || !handles || !data || n < 1) return fail(ctx, RHYME_GPU_EINVAL, "bad argument");
  const int D = ctx->params.ndim;
  if (ncmp < D + 2) return fail(ctx, RHYME_GPU_EINVAL, "ncmp %d < NDIM+2", ncmp);
  std::vector<PackDesc> desc(n);
  long long out_len = 0, hydro = 0;
  for (int i = 0; i < n; ++i) {
    Box* b = find_box(ctx, handles[i]);
    if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handles[i]);
    PackDesc& d = desc[i];
    d.U = b->state[b->cur];
    d.g = b->g;
    d.cells = (long long)b->g.n[0] * b->g.n[1] * b->g.n[2];
    d.hydro_off = hydro;
    d.out_off = out_len;
    hydro += (D + 2) * d.cells;
    out_len += (long long)ncmp * d.cells;
  }
  if (capacity < out_len)
    return fail(ctx, RHYME_GPU_EINVAL, "output holds %lld values, the level needs %lld", capacity, out_len);
  {
    int rc = ensure_copy_stream(ctx);
    if (rc != RHYME_GPU_OK) return rc;
  }
  // the staging buffers of an earlier output are reused once its copies ended
  if (ctx->out_pending) {
    int rc = wait_event(ctx, ctx->out_done);
    if (rc != RHYME_GPU_OK) return rc;
    ctx->out_pending = false;
  }
  if ((size_t)out_len > ctx->out_cap) {
    CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->out_dev);
    ctx->out_dev = nullptr;
    ctx->out_cap = 0;
    CK(cudaMalloc((void**)&ctx->out_dev, sizeof(float) * (size_t)out_len));
    ctx->out_cap = (size_t)out_len;
  }
  if ((size_t)n > ctx->desc_cap) {
    CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->out_desc);
    ctx->out_desc = nullptr;
    ctx->desc_cap = 0;
    CK(cudaMalloc((void**)&ctx->out_desc, sizeof(PackDesc) * (size_t)n));
    ctx->desc_cap = (size_t)n;
  }
  // pageable source: the copy is staged before the call returns
  CK(cudaMemcpyAsync(ctx->out_desc, desc.data(), sizeof(PackDesc) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_pack_level(ctx->out_desc, n, hydro, D, ctx->out_dev, ctx->stream));
  CK(cudaEventRecord(ctx->out_packed, ctx->stream));
  CK(cudaStreamWaitEvent(ctx->copy, ctx->out_packed, 0));
  if (ncmp == D + 2) {
    CK(cudaMemcpyAsync(data, ctx->out_dev, sizeof(float) * (size_t)out_len, cudaMemcpyDeviceToHost, ctx->copy));
  } else {  // the hydro blocks of a box are contiguous; the other components stay as they are
    for (int i = 0; i < n; ++i)
      CK(cudaMemcpyAsync(data + desc[i].out_off, ctx->out_dev + desc[i].out_off,
                         sizeof(float) * (size_t)(D + 2) * desc[i].cells, cudaMemcpyDeviceToHost, ctx->copy));
  }
  CK(cudaEventRecord(ctx->out_done, ctx->copy));
  ctx->out_pending = true;
  return RHYME_GPU_OK;
}

extern "C" int rhyme_gpu_output_wait(rhyme_gpu_ctx* ctx) {
  if (!ctx) return RHYME_GPU_EINVAL;
  if (!ctx->out_pending) return RHYME_GPU_OK;
  int rc = wait_event(ctx, ctx->out_done);
  if (rc == RHYME_GPU_OK) ctx->out_pending = false;
  return rc;
}

// ---- conservation totals and sanity checks ---------------------------------

extern "C" int rhyme_gpu_box_totals(rhyme_gpu_ctx* ctx, int handle, double totals[2]) {
  if (!ctx || !totals) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  const int nb = 152 * 2;
  void* parts = nullptr;
  double* out = nullptr;
  CK(cudaMallocAsync(&parts, 2 * nb * 2 * sizeof(double), ctx->stream));
  CK(cudaMallocAsync((void**)&out, 2 * sizeof(double), ctx->stream));
  cudaError_t e = launch_totals(ctx->params.ndim, b->state[b->cur], b->g.field, parts, nb, out, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctx->pinned_dt, out, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaFreeAsync(parts, ctx->stream);
  cudaFreeAsync(out, ctx->stream);
  if (e != cudaSuccess) return fail(ctx, RHYME_GPU_ECUDA, "totals: %s", cudaGetErrorString(e));
  int rc = wait_stream(ctx);
  if (rc != RHYME_GPU_OK) return rc;
  totals[0] = ctx->pinned_dt[0];
  totals[1] = ctx->pinned_dt[1];
  return RHYME_GPU_OK;
}

extern "C" int rhyme_gpu_sanity_check(rhyme_gpu_ctx* ctx, int handle, rhyme_gpu_sanity_report* rep) {
  if (!ctx || !rep) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  const int D = ctx->params.ndim;
  SanityRanges R;
  for (int p = 0; p < SC_COUNT; ++p) {
    R.range[p][0] = rep->prop[p].range[0];
    R.range[p][1] = rep->prop[p].range[1];
    R.enabled[p] = rep->prop[p].enabled ? 1 : 0;
  }
  if (D < 2) R.enabled[SC_VY] = 0;
  if (D < 3) R.enabled[SC_VZ] = 0;
  const long long total = (long long)b->g.n[0] * b->g.n[1] * b->g.n[2];
  int nb = (int)std::min<long long>(152 * 2, (total + 255) / 256);
  if (nb < 1) nb = 1;
  SanityPartial* parts = nullptr;
  SanityPartial* out = nullptr;
  CK(cudaMallocAsync((void**)&parts, sizeof(SanityPartial) * nb, ctx->stream));
  CK(cudaMallocAsync((void**)&out, sizeof(SanityPartial), ctx->stream));
  SanityPartial host;
  cudaError_t e = launch_sanity(D, b->state[b->cur], b->g, b->dp.G, R, parts, nb, out, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&host, out, sizeof(SanityPartial), cudaMemcpyDeviceToHost, ctx->stream);
  cudaFreeAsync(parts, ctx->stream);
  cudaFreeAsync(out, ctx->stream);
  if (e != cudaSuccess) return fail(ctx, RHYME_GPU_ECUDA, "sanity check: %s", cudaGetErrorString(e));
  int rc = wait_stream(ctx);
  if (rc != RHYME_GPU_OK) return rc;
  auto cell_of = [&](long long t, int* c) {
    c[0] = c[1] = c[2] = 0;
    if (t < 0) return;
    c[0] = (int)(t % b->g.n[0]) + 1;
    const long long q = t / b->g.n[0];
    if (D > 1) c[1] = (int)(q % b->g.n[1]) + 1;
    if (D > 2) c[2] = (int)(q / b->g.n[1]) + 1;
  };
  for (int p = 0; p < SC_COUNT; ++p) {
    rhyme_gpu_sanity_property& o = rep->prop[p];
    o.nbelow = host.nbelow[p];
    o.nabove = host.nabove[p];
    o.vbelow = host.vbelow[p];
    o.vbelow_prev = host.pbelow[p];
    o.vabove = host.vabove[p];
    o.vabove_prev = host.pabove[p];
    cell_of(host.ibelow[p], o.cbelow);
    cell_of(host.iabove[p], o.cabove);
  }
  for (int c = 0; c < 5; ++c) rep->nan[c] = (c < D + 2) ? host.nan[c] : 0;
  rep->rho_min = host.rho_min;
  rep->e_tot_min = host.e_min;
  cell_of(host.irho_min, rep->rho_min_at);
  cell_of(host.ie_min, rep->e_tot_min_at);
  return RHYME_GPU_OK;
}

// ---- initial conditions painted on the device -------------------------------

namespace {

// Public shape -> device shape for one box: primitive vectors packed as
// (rho, v_1..v_NDIM, p); sharp-cuboid bounds as
// rhyme_drawing_sharp_cuboid.f90:44-53 computes them (level 0).
int make_paint_shapes(rhyme_gpu_ctx* ctx, const Box* b, const int* le, const rhyme_gpu_shape* in, int n,
                      std::vector<PaintShape>* out) {
  const int D = ctx->params.ndim;
  out->resize(n);
  for (int i = 0; i < n; ++i) {
    const rhyme_gpu_shape& s = in[i];
    PaintShape& p = (*out)[i];
    memset(&p, 0, sizeof(p));
    if (s.type < RHYME_GPU_DRAW_CANVAS || s.type > RHYME_GPU_DRAW_SYMMETRIC_DECAYING)
      return fail(ctx, RHYME_GPU_EINVAL, "shape %d: unknown type %d", i, s.type);
    if (s.axis < 0 || s.axis >= D) return fail(ctx, RHYME_GPU_EINVAL, "shape %d: axis %d", i, s.axis);
    if (s.type == RHYME_GPU_DRAW_SMOOTHED_SLAB && D < 2)
      return fail(ctx, RHYME_GPU_EINVAL, "shape %d: a smoothed slab needs NDIM > 1", i);
    if (s.type == RHYME_GPU_DRAW_SYMMETRIC_DECAYING && (D < 2 || !(s.sigma > 0.0)))
      return fail(ctx, RHYME_GPU_EINVAL, "shape %d: symmetric decaying needs NDIM > 1 and sigma > 0", i);
    if (s.type == RHYME_GPU_DRAW_HARMONIC && !(s.wavelength != 0.0))
      return fail(ctx, RHYME_GPU_EINVAL, "shape %d: harmonic wavelength 0", i);
    p.type = s.type;
    p.axis = s.axis;
    p.periodic = s.periodic ? 1 : 0;
    p.keep_outside = s.keep_outside ? 1 : 0;
    auto pack = [&](const double* w5, double* w) {
      w[0] = w5[0];
      for (int a = 0; a < D; ++a) w[1 + a] = w5[1 + a];
      w[D + 1] = w5[4];
    };
    pack(s.prim[0], p.prim[0]);
    pack(s.prim[1], p.prim[1]);
    pack(s.base, p.base);
    for (int a = 0; a < 3; ++a) p.origin[a] = s.origin[a];
    p.r = s.r;
    p.sigma = s.sigma;
    p.pos[0] = s.pos[0];
    p.pos[1] = s.pos[1];
    p.slab_sigma[0] = s.slab_sigma[0];
    p.slab_sigma[1] = s.slab_sigma[1];
    p.amplitude = s.amplitude;
    p.wavelength = s.wavelength;
    p.phase = s.phase;
    for (int a = 0; a < 3; ++a) {
      const int dims = b->g.n[a];
      int lb = s.left_corner[a] - le[a];
      lb = (lb < 1) ? 1 : lb;
      lb = (lb > dims) ? dims + 1 : lb;
      int ub = s.left_corner[a] + s.lengths[a] - le[a];
      ub = (ub < 1) ? 0 : ub;
      ub = (ub > dims) ? dims : ub;
      p.lb[a] = (a < D) ? lb : 1;
      p.ub[a] = (a < D) ? ub : 1;
    }
  }
  return RHYME_GPU_OK;
}

}  // namespace

extern "C" int rhyme_gpu_paint(rhyme_gpu_ctx* ctx, int handle, const int left_edge[3], const rhyme_gpu_shape* shapes,
                               int n) {
  if (!ctx || !left_edge || (n > 0 && !shapes) || n < 0) return fail(ctx, RHYME_GPU_EINVAL, "bad argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  if (n == 0) return RHYME_GPU_OK;
  std::vector<PaintShape> ps;
  int rc = make_paint_shapes(ctx, b, left_edge, shapes, n, &ps);
  if (rc != RHYME_GPU_OK) return rc;
  state_changed(b);
  PaintShape* d = nullptr;
  CK(cudaMallocAsync((void**)&d, sizeof(PaintShape) * n, ctx->stream));
  cudaError_t e = cudaMemcpyAsync(d, ps.data(), sizeof(PaintShape) * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = launch_paint(ctx->params.ndim, d, n, b->dp.G, b->g, left_edge, b->state[b->cur],
                     ctx->mixed ? b->Uf[b->cur] : nullptr, ctx->stream);
  cudaFreeAsync(d, ctx->stream);
  if (e != cudaSuccess) return fail(ctx, RHYME_GPU_ECUDA, "paint: %s", cudaGetErrorString(e));
  return RHYME_GPU_OK;
}

extern "C" int rhyme_gpu_sweep_plan(rhyme_gpu_ctx* ctx, int handle, const double dx[3], int tile_cells[3],
                                    int tile_pencils[3]) {
  if (!ctx || !dx || !tile_cells || !tile_pencils) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  for (int a = 0; a < 3; ++a) tile_cells[a] = tile_pencils[a] = 0;
  if (!ctx->mixed) return RHYME_GPU_OK;
  int rc = box_plan(ctx, b, make_dx(ctx->params.ndim, dx));
  if (rc != RHYME_GPU_OK) return rc;
  for (int a = 0; a < ctx->params.ndim; ++a) sweep_shape(ctx->params.ndim, b->plan.shape[a], &tile_cells[a], &tile_pencils[a]);
  return RHYME_GPU_OK;
}

extern "C" int rhyme_gpu_fallback_count(rhyme_gpu_ctx* ctx, int handle, long long* count) {
  if (!ctx || !count) return fail(ctx, RHYME_GPU_EINVAL, "null argument");
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  int* st = (int*)(ctx->pinned_dt + 2);
  CK(cudaMemcpyAsync(st, b->fb_count, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemsetAsync(b->fb_count, 0, sizeof(int), ctx->stream));
  int rc = wait_stream(ctx);
  if (rc != RHYME_GPU_OK) return rc;
  *count = *st;
  return RHYME_GPU_OK;
}

// ---------------------------------------------------------------------------
// Per-box parameters and batches of boxes
// ---------------------------------------------------------------------------
extern "C" int rhyme_gpu_set_box_params(rhyme_gpu_ctx* ctx, int handle, const int bc[6], int limiter,
                                        double omega) {
  if (!ctx) return RHYME_GPU_EINVAL;
  Box* b = find_box(ctx, handle);
  if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handle);
  const int D = ctx->params.ndim;
  if (limiter < 1 || limiter > 4) return fail(ctx, RHYME_GPU_EINVAL, "unknown slope limiter %d", limiter);
  if (bc)
    for (int i = 0; i < 2 * D; ++i)
      if (bc[i] < 1 || bc[i] > 5) return fail(ctx, RHYME_GPU_EINVAL, "unknown boundary type %d", bc[i]);
  if (bc)
    for (int i = 0; i < 2 * D; ++i) b->dp.bc[i] = bc[i];
  b->dp.limiter = limiter;
  b->dp.omega = omega;
  b->mp.limiter = limiter;
  b->mp.omega = (float)omega;
  b->mp.omega64 = omega;
  b->graph_valid = false;
  return RHYME_GPU_OK;
}

struct rhyme_gpu_batch {
  rhyme_gpu_ctx* ctx = nullptr;
  std::vector<int> handles;
  std::vector<int> base_cur;  // box parity when the tables were built
  int k = 0;                  // steps taken since (mod 2)
  BoxDesc* table[2] = {nullptr, nullptr};
  WorkItem* items = nullptr;
  int* heads = nullptr;
  BatchLists L{};
  FallbackQueue q{};
  int* qblock = nullptr;  // n, status, total
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int runs = 0;  // batch_run calls since the tables were built
};

namespace {

void batch_free(rhyme_gpu_batch* B) {
  cudaStream_t st = B->ctx->stream;
  for (int p = 0; p < 2; ++p) {
    if (B->graph[p]) cudaGraphExecDestroy(B->graph[p]);
    B->graph[p] = nullptr;
    if (B->table[p]) cudaFreeAsync(B->table[p], st);
    B->table[p] = nullptr;
  }
  if (B->items) cudaFreeAsync(B->items, st);
  if (B->heads) cudaFreeAsync(B->heads, st);
  if (B->q.e) cudaFreeAsync(B->q.e, st);
  if (B->qblock) cudaFreeAsync(B->qblock, st);
  B->items = nullptr;
  B->heads = nullptr;
  B->q.e = nullptr;
  B->qblock = nullptr;
}

// Builds the box tables (both parities), the work-item lists and the
// per-parity step graphs.
int batch_build(rhyme_gpu_batch* B) {
  rhyme_gpu_ctx* ctx = B->ctx;
  const int D = ctx->params.ndim;
  const int n = (int)B->handles.size();
  batch_free(B);
  B->base_cur.resize(n);
  B->k = 0;
  B->runs = 0;
  // order: largest boxes first (the queues hand them out first)
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  auto cells_of = [&](int i) {
    const Box* b = ctx->boxes[B->handles[i]];
    return (long long)b->g.n[0] * b->g.n[1] * b->g.n[2];
  };
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return cells_of(a) > cells_of(c); });

  std::vector<BoxDesc> tab[2];
  tab[0].resize(n);
  tab[1].resize(n);
  std::vector<WorkItem> cfl, ghost, faces, flux, update, sweep[3][kSweepShapes];
  long long qcap = 0;
  for (int i = 0; i < n; ++i) {
    Box* b = ctx->boxes[B->handles[i]];
    int rc = box_plan(ctx, b, b->dx);
    if (rc != RHYME_GPU_OK) return rc;
    B->base_cur[i] = b->cur;
    const long long cells = (long long)b->g.n[0] * b->g.n[1] * b->g.n[2];
    qcap += D * cells / 16;
    for (int p = 0; p < 2; ++p) {
      BoxDesc& d = tab[p][i];
      memset(&d, 0, sizeof(d));
      const int c = b->cur ^ p;
      d.U = b->state[c];
      d.V = b->state[1 - c];
      d.Uf = b->Uf[c];
      d.acc = b->acc;
      d.faces = b->s.faces;
      d.fluxes = b->s.fluxes;
      d.ctl = b->s.dt;
      d.g = b->g;
      d.dx = b->dx;
      d.omega = b->dp.omega;
      d.omega_f = (float)b->dp.omega;
      d.limiter = b->dp.limiter;
      d.solver_type = b->dp.solver_type;
      for (int f = 0; f < 6; ++f) {
        d.bc[f] = b->dp.bc[f];
        for (int cc = 0; cc < 5; ++cc) d.inflow[f][cc] = b->dp.inflow[f][cc];
      }
      d.cfl_items = (int)((cells + kBatchChunk - 1) / kBatchChunk);
    }
  }
  for (int oi = 0; oi < n; ++oi) {
    const int i = order[oi];
    const Box* b = ctx->boxes[B->handles[i]];
    const Geom& g = b->g;
    const long long cells = (long long)g.n[0] * g.n[1] * g.n[2];
    for (long long c = 0; c * kBatchChunk < cells; ++c) cfl.push_back({i, 0, c});
    long long lines = 0;
    for (int a = 0; a < D; ++a) {
      long long t = D + 2;
      for (int o = 0; o < D; ++o)
        if (o != a) t *= g.n[o];
      lines += t;
    }
    for (long long c = 0; c * kBatchChunk < lines; ++c) ghost.push_back({i, 0, c});
    if (ctx->mixed) {
      for (int a = 0; a < D; ++a) {
        const int k = b->plan.shape[a];
        const long long nt = sweep_tile_count(D, a, k, g.n);
        for (long long t = 0; t < nt; ++t) sweep[a][k].push_back({i, a, t});
      }
    } else {
      for (int a = 0; a < D; ++a) {
        long long fc = 1, ic = 1;
        for (int o = 0; o < 3; ++o) {
          fc *= (o == a) ? g.n[o] + 2 : g.n[o];
          ic *= (o == a) ? g.n[o] + 1 : g.n[o];
        }
        for (long long c = 0; c * kBatchFluxChunk < fc; ++c) faces.push_back({i, a, c});
        for (long long c = 0; c * kBatchFluxChunk < ic; ++c) flux.push_back({i, a, c});
      }
      for (long long c = 0; c * kBatchChunk < cells; ++c) update.push_back({i, 0, c});
    }
  }
  std::vector<WorkItem> all;
  constexpr int kLists = 5 + 3 * kSweepShapes;
  size_t off[kLists];
  std::vector<WorkItem>* lists[kLists] = {&cfl, &ghost, &faces, &flux, &update};
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < kSweepShapes; ++k) lists[5 + kSweepShapes * a + k] = &sweep[a][k];
  for (int k = 0; k < kLists; ++k) {
    off[k] = all.size();
    all.insert(all.end(), lists[k]->begin(), lists[k]->end());
  }
  for (int p = 0; p < 2; ++p) {
    CK(cudaMallocAsync((void**)&B->table[p], sizeof(BoxDesc) * std::max(n, 1), ctx->stream));
    CK(cudaMemcpyAsync(B->table[p], tab[p].data(), sizeof(BoxDesc) * n, cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(cudaMallocAsync((void**)&B->items, sizeof(WorkItem) * std::max<size_t>(all.size(), 1), ctx->stream));
  CK(cudaMemcpyAsync(B->items, all.data(), sizeof(WorkItem) * all.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMallocAsync((void**)&B->heads, kBatchHeads * sizeof(int), ctx->stream));
  CK(cudaMallocAsync((void**)&B->qblock, 16 * sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(B->qblock, 0, 16 * sizeof(int), ctx->stream));
  B->q.cap = 0;
  if (ctx->mixed) {
    B->q.cap = (int)std::min<long long>(std::max<long long>(65536, qcap), 1LL << 30);
    CK(cudaMallocAsync((void**)&B->q.e, sizeof(FallbackEntry) * (size_t)B->q.cap, ctx->stream));
  }
  B->q.n = B->qblock + 0;
  B->q.status = B->qblock + 1;
  B->q.total = B->qblock + 2;
  BatchLists& L = B->L;
  L.cfl = B->items + off[0];
  L.ghost = B->items + off[1];
  L.faces = B->items + off[2];
  L.flux = B->items + off[3];
  L.update = B->items + off[4];
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < kSweepShapes; ++k) {
      L.sweep[a][k] = B->items + off[5 + kSweepShapes * a + k];
      L.n_sweep[a][k] = (int)sweep[a][k].size();
    }
  L.n_cfl = (int)cfl.size();
  L.n_ghost = (int)ghost.size();
  L.n_faces = (int)faces.size();
  L.n_flux = (int)flux.size();
  L.n_update = (int)update.size();
  L.heads = B->heads;
  return RHYME_GPU_OK;
}

// One step per parity captured in a CUDA graph (on the first run of several
// steps; short runs, as in a serving loop whose batch changes every few
// steps, launch directly).
int batch_capture(rhyme_gpu_batch* B) {
  rhyme_gpu_ctx* ctx = B->ctx;
  for (int p = 0; p < 2; ++p) {
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_batch_step(ctx->dp, ctx->mp, ctx->mixed, ctx->params.ndim, B->table[p], B->L, B->q,
                                      ctx->stream);
    cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (e2 == cudaSuccess) cudaGraphDestroy(graph);
      return fail(ctx, RHYME_GPU_ECUDA, "batch graph capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    cudaError_t e3 = cudaGraphInstantiate(&B->graph[p], graph, 0);
    cudaGraphDestroy(graph);
    if (e3 != cudaSuccess) return fail(ctx, RHYME_GPU_ECUDA, "batch graph instantiate: %s", cudaGetErrorString(e3));
  }
  return RHYME_GPU_OK;
}

}  // namespace

extern "C" int rhyme_gpu_batch_create(rhyme_gpu_ctx* ctx, const int* handles, const double* dx, int n,
                                      rhyme_gpu_batch** out) {
  if (!ctx || !handles || !dx || !out || n < 1) return fail(ctx, RHYME_GPU_EINVAL, "bad argument");
  *out = nullptr;
  const int D = ctx->params.ndim;
  for (int i = 0; i < n; ++i) {
    Box* b = find_box(ctx, handles[i]);
    if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "unknown box handle %d", handles[i]);
    for (int j = 0; j < i; ++j)
      if (handles[j] == handles[i]) return fail(ctx, RHYME_GPU_EINVAL, "box handle %d listed twice", handles[i]);
    for (int a = 0; a < D; ++a)
      if (!(dx[3 * i + a] > 0.0)) return fail(ctx, RHYME_GPU_EINVAL, "dx of box %d must be positive", handles[i]);
    b->dx = make_dx(D, dx + 3 * i);
  }
  rhyme_gpu_batch* B = new rhyme_gpu_batch();
  B->ctx = ctx;
  B->handles.assign(handles, handles + n);
  int rc = batch_build(B);
  if (rc != RHYME_GPU_OK) {
    batch_free(B);
    delete B;
    return rc;
  }
  *out = B;
  return RHYME_GPU_OK;
}

extern "C" int rhyme_gpu_batch_run(rhyme_gpu_batch* B, int nsteps) {
  if (!B) return RHYME_GPU_EINVAL;
  rhyme_gpu_ctx* ctx = B->ctx;
  if (nsteps < 0) return fail(ctx, RHYME_GPU_EINVAL, "nsteps must be >= 0");
  // rebuild if a box was stepped on its own since the tables were built
  for (size_t i = 0; i < B->handles.size(); ++i) {
    Box* b = find_box(ctx, B->handles[i]);
    if (!b) return fail(ctx, RHYME_GPU_ENOTFOUND, "box %d of the batch was unregistered", B->handles[i]);
    if (b->cur != (B->base_cur[i] ^ B->k)) {
      int rc = batch_build(B);
      if (rc != RHYME_GPU_OK) return rc;
      break;
    }
  }
  // a CUDA graph per parity once the batch runs several steps, in one call
  // or over repeated calls (a server stepping a stable set of requests)
  if ((nsteps >= 4 || B->runs >= 2) && nsteps > 0 && !B->graph[0]) {
    int rc = batch_capture(B);
    if (rc != RHYME_GPU_OK) return rc;
  }
  B->runs++;
  for (int s = 0; s < nsteps; ++s) {
    if (B->graph[0])
      CK(cudaGraphLaunch(B->graph[B->k], ctx->stream));
    else
      CK(launch_batch_step(ctx->dp, ctx->mp, ctx->mixed, ctx->params.ndim, B->table[B->k], B->L, B->q,
                           ctx->stream));
    B->k ^= 1;
  }
  for (size_t i = 0; i < B->handles.size(); ++i) {
    Box* b = ctx->boxes[B->handles[i]];
    b->cur = B->base_cur[i] ^ B->k;
    if (nsteps > 0) state_changed(b);
  }
  return RHYME_GPU_OK;
}

extern "C" int rhyme_gpu_batch_dt(rhyme_gpu_batch* B, double* dts) {
  if (!B || !dts) return RHYME_GPU_EINVAL;
  rhyme_gpu_ctx* ctx = B->ctx;
  for (size_t i = 0; i < B->handles.size(); ++i)
    CK(cudaMemcpyAsync(dts + i, ctx->boxes[B->handles[i]]->s.dt, sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
  return wait_stream(ctx);
}

extern "C" int rhyme_gpu_batch_destroy(rhyme_gpu_batch* B) {
  if (!B) return RHYME_GPU_OK;
  cudaStreamSynchronize(B->ctx->stream);
  batch_free(B);
  delete B;
  return RHYME_GPU_OK;
}

// ---------------------------------------------------------------------------
// Serving loop: continuous batching of hydro solves
// ---------------------------------------------------------------------------
namespace {

struct ServerReq {
  rhyme_gpu_request r{};
  int state = RHYME_GPU_REQ_PENDING;
  double t_submit = 0, t_admit = 0, t_done = 0;
  int steps_done = 0;
  int handle = -1;
  long long bytes = 0;
  long long cells = 0;
  void* staging = nullptr;
  size_t staging_bytes = 0;
  void* out_staging = nullptr;  // FP32 level output (r.output set)
  size_t out_staging_bytes = 0;
  std::vector<rhyme_gpu_shape> shapes;  // painted initial state (r.nshapes > 0)
  cudaEvent_t ev = nullptr;
};

}  // namespace

struct rhyme_gpu_server {
  rhyme_gpu_ctx* ctx[3] = {nullptr, nullptr, nullptr};
  long long budget = 0, used = 0;
  int max_active = 0;
  int n_active = 0;
  std::vector<ServerReq> reqs;
  std::vector<int> pending;  // FIFO (front at index pend_head)
  size_t pend_head = 0;
  std::vector<int> active[3];
  rhyme_gpu_batch* batch[3] = {nullptr, nullptr, nullptr};
  bool dirty[3] = {false, false, false};
  std::vector<int> draining;
  cudaStream_t copy = nullptr;
  std::chrono::steady_clock::time_point t0;
  std::vector<std::pair<size_t, void*>> pinned_free;  // page-locked staging pool
  std::string err;
  long long cell_updates = 0;
};

namespace {

double server_now(const rhyme_gpu_server* S) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - S->t0).count();
}

void* pinned_get(rhyme_gpu_server* S, size_t bytes, size_t* got) {
  size_t best = (size_t)-1, bi = 0;
  for (size_t i = 0; i < S->pinned_free.size(); ++i)
    if (S->pinned_free[i].first >= bytes && S->pinned_free[i].first < best) {
      best = S->pinned_free[i].first;
      bi = i;
    }
  if (best != (size_t)-1 && best <= 4 * bytes + (1 << 20)) {
    void* p = S->pinned_free[bi].second;
    *got = best;
    S->pinned_free.erase(S->pinned_free.begin() + bi);
    return p;
  }
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  *got = bytes;
  return p;
}

void pinned_put(rhyme_gpu_server* S, void* p, size_t bytes) { S->pinned_free.push_back({bytes, p}); }

int server_fail(rhyme_gpu_server* S, int code, const char* msg) {
  S->err = msg;
  return code;
}

void server_drop_batch(rhyme_gpu_server* S, int k) {
  if (S->batch[k]) {
    batch_free(S->batch[k]);
    delete S->batch[k];
    S->batch[k] = nullptr;
  }
}

}  // namespace

extern "C" {

int rhyme_gpu_server_create(const rhyme_gpu_params* base, const double courant[3], long long hbm_budget_bytes,
                            int max_active, rhyme_gpu_server** out) {
  if (!base || !courant || !out || hbm_budget_bytes <= 0 || max_active < 1) return RHYME_GPU_EINVAL;
  *out = nullptr;
  rhyme_gpu_server* S = new rhyme_gpu_server();
  S->budget = hbm_budget_bytes;
  S->max_active = max_active;
  S->t0 = std::chrono::steady_clock::now();
  for (int k = 0; k < 3; ++k) {
    rhyme_gpu_params p = *base;
    p.ndim = k + 1;
    p.courant = courant[k];
    for (int i = 0; i < 6; ++i)
      if (p.bc[i] < 1 || p.bc[i] > 4) p.bc[i] = RHYME_GPU_OUTFLOW;
    int rc = rhyme_gpu_create(&S->ctx[k], &p);
    if (rc != RHYME_GPU_OK) {
      for (int j = 0; j < k; ++j) rhyme_gpu_destroy(S->ctx[j]);
      delete S;
      return rc;
    }
  }
  if (cudaStreamCreateWithFlags(&S->copy, cudaStreamNonBlocking) != cudaSuccess) {
    for (int k = 0; k < 3; ++k) rhyme_gpu_destroy(S->ctx[k]);
    delete S;
    return RHYME_GPU_ECUDA;
  }
  *out = S;
  return RHYME_GPU_OK;
}

const char* rhyme_gpu_server_last_error(const rhyme_gpu_server* S) { return S ? S->err.c_str() : ""; }

int rhyme_gpu_server_submit(rhyme_gpu_server* S, const rhyme_gpu_request* r, int* id) {
  if (!S || !r || !id || !r->cells) return RHYME_GPU_EINVAL;
  if (r->ndim < 1 || r->ndim > 3 || r->nsteps < 0) return server_fail(S, RHYME_GPU_EINVAL, "bad request");
  for (int a = 0; a < 3; ++a)
    if ((a < r->ndim && r->dims[a] < 1) || (a >= r->ndim && r->dims[a] != 1))
      return server_fail(S, RHYME_GPU_EINVAL, "bad request dims");
  if (r->nshapes < 0 || (r->nshapes > 0 && !r->shapes)) return server_fail(S, RHYME_GPU_EINVAL, "bad shape list");
  ServerReq q;
  q.r = *r;
  if (r->nshapes > 0) q.shapes.assign(r->shapes, r->shapes + r->nshapes);  // kept until admission
  q.r.shapes = nullptr;
  q.t_submit = server_now(S);
  q.bytes = box_device_bytes(r->ndim, S->ctx[0]->mixed, r->dims);
  q.cells = (long long)r->dims[0] * r->dims[1] * r->dims[2];
  if (q.bytes > S->budget) return server_fail(S, RHYME_GPU_ENOMEM, "request larger than the HBM budget");
  S->reqs.push_back(q);
  *id = (int)S->reqs.size() - 1;
  S->pending.push_back(*id);
  return RHYME_GPU_OK;
}

int rhyme_gpu_server_tick(rhyme_gpu_server* S, int* n_active, int* n_pending, int* n_draining) {
  if (!S) return RHYME_GPU_EINVAL;
  // 1. finished downloads: copy out of the staging buffer
  for (size_t i = 0; i < S->draining.size();) {
    ServerReq& q = S->reqs[S->draining[i]];
    cudaError_t e = cudaEventQuery(q.ev);
    if (e == cudaErrorNotReady) {
      ++i;
      continue;
    }
    if (e != cudaSuccess) return server_fail(S, RHYME_GPU_ECUDA, cudaGetErrorString(e));
    const int D = q.r.ndim;
    const Geom g = make_geom(D, q.r.dims);
    memcpy(q.r.cells, q.staging, (size_t)(D + 2) * g.field * sizeof(double));
    pinned_put(S, q.staging, q.staging_bytes);
    q.staging = nullptr;
    if (q.out_staging) {
      memcpy(q.r.output, q.out_staging, (size_t)(D + 2) * q.cells * sizeof(float));
      pinned_put(S, q.out_staging, q.out_staging_bytes);
      q.out_staging = nullptr;
    }
    cudaEventDestroy(q.ev);
    q.ev = nullptr;
    q.t_done = server_now(S);
    q.state = RHYME_GPU_REQ_DONE;
    S->used -= q.bytes;
    S->draining[i] = S->draining.back();
    S->draining.pop_back();
  }
  // 2. admission, first come first served, against the budget and the cap
  while (S->pend_head < S->pending.size()) {
    const int id = S->pending[S->pend_head];
    ServerReq& q = S->reqs[id];
    if (S->used + q.bytes > S->budget || S->n_active >= S->max_active) break;
    const int k = q.r.ndim - 1;
    rhyme_gpu_ctx* ctx = S->ctx[k];
    const Geom g = make_geom(q.r.ndim, q.r.dims);
    const size_t hb = (size_t)(q.r.ndim + 2) * g.field * sizeof(double);
    q.staging = pinned_get(S, hb, &q.staging_bytes);
    if (!q.staging) return server_fail(S, RHYME_GPU_ENOMEM, "pinned staging allocation failed");
    const bool painted = !q.shapes.empty();
    if (!painted) memcpy(q.staging, q.r.cells, hb);
    int h = -1;
    int rc = register_box_impl(ctx, 0, id, (double*)q.staging, q.r.dims, 2, q.r.ndim + 2, false, !painted, &h, true);
    if (rc != RHYME_GPU_OK) return server_fail(S, rc, ctx->err.c_str());
    if (painted) {  // initial state painted on the device from zero cells: no upload
      Box* nb = ctx->boxes[h];
      for (int i = 0; i < 2; ++i) {
        cudaError_t e = cudaMemsetAsync(nb->state[i], 0, nb->hydro_bytes, ctx->stream);
        if (e == cudaSuccess && nb->Uf[i]) e = cudaMemsetAsync(nb->Uf[i], 0, nb->hydro_bytes / 2, ctx->stream);
        if (e != cudaSuccess) return server_fail(S, RHYME_GPU_ECUDA, cudaGetErrorString(e));
      }
      const int le[3] = {1, 1, 1};
      rc = rhyme_gpu_paint(ctx, h, le, q.shapes.data(), (int)q.shapes.size());
      if (rc != RHYME_GPU_OK) return server_fail(S, rc, ctx->err.c_str());
    }
    rc = rhyme_gpu_set_box_params(ctx, h, q.r.bc, q.r.limiter, q.r.omega);
    if (rc != RHYME_GPU_OK) return server_fail(S, rc, ctx->err.c_str());
    ctx->boxes[h]->dx = make_dx(q.r.ndim, q.r.dx);
    q.handle = h;
    q.state = RHYME_GPU_REQ_ACTIVE;
    q.t_admit = server_now(S);
    S->used += q.bytes;
    S->n_active++;
    S->active[k].push_back(id);
    S->dirty[k] = true;
    S->pend_head++;
  }
  // 3. steps of every active request, one batch per dimensionality: as many
  // as the request nearest to completion still needs (its retirement frees
  // budget for the pending ones), at most kMaxTickSteps, so that arrivals
  // wait at most that many steps to be admitted
  constexpr int kMaxTickSteps = 8;
  int tick_steps = kMaxTickSteps;
  for (int k = 0; k < 3; ++k)
    for (int id : S->active[k]) tick_steps = std::min(tick_steps, S->reqs[id].r.nsteps - S->reqs[id].steps_done);
  tick_steps = std::max(tick_steps, 1);
  for (int k = 0; k < 3; ++k) {
    if (S->active[k].empty()) continue;
    rhyme_gpu_ctx* ctx = S->ctx[k];
    if (S->dirty[k] || !S->batch[k]) {
      server_drop_batch(S, k);
      std::vector<int> hs;
      std::vector<double> dxs;
      for (int id : S->active[k]) {
        hs.push_back(S->reqs[id].handle);
        for (int a = 0; a < 3; ++a) dxs.push_back(S->reqs[id].r.dx[a] > 0 ? S->reqs[id].r.dx[a] : 1.0);
      }
      int rc = rhyme_gpu_batch_create(ctx, hs.data(), dxs.data(), (int)hs.size(), &S->batch[k]);
      if (rc != RHYME_GPU_OK) return server_fail(S, rc, ctx->err.c_str());
      S->dirty[k] = false;
    }
    int rc = rhyme_gpu_batch_run(S->batch[k], tick_steps);
    if (rc != RHYME_GPU_OK) return server_fail(S, rc, ctx->err.c_str());
    for (int id : S->active[k]) {
      S->reqs[id].steps_done += tick_steps;
      S->cell_updates += S->reqs[id].cells * tick_steps;
    }
  }
  // 4. retire finished requests: download on the copy stream, free in order
  for (int k = 0; k < 3; ++k) {
    rhyme_gpu_ctx* ctx = S->ctx[k];
    for (size_t i = 0; i < S->active[k].size();) {
      const int id = S->active[k][i];
      ServerReq& q = S->reqs[id];
      if (q.steps_done < q.r.nsteps) {
        ++i;
        continue;
      }
      Box* b = ctx->boxes[q.handle];
      cudaEvent_t done_compute;
      if (cudaEventCreateWithFlags(&done_compute, cudaEventDisableTiming) != cudaSuccess)
        return server_fail(S, RHYME_GPU_ECUDA, "event");
      cudaEventRecord(done_compute, ctx->stream);
      cudaStreamWaitEvent(S->copy, done_compute, 0);
      cudaEventDestroy(done_compute);
      cudaMemcpyAsync(q.staging, b->state[b->cur], b->hydro_bytes, cudaMemcpyDeviceToHost, S->copy);
      if (q.r.output) {
        // one-box level output: packed on the compute stream, drained on the copy stream
        const int D = q.r.ndim;
        const size_t ob = (size_t)(D + 2) * q.cells * sizeof(float);
        q.out_staging = pinned_get(S, ob, &q.out_staging_bytes);
        if (!q.out_staging) return server_fail(S, RHYME_GPU_ENOMEM, "pinned staging allocation failed");
        PackDesc pd;
        pd.U = b->state[b->cur];
        pd.g = b->g;
        pd.cells = q.cells;
        pd.hydro_off = 0;
        pd.out_off = 0;
        PackDesc* d_pd = nullptr;
        float* d_out = nullptr;
        cudaError_t e = cudaMallocAsync((void**)&d_pd, sizeof(PackDesc), ctx->stream);
        if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_out, ob, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_pd, &pd, sizeof(PackDesc), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = launch_pack_level(d_pd, 1, (long long)(D + 2) * q.cells, D, d_out, ctx->stream);
        cudaEvent_t packed;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&packed, cudaEventDisableTiming);
        if (e == cudaSuccess) {
          cudaEventRecord(packed, ctx->stream);
          cudaStreamWaitEvent(S->copy, packed, 0);
          cudaEventDestroy(packed);
          e = cudaMemcpyAsync(q.out_staging, d_out, ob, cudaMemcpyDeviceToHost, S->copy);
        }
        if (d_pd) cudaFreeAsync(d_pd, S->copy);
        if (d_out) cudaFreeAsync(d_out, S->copy);
        if (e != cudaSuccess) return server_fail(S, RHYME_GPU_ECUDA, cudaGetErrorString(e));
      }
      cudaEventCreateWithFlags(&q.ev, cudaEventDisableTiming);
      cudaEventRecord(q.ev, S->copy);
      // the batch tables reference this box: drop the batch before freeing
      server_drop_batch(S, k);
      S->dirty[k] = true;
      destroy_box(b, S->copy);
      ctx->boxes[q.handle] = nullptr;
      q.state = RHYME_GPU_REQ_DRAINING;
      S->draining.push_back(id);
      S->n_active--;
      S->active[k][i] = S->active[k].back();
      S->active[k].pop_back();
    }
  }
  if (n_active) *n_active = S->n_active;
  if (n_pending) *n_pending = (int)(S->pending.size() - S->pend_head);
  if (n_draining) *n_draining = (int)S->draining.size();
  return RHYME_GPU_OK;
}

int rhyme_gpu_server_request(rhyme_gpu_server* S, int id, int* state, double times[3], int* steps_done) {
  if (!S || id < 0 || id >= (int)S->reqs.size()) return RHYME_GPU_EINVAL;
  const ServerReq& q = S->reqs[id];
  if (state) *state = q.state;
  if (times) {
    times[0] = q.t_submit;
    times[1] = q.t_admit;
    times[2] = q.t_done;
  }
  if (steps_done) *steps_done = q.steps_done;
  return RHYME_GPU_OK;
}

int rhyme_gpu_server_stats(rhyme_gpu_server* S, long long* cell_updates, long long* hbm_used) {
  if (!S) return RHYME_GPU_EINVAL;
  if (cell_updates) *cell_updates = S->cell_updates;
  if (hbm_used) *hbm_used = S->used;
  return RHYME_GPU_OK;
}

int rhyme_gpu_server_destroy(rhyme_gpu_server* S) {
  if (!S) return RHYME_GPU_OK;
  for (int k = 0; k < 3; ++k) {
    if (S->ctx[k]) cudaStreamSynchronize(S->ctx[k]->stream);
    server_drop_batch(S, k);
  }
  if (S->copy) cudaStreamSynchronize(S->copy);
  for (auto& q : S->reqs) {
    if (q.ev) cudaEventDestroy(q.ev);
    if (q.staging) cudaFreeHost(q.staging);
  }
  for (auto& f : S->pinned_free) cudaFreeHost(f.second);
  for (int k = 0; k < 3; ++k) rhyme_gpu_destroy(S->ctx[k]);
  if (S->copy) cudaStreamDestroy(S->copy);
  delete S;
  return RHYME_GPU_OK;
}

}  // extern "C"
