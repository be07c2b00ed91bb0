/*
 * The driver loop of src/main.f90:106-177 for one box, written in C99
 * against include/rhyme_gpu.h alone: a caller of the C-ABI that is neither
 * the Fortran shim nor Python. tests/test_abi.py compiles it as strict C99
 * and as C++ and links it against the library, which shows that the header
 * is plain C and that every call below resolves in librhyme_gpu.so.
 *
 * Run on a machine with a GPU, it steps a 1-D Sod tube of N cells (outflow
 * faces, van Leer, courant 0.8, diatomic gas) for NSTEPS steps and prints
 * the total mass before and after and the last dt; it exits non-zero on any
 * error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rhyme_gpu.h"

#define N 256
#define NSTEPS 50
#define GHOST 2
#define NCMP 3 /* rho, rho u, e_tot */

static int check(int rc, const rhyme_gpu_ctx* ctx, const char* what) {
  if (rc != RHYME_GPU_OK) {
    fprintf(stderr, "%s: %d (%s)\n", what, rc, ctx ? rhyme_gpu_last_error(ctx) : "");
    return 1;
  }
  return 0;
}

static double mass(const double* cells) {
  double m = 0.0;
  int i;
  for (i = GHOST; i < N + GHOST; ++i) m += cells[i];
  return m;
}

int main(void) {
  const int ext = N + 2 * GHOST;
  const double gamma = 7.0 / 5.0;
  double* cells = (double*)calloc((size_t)ext * NCMP, sizeof(double));
  rhyme_gpu_params p;
  rhyme_gpu_ctx* ctx = NULL;
  int dims[3] = {N, 1, 1};
  double dx[3] = {1.0 / N, 1.0, 1.0};
  double dt = 0.0, m0;
  int handle = -1, i, k, side;

  if (!cells) return 1;
  memset(&p, 0, sizeof p);
  /* Sod: (1, 0, 1) | (0.125, 0, 0.1); cells(i, comp) in Fortran order */
  for (i = GHOST; i < N + GHOST; ++i) {
    int left = i < GHOST + N / 2;
    cells[i] = left ? 1.0 : 0.125;
    cells[ext + i] = 0.0;
    cells[2 * ext + i] = (left ? 1.0 : 0.1) / (gamma - 1.0);
  }
  m0 = mass(cells);

  p.ndim = 1;
  p.limiter = RHYME_GPU_VAN_LEER;
  p.n_iteration = 100;
  p.solver_type = RHYME_GPU_MEMORY_INTENSIVE;
  for (side = 0; side < 6; ++side) p.bc[side] = RHYME_GPU_OUTFLOW;
  p.precision = RHYME_GPU_FP64;
  p.gamma = gamma;
  p.kb_amu = 1.380649e-23 / 1.66053906660e-27;
  p.courant = 0.8;
  p.tolerance = 1e-6;

  if (rhyme_gpu_abi_version() != RHYME_GPU_ABI_VERSION) return 1;
  if (check(rhyme_gpu_create(&ctx, &p), ctx, "create")) return 1;
  if (check(rhyme_gpu_register_box(ctx, 0, 1, cells, dims, GHOST, NCMP, &handle), ctx, "register"))
    return 1;
  for (k = 0; k < NSTEPS; ++k) {
    if (check(rhyme_gpu_cfl_time_step(ctx, handle, dx, &dt), ctx, "cfl")) return 1;
    if (check(rhyme_gpu_set_boundaries(ctx, handle), ctx, "boundaries")) return 1;
    if (check(rhyme_gpu_mh_solve(ctx, handle, dx, dt), ctx, "solve")) return 1;
  }
  if (check(rhyme_gpu_sync_to_host(ctx, handle), ctx, "sync")) return 1;
  printf("mass %.17g -> %.17g, last dt %.17g\n", m0, mass(cells), dt);
  if (check(rhyme_gpu_unregister_box(ctx, handle), ctx, "unregister")) return 1;
  if (check(rhyme_gpu_destroy(ctx), NULL, "destroy")) return 1;
  free(cells);
  return 0;
}
