// kernels_output.cu -- device side of the Chombo output drain.
//
// rhyme_chombo_write_level_data.f90:36-70 builds a level's
// "data:datatype=0" dataset on the host: for each box in order, for each
// component, the interior cells in Fortran order converted to default real
// (FP32). The kernel below writes the hydro components of every listed box
// straight from device memory into a device buffer with that layout, so the
// level's output leaves the GPU as FP32 in one pass instead of as the FP64
// ghosted state.
#include "rgpu_internal.h"

namespace rgpu {

namespace {

// Element e of the flattened hydro data of all boxes: box by binary search
// on the prefix offsets, then component and cell.
__global__ void __launch_bounds__(256)
    pack_level_kernel(const PackDesc* __restrict__ D, int n, long long total, int ndim, float* __restrict__ out) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (D[mid].hydro_off <= e) lo = mid;
      else hi = mid - 1;
    }
    const PackDesc& d = D[lo];
    const long long r = e - d.hydro_off;
    const int c = (int)(r / d.cells);
    const long long cell = r - (long long)c * d.cells;
    const long long n0 = d.g.n[0], n1 = d.g.n[1];
    const int i = (int)(cell % n0) + 1;
    const long long q = cell / n0;
    const int j = (int)(q % n1) + 1;
    const int k = (int)(q / n1) + 1;
    out[d.out_off + r] = (float)d.U[(long long)c * d.g.field + d.g.at(ndim, i, j, k)];
  }
}

}  // namespace

cudaError_t launch_pack_level(const PackDesc* desc, int n, long long total, int ndim, float* out,
                              cudaStream_t st) {
  if (n <= 0 || total <= 0) return cudaSuccess;
  long long blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  pack_level_kernel<<<(int)blocks, 256, 0, st>>>(desc, n, total, ndim, out);
  return cudaGetLastError();
}

}  // namespace rgpu
