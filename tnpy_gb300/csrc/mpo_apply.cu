// One MPO tensor applied to one MPS tensor: the site tensors of O|psi> as an MPS of bond
// chi * D, used to restore psi = (H - eps) phi after shift-invert DMRG
// (ShiftInvertDMRG._restore_mps, tnpy/finite_dmrg.py:314-343):
//   out[(a, w), k, (c, v)] = sum_b W[w, v, k, b] A[a, b, c]
// with the fused bonds in (MPS bond, MPO bond) order, one thread per output element.
#include <cuda_runtime.h>

#include "tnx_internal.cuh"

namespace tnx {
namespace {
__global__ void mpo_apply_kernel(const double* __restrict__ A, const double* __restrict__ W, double* __restrict__ out,
                                 int64_t chi_l, int d, int64_t chi_r, int dl, int dr) {
  const int64_t total = chi_l * dl * d * chi_r * dr;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    int64_t r = e;
    const int v = int(r % dr);
    r /= dr;
    const int64_t c = r % chi_r;
    r /= chi_r;
    const int k = int(r % d);
    r /= d;
    const int w = int(r % dl);
    const int64_t a = r / dl;
    double acc = 0.0;
    for (int b = 0; b < d; ++b) acc = fma(W[((int64_t(w) * dr + v) * d + k) * d + b], A[(a * d + b) * chi_r + c], acc);
    out[e] = acc;
  }
}
}  // namespace
}  // namespace tnx

using namespace tnx;

extern "C" int tnx_mpo_apply_site(const double* A, const double* W, double* out, int64_t chi_l, int64_t d,
                                  int64_t chi_r, int64_t dl, int64_t dr, void* stream) {
  TNX_CHECK_ARG(A && W && out, "null pointer");
  TNX_CHECK_ARG(chi_l > 0 && d > 0 && chi_r > 0 && dl > 0 && dr > 0, "non-positive dimension");
  TNX_CHECK_SHAPE(d <= 64 && dl <= 1024 && dr <= 1024, "dimension too large");
  const int64_t total = chi_l * dl * d * chi_r * dr;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  mpo_apply_kernel<<<unsigned(blocks), 256, 0, as_stream(stream)>>>(A, W, out, chi_l, int(d), chi_r, int(dl),
                                                                     int(dr));
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}
