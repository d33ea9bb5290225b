// Exact diagonalisation on the device: the dense Hamiltonian of an MPO and its full spectrum.
//
// Replaces FullHamiltonian (tnpy/operators.py:119-166) and the np.linalg.eigh of
// ExactDiagonalization (tnpy/exact_diagonalization.py:10-60). Element (K, B) of H, with K and B
// the ket and bra basis strings (site 0 the most significant digit), is the MPO's transfer
// product e_0^T W_0[:, :, k_0, b_0] ... W_{n-1}[:, :, k_{n-1}, b_{n-1}] e_0: one thread per
// element carries the D-vector through the n sites. The spectrum comes from the one-sided Jacobi
// SVD (svd_jacobi.cu) of the shifted matrix H + c I, c = max row sum |H| + 1, which is symmetric
// positive definite: its singular values are the eigenvalues plus c and its left singular
// vectors the eigenvectors.
#include <cuda_runtime.h>

#include <cmath>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

constexpr int ED_DMAX = 32;

// W: [n][D][D][d][d] (the uniform MPO padded to bond D: site 0 uses row 0, site n-1 column 0)
__global__ void full_h_kernel(const double* __restrict__ W, int n, int D, int d, int64_t dim,
                              double* __restrict__ H) {
  const int64_t total = dim * dim;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t K = e / dim, B = e % dim;
    double v[ED_DMAX], w[ED_DMAX];
    for (int a = 0; a < D; ++a) v[a] = a == 0 ? 1.0 : 0.0;
    int64_t place = dim / d;  // weight of site s's digit, site 0 the most significant
    for (int s = 0; s < n; ++s) {
      const int k = int((K / place) % d), b = int((B / place) % d);
      const double* Ws = W + int64_t(s) * D * D * d * d;
      for (int c = 0; c < D; ++c) w[c] = 0.0;
      for (int a = 0; a < D; ++a) {
        const double va = v[a];
        if (va == 0.0) continue;
        for (int c = 0; c < D; ++c) w[c] = fma(va, Ws[((a * D + c) * d + k) * d + b], w[c]);
      }
      for (int c = 0; c < D; ++c) v[c] = w[c];
      if (place > 1) place /= d;
    }
    H[e] = v[0];
  }
}

// shift[0] = max_i sum_j |H_ij| + 1 (one block, grid-stride over rows)
__global__ void row_bound_kernel(const double* __restrict__ H, int64_t dim, double* __restrict__ shift) {
  __shared__ double red[32];
  double m = 0.0;
  for (int64_t i = threadIdx.x; i < dim; i += blockDim.x) {
    double s = 0.0;
    for (int64_t j = 0; j < dim; ++j) s += fabs(H[i * dim + j]);
    m = fmax(m, s);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) t = fmax(t, red[i]);
    shift[0] = t + 1.0;
  }
}

__global__ void add_diag_kernel(double* __restrict__ H, int64_t dim, const double* __restrict__ shift, double sign) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < dim; i += int64_t(gridDim.x) * blockDim.x)
    H[i * dim + i] += sign * shift[0];
}

}  // namespace
}  // namespace tnx

using namespace tnx;

extern "C" {

int tnx_full_hamiltonian(const double* W, int n, int D, int d, double* H, void* stream) {
  TNX_CHECK_ARG(W && H, "null pointer");
  TNX_CHECK_ARG(n >= 1 && D >= 1 && d >= 2, "non-positive size");
  TNX_CHECK_SHAPE(D <= ED_DMAX, "MPO bond %d > %d", D, ED_DMAX);
  const double dimf = std::pow(double(d), double(n));
  TNX_CHECK_SHAPE(dimf <= 65536.0, "d^n = %.0f exceeds the dense limit 65536", dimf);
  const int64_t dim = int64_t(dimf + 0.5);
  full_h_kernel<<<152 * 8, 256, 0, as_stream(stream)>>>(W, n, D, d, dim, H);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

int tnx_shift_to_spd(double* H, int64_t dim, double* shift, int undo, void* stream) {
  TNX_CHECK_ARG(H && shift && dim > 0, "null pointer or empty matrix");
  cudaStream_t st = as_stream(stream);
  if (!undo) {
    row_bound_kernel<<<1, 1024, 0, st>>>(H, dim, shift);
    TNX_LAUNCH_CHECK();
  }
  add_diag_kernel<<<unsigned((dim + 255) / 256), 256, 0, st>>>(H, dim, shift, undo ? -1.0 : 1.0);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

}  // extern "C"
