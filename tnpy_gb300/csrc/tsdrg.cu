// tSDRG on the device: batched two-block Hamiltonians and spectrum projectors.
//
// Reference: TreeTensorNetworkSDRG.block_hamiltonian (tnpy/tsdrg.py:607-631) and
// spectrum_projector (:633-669). MPO tensors of the coarse-grained chain are kept in the
// uniform layout W[dl][dr][m][m] (ket, bra); the left end has dl = 1 and the right end
// dr = 1, so the reference's isel(row 0) / isel(column -1) on four-index tensors is
// W1[0] / W2[:, dr-1] for every tensor.
//
// Every entry point takes a batch of independent items (different blocks of one chain, or
// blocks of many disorder realisations) with per-item sizes ("uneven" batches).
#include <cuda_runtime.h>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

// H[(k1 k2),(b1 b2)] = sum_w W1[0,w,k1,b1] W2[w,dr2-1,k2,b2]
// meta[4b..4b+3] = m1, m2, dl1 (unused), dr2; one CTA per item, grid-stride over entries
__global__ void block_h_kernel(const double* const* __restrict__ w1, const double* const* __restrict__ w2,
                               const int* __restrict__ meta, int D, double* __restrict__ h,
                               const int64_t* __restrict__ h_off) {
  const int b = blockIdx.x;
  const int m1 = meta[4 * b], m2 = meta[4 * b + 1], dr2 = meta[4 * b + 3];
  const int m = m1 * m2;
  const double* A = w1[b];  // row 0 of [dl1][D][m1][m1]
  const double* B = w2[b];  // [D][dr2][m2][m2]
  double* H = h + h_off[b];
  for (int e = blockIdx.y * blockDim.x + threadIdx.x; e < m * m; e += gridDim.y * blockDim.x) {
    const int row = e / m, col = e % m;
    const int k1 = row / m2, k2 = row % m2, b1 = col / m2, b2 = col % m2;
    double acc = 0.0;
    for (int w = 0; w < D; ++w) {
      const double a = A[(size_t(w) * m1 + k1) * m1 + b1];
      if (a != 0.0) acc = fma(a, B[((size_t(w) * dr2 + dr2 - 1) * m2 + k2) * m2 + b2], acc);
    }
    H[e] = acc;
  }
}

// W'[l,r,i,j] = V_i^T (sum_w A_lw (x) B_wr) V_j with A_lw = W1[l,w] (m1 x m1), B_wr = W2[w,r]
// (m2 x m2) and V_i the i-th kept eigenvector viewed as an m1 x m2 matrix:
// (A (x) B) vec(X) = vec(A X B^T). One CTA per (item, l, r); A, B and one column of V in
// shared memory. meta5[5b..5b+4] = m1, m2, dl1, dr2, k.
constexpr int PMAX = 32;  // m1, m2 <= 32 (the kept dimension of a tree node)

__global__ void __launch_bounds__(256) project_kernel(const double* const* __restrict__ w1,
                                                      const double* const* __restrict__ w2,
                                                      const double* const* __restrict__ v, const int* __restrict__ meta,
                                                      int D, double* const* __restrict__ out) {
  const int b = blockIdx.x;
  const int m1 = meta[5 * b], m2 = meta[5 * b + 1], dl1 = meta[5 * b + 2], dr2 = meta[5 * b + 3], k = meta[5 * b + 4];
  const int ldv = k;  // V_b is a contiguous [m1*m2][k] matrix
  const int l = blockIdx.y / D, r = blockIdx.y % D;
  if (l >= dl1 || r >= dr2) return;
  __shared__ double As[PMAX][PMAX + 1], Bs[PMAX][PMAX + 1], X[PMAX][PMAX + 1], T[PMAX][PMAX + 1];
  __shared__ double Y[PMAX * PMAX];
  const double* W1 = w1[b];
  const double* W2 = w2[b];
  const double* V = v[b];
  double* O = out[b] + (size_t(l) * dr2 + r) * k * k;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int m = m1 * m2;
  for (int j = 0; j < k; ++j) {
    // Yj = sum_w A_lw X_j B_wr^T, X_j = V[:, j] as m1 x m2
    for (int e = tid; e < m; e += nt) X[e / m2][e % m2] = V[size_t(e) * ldv + j];
    for (int e = tid; e < m; e += nt) Y[e] = 0.0;
    __syncthreads();
    for (int w = 0; w < D; ++w) {
      for (int e = tid; e < m1 * m1; e += nt) As[e / m1][e % m1] = W1[((size_t(l) * D + w) * m1) * m1 + e];
      for (int e = tid; e < m2 * m2; e += nt) Bs[e / m2][e % m2] = W2[((size_t(w) * dr2 + r) * m2) * m2 + e];
      __syncthreads();
      // T = A X  (m1 x m2)
      for (int e = tid; e < m; e += nt) {
        const int i1 = e / m2, i2 = e % m2;
        double s = 0.0;
        for (int q = 0; q < m1; ++q) s = fma(As[i1][q], X[q][i2], s);
        T[i1][i2] = s;
      }
      __syncthreads();
      // Y += T B^T
      for (int e = tid; e < m; e += nt) {
        const int i1 = e / m2, i2 = e % m2;
        double s = 0.0;
        for (int q = 0; q < m2; ++q) s = fma(T[i1][q], Bs[i2][q], s);
        Y[e] += s;
      }
      __syncthreads();
    }
    // O[i][j] = V_i . Y_j for every i (thread-strided over i)
    for (int i = tid; i < k; i += nt) {
      double s = 0.0;
      for (int e = 0; e < m; ++e) s = fma(V[size_t(e) * ldv + i], Y[e], s);
      O[size_t(i) * k + j] = s;
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace tnx

using namespace tnx;

extern "C" {

int tnx_tsdrg_block_hamiltonian(const double* const* w1, const double* const* w2, const int* meta, int D, double* h,
                                const int64_t* h_off, int batch, int max_m, void* stream) {
  TNX_CHECK_ARG(w1 && w2 && meta && h && h_off, "null pointer");
  TNX_CHECK_ARG(batch >= 0 && D > 0 && max_m > 0, "bad batch / D / max_m");
  if (batch == 0) return TNX_OK;
  TNX_CHECK_SHAPE(max_m <= 4096, "block dimension > 4096");
  const int m2 = max_m * max_m;
  int gy = (m2 + 255) / 256;
  if (gy > 64) gy = 64;
  block_h_kernel<<<dim3(batch, gy), 256, 0, as_stream(stream)>>>(w1, w2, meta, D, h, h_off);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

int tnx_tsdrg_project(const double* const* w1, const double* const* w2, const double* const* v, const int* meta, int D,
                      double* const* out, int batch, int max_m1, int max_m2, int max_k, void* stream) {
  TNX_CHECK_ARG(w1 && w2 && v && meta && out, "null pointer");
  TNX_CHECK_ARG(batch >= 0 && D > 0, "bad batch / D");
  if (batch == 0) return TNX_OK;
  TNX_CHECK_SHAPE(max_m1 <= PMAX && max_m2 <= PMAX && max_k <= PMAX,
                  "tsdrg projector supports node dimensions <= %d (got %d, %d, k=%d)", PMAX, max_m1, max_m2, max_k);
  project_kernel<<<dim3(batch, D * D), 256, 0, as_stream(stream)>>>(w1, w2, v, meta, D, out);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

}  // extern "C"
