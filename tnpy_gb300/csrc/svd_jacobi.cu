// Singular value decomposition by one-sided (Hestenes) Jacobi in FP64, replacing
// np.linalg.svd in linalg.svd (tnpy/linalg.py:9-23) and the Schmidt values of the SVD gauge
// move (tnpy/matrix_product_state.py:200-223) where they are reported.
//
// The columns of a working copy C of A (m x n, m >= n) are rotated in pairs until every pair is
// orthogonal to working accuracy: for columns (p, q) with a = |c_p|^2, b = |c_q|^2, g = c_p.c_q,
// the plane rotation that zeroes g is applied to C and to V (V starts as the identity), so that
// C = A V keeps orthogonal columns at the end: sigma_j = |c_j|, u_j = c_j / sigma_j, A = U S V^T.
// The singular values come from the matrix itself, not from a Gram matrix A^T A, so a small
// sigma keeps an absolute error of ~eps * sigma_max instead of ~sqrt(eps) * sigma_max.
//
// Parallel order: the round-robin ("circle") tournament on ne = n rounded up to even columns
// (a zero column pads odd n): each of the ne - 1 rounds rotates ne / 2 disjoint pairs, one CTA
// per pair; a sweep is ne - 1 launches, and sweeps repeat until a sweep rotates no pair
// (|g| <= tol sqrt(a b), tol = sqrt(m) * 2^-52) or 40 sweeps pass. The host reads one counter
// per sweep. Working copies are column-major so that every column is contiguous.
#include <cuda_runtime.h>

#include <cmath>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

constexpr int JT = 256;
constexpr int kMaxSweeps = 40;

__global__ void jac_init_kernel(const double* __restrict__ A, int64_t m, int64_t n, int64_t ne,
                                double* __restrict__ C, double* __restrict__ V) {
  const int64_t total = m * ne;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t j = e / m, i = e - j * m;
    C[e] = j < n ? A[i * n + j] : 0.0;
  }
  if (V) {
    const int64_t tv = ne * ne;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < tv; e += int64_t(gridDim.x) * blockDim.x)
      V[e] = (e / ne == e % ne) ? 1.0 : 0.0;
  }
}

__device__ __forceinline__ void pair_of(int round, int k, int ne, int& p, int& q) {
  if (k == 0) {
    p = ne - 1;
    q = round;
  } else {
    p = (round + k) % (ne - 1);
    q = (round - k + (ne - 1)) % (ne - 1);
  }
}

__global__ void __launch_bounds__(JT) jac_round_kernel(double* __restrict__ C, int64_t m, double* __restrict__ V,
                                                      int ne, int round, double tol, int* __restrict__ rotated) {
  __shared__ double red[3][JT / 32];
  __shared__ double cs[2];
  int p, q;
  pair_of(round, blockIdx.x, ne, p, q);
  double* cp = C + int64_t(p) * m;
  double* cq = C + int64_t(q) * m;
  double a = 0.0, b = 0.0, g = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += JT) {
    const double x = cp[i], y = cq[i];
    a = fma(x, x, a);
    b = fma(y, y, b);
    g = fma(x, y, g);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    g += __shfl_xor_sync(0xffffffffu, g, o);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][w] = a;
    red[1][w] = b;
    red[2][w] = g;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a = b = g = 0.0;
    for (int i = 0; i < JT / 32; ++i) {
      a += red[0][i];
      b += red[1][i];
      g += red[2][i];
    }
    double c = 1.0, s = 0.0;
    if (a > 0.0 && b > 0.0 && fabs(g) > tol * sqrt(a) * sqrt(b)) {
      // t = tan(theta): the smaller root of t^2 + 2 zeta t - 1 = 0, zeta = (b - a) / (2 g)
      const double zeta = (b - a) / (2.0 * g);
      const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      c = 1.0 / sqrt(1.0 + t * t);
      s = c * t;
      atomicAdd(rotated, 1);
    }
    cs[0] = c;
    cs[1] = s;
  }
  __syncthreads();
  const double c = cs[0], s = cs[1];
  if (s == 0.0) return;
  for (int64_t i = threadIdx.x; i < m; i += JT) {
    const double x = cp[i], y = cq[i];
    cp[i] = c * x - s * y;
    cq[i] = s * x + c * y;
  }
  if (V) {
    double* vp = V + int64_t(p) * ne;
    double* vq = V + int64_t(q) * ne;
    for (int i = threadIdx.x; i < ne; i += JT) {
      const double x = vp[i], y = vq[i];
      vp[i] = c * x - s * y;
      vq[i] = s * x + c * y;
    }
  }
}

// sigma_j = |c_j| for j < n
__global__ void __launch_bounds__(JT) jac_norms_kernel(const double* __restrict__ C, int64_t m,
                                                      double* __restrict__ sig) {
  __shared__ double red[JT / 32];
  const double* c = C + int64_t(blockIdx.x) * m;
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += JT) a = fma(c[i], c[i], a);
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < JT / 32; ++i) t += red[i];
    sig[blockIdx.x] = sqrt(t);
  }
}

// order[rank] = j, descending sigma (ties by index): one CTA, rank by counting
__global__ void jac_rank_kernel(const double* __restrict__ sig, int n, int* __restrict__ order) {
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const double sj = sig[j];
    int r = 0;
    for (int i = 0; i < n; ++i) {
      const double si = sig[i];
      r += (si > sj) || (si == sj && i < j);
    }
    order[r] = j;
  }
}

// S[r] = sigma, U[:, r] = c_j / sigma (zero column for sigma = 0), VT[r, :] = V[:, j]
__global__ void jac_out_kernel(const double* __restrict__ C, int64_t m, const double* __restrict__ V, int ne,
                               int64_t n, const double* __restrict__ sig, const int* __restrict__ order,
                               double* __restrict__ S, double* __restrict__ U, double* __restrict__ VT) {
  const int r = blockIdx.x;
  const int j = order[r];
  const double sj = sig[j];
  if (threadIdx.x == 0 && S) S[r] = sj;
  if (U) {
    const double inv = sj > 0.0 ? 1.0 / sj : 0.0;
    const double* c = C + int64_t(j) * m;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) U[i * n + r] = c[i] * inv;
  }
  if (VT && V) {
    const double* v = V + int64_t(j) * ne;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) VT[int64_t(r) * n + i] = v[i];
  }
}

struct JacWs {
  double *C, *V, *sig;
  int *order, *counter;
};

size_t jac_layout(int64_t m, int64_t n, bool want_v, void* base, JacWs* w) {
  const int64_t ne = n + (n & 1);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align_up(bytes);
    return o;
  };
  const size_t oC = take(size_t(m) * ne * 8), oV = take(want_v ? size_t(ne) * ne * 8 : 0),
               os = take(size_t(ne) * 8), oo = take(size_t(ne) * 4), oc = take(16);
  if (w && base) {
    char* b = static_cast<char*>(base);
    w->C = reinterpret_cast<double*>(b + oC);
    w->V = want_v ? reinterpret_cast<double*>(b + oV) : nullptr;
    w->sig = reinterpret_cast<double*>(b + os);
    w->order = reinterpret_cast<int*>(b + oo);
    w->counter = reinterpret_cast<int*>(b + oc);
  }
  return off;
}

}  // namespace
}  // namespace tnx

using namespace tnx;

extern "C" {

size_t tnx_svd_workspace_bytes(int64_t m, int64_t n, int want_vt) {
  if (m <= 0 || n <= 0 || m < n) return 0;
  return jac_layout(m, n, want_vt != 0, nullptr, nullptr);
}

int tnx_svd(const double* A, int64_t m, int64_t n, double* S, double* U, double* VT, int* sweeps_out,
            void* workspace, size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(A && S, "null pointer");
  TNX_CHECK_ARG(m > 0 && n > 0, "non-positive dimension");
  TNX_CHECK_SHAPE(m >= n, "tnx_svd needs m >= n (got %lld x %lld); pass the transpose", (long long)m, (long long)n);
  TNX_CHECK_SHAPE(n <= (int64_t(1) << 20) && m <= (int64_t(1) << 40), "matrix too large");
  const size_t need = jac_layout(m, n, VT != nullptr, nullptr, nullptr);
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_svd: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  JacWs w;
  jac_layout(m, n, VT != nullptr, workspace, &w);
  const int ne = int(n + (n & 1));
  jac_init_kernel<<<152 * 4, 256, 0, st>>>(A, m, n, ne, w.C, w.V);
  TNX_LAUNCH_CHECK();
  const double tol = sqrt(double(m)) * 2.220446049250313e-16;
  int sweeps = 0, host_count = 1;
  if (ne >= 2) {
    for (; sweeps < kMaxSweeps && host_count > 0; ++sweeps) {
      TNX_CUDA(cudaMemsetAsync(w.counter, 0, sizeof(int), st));
      for (int r = 0; r < ne - 1; ++r) {
        jac_round_kernel<<<ne / 2, JT, 0, st>>>(w.C, m, w.V, ne, r, tol, w.counter);
        TNX_LAUNCH_CHECK();
      }
      TNX_CUDA(cudaMemcpyAsync(&host_count, w.counter, sizeof(int), cudaMemcpyDeviceToHost, st));
      TNX_CUDA(cudaStreamSynchronize(st));
    }
  }
  jac_norms_kernel<<<int(n), JT, 0, st>>>(w.C, m, w.sig);
  TNX_LAUNCH_CHECK();
  jac_rank_kernel<<<1, 1024, 0, st>>>(w.sig, int(n), w.order);
  TNX_LAUNCH_CHECK();
  jac_out_kernel<<<int(n), 256, 0, st>>>(w.C, m, w.V, ne, n, w.sig, w.order, S, U, VT);
  TNX_LAUNCH_CHECK();
  if (sweeps_out) *sweeps_out = sweeps;
  if (host_count > 0) {
    TNX_CUDA(cudaStreamSynchronize(st));
    set_error("tnx_svd: %d rotations still above tolerance after %d sweeps", host_count, sweeps);
    return TNX_ERR_NOT_CONVERGED;
  }
  return TNX_OK;
}

}  // extern "C"
