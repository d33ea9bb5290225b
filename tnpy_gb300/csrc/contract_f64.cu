// FP64 contraction kernels of the one-site effective Hamiltonian and the environment
// updates (the plain FP64 form), plus the C ABI entry points that sequence them.
//
// Reference: Environment.one_site_matvec (tnpy/matrix_product_state.py:411-440),
// update_left / update_right (:296-336), one_site_full_matrix (:372-409).
//
// Every contraction is L x MPS -> MPO -> R split into two GEMMs (K = chi and K = chi*D)
// around a small dense MPO step (K = D*d), i.e. 4*chi^3*D*d + 2*chi^2*D^2*d^2 flops.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "tnx_internal.cuh"

namespace tnx {

// ---------------------------------------------------------------------------------
// FP64 SIMT GEMM: 64x64 tile, 16-deep K slab, 256 threads, 4x4 outputs per thread
// interleaved by 16 so that shared-memory reads of a warp hit distinct banks.
// GB300 runs FP64 at ~1/64 of the FP32 rate, so this kernel is bound by the FP64 pipe
// for every shape that matters; the tiling only has to keep that pipe fed.
// ---------------------------------------------------------------------------------
namespace {
constexpr int GB_M = 64, GB_N = 64, GB_K = 16, GB_T = 256;

template <bool TA, bool TB>
__global__ void __launch_bounds__(GB_T) gemm_f64_kernel(int64_t M, int64_t N, int64_t K, double alpha,
                                                     const double* __restrict__ A, int64_t lda,
                                                     int64_t sa, const double* __restrict__ B,
                                                     int64_t ldb, int64_t sb, double beta,
                                                     double* __restrict__ C, int64_t ldc,
                                                     int64_t sc, int64_t k_total,
                                                     const int* __restrict__ bmask) {
  __shared__ double As[GB_K][GB_M + 1];
  __shared__ double Bs[GB_K][GB_N + 1];
  const int64_t bz = blockIdx.z;
  if (bmask && !bmask[bz]) return;  // a batch entry the caller masked out
  A += bz * sa;
  B += bz * sb;
  C += bz * sc;
  const int64_t m0 = int64_t(blockIdx.y) * GB_M, n0 = int64_t(blockIdx.x) * GB_N;
  // split-K mode (k_total > 0): batch index bz owns K range [bz*K, min((bz+1)*K, k_total))
  if (k_total > 0) {
    const int64_t rem = k_total - bz * K;
    K = rem < K ? rem : K;
  }
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int64_t k0 = 0; k0 < K; k0 += GB_K) {
    // A tile: As[kk][mm] = op(A)[m0+mm][k0+kk]
#pragma unroll
    for (int r = 0; r < (GB_M * GB_K) / GB_T; ++r) {
      int e = tid + r * GB_T;
      int mm, kk;
      if (TA) {  // stored K x M: consecutive threads walk m
        mm = e % GB_M;
        kk = e / GB_M;
      } else {  // stored M x K: consecutive threads walk k
        kk = e % GB_K;
        mm = e / GB_K;
      }
      int64_t gm = m0 + mm, gk = k0 + kk;
      double v = 0.0;
      if (gm < M && gk < K) v = TA ? A[gk * lda + gm] : A[gm * lda + gk];
      As[kk][mm] = v;
    }
    // B tile: Bs[kk][nn] = op(B)[k0+kk][n0+nn]
#pragma unroll
    for (int r = 0; r < (GB_N * GB_K) / GB_T; ++r) {
      int e = tid + r * GB_T;
      int nn, kk;
      if (TB) {  // stored N x K
        kk = e % GB_K;
        nn = e / GB_K;
      } else {  // stored K x N
        nn = e % GB_N;
        kk = e / GB_N;
      }
      int64_t gn = n0 + nn, gk = k0 + kk;
      double v = 0.0;
      if (gn < N && gk < K) v = TB ? B[gn * ldb + gk] : B[gk * ldb + gn];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GB_K; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int64_t gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      double v = alpha * acc[i][j];
      if (beta != 0.0) v = fma(beta, C[gm * ldc + gn], v);
      C[gm * ldc + gn] = v;
    }
  }
}
}  // namespace

int gemm_f64(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
             int64_t lda, int64_t sa, const double* B, int64_t ldb, int64_t sb, double beta,
             double* C, int64_t ldc, int64_t sc, int64_t batch, cudaStream_t st, int64_t k_total,
             const int* bmask) {
  if (m <= 0 || n <= 0 || batch <= 0) return TNX_OK;
  if (k <= 0) {
    // C = beta * C; only the beta == 0 case is used here
    TNX_CHECK_ARG(beta == 0.0, "gemm_f64: k == 0 with beta != 0 not supported");
    for (int64_t b = 0; b < batch; ++b)
      for (int64_t r = 0; r < m; ++r) TNX_CUDA(cudaMemsetAsync(C + b * sc + r * ldc, 0, n * 8, st));
    return TNX_OK;
  }
  TNX_CHECK_SHAPE(batch <= 65535, "gemm_f64: batch %lld > 65535", (long long)batch);
  dim3 grid((unsigned)((n + GB_N - 1) / GB_N), (unsigned)((m + GB_M - 1) / GB_M), (unsigned)batch);
  TNX_CHECK_SHAPE(grid.y <= 65535, "gemm_f64: m too large");
  profile_mark(KF_F64_GEMM, st, true);
  if (!ta && !tb)
    gemm_f64_kernel<false, false><<<grid, GB_T, 0, st>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, k_total,
                                                          bmask);
  else if (ta && !tb)
    gemm_f64_kernel<true, false><<<grid, GB_T, 0, st>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, k_total,
                                                          bmask);
  else if (!ta && tb)
    gemm_f64_kernel<false, true><<<grid, GB_T, 0, st>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, k_total,
                                                          bmask);
  else
    gemm_f64_kernel<true, true><<<grid, GB_T, 0, st>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, k_total,
                                                          bmask);
  profile_mark(KF_F64_GEMM, st, false);
  profile_work(KF_F64_GEMM, 2.0 * double(m) * n * k * batch, 8.0 * (double(m) * k + double(k) * n + double(m) * n) * batch);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

namespace {
// C = alpha * sum_z P[z] + beta * C (P: nsplit partial m x n row-major products)
__global__ void splitk_reduce_kernel(const double* __restrict__ P, int nsplit, int64_t m, int64_t n, double alpha,
                                     double beta, double* __restrict__ C, int64_t ldc) {
  const int64_t mn = m * n;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < mn; e += int64_t(gridDim.x) * blockDim.x) {
    double acc = 0.0;
    for (int z = 0; z < nsplit; ++z) acc += P[z * mn + e];
    const int64_t i = e / n, j = e % n;
    double v = alpha * acc;
    if (beta != 0.0) v = fma(beta, C[i * ldc + j], v);
    C[i * ldc + j] = v;
  }
}
}  // namespace

int gemm_f64_splitk(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
                    const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int nsplit, double* part,
                    cudaStream_t st, bool df) {
  if (nsplit <= 1) return gemm_fp64_class(df, ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1, st);
  const int64_t kc = (k + nsplit - 1) / nsplit;
  nsplit = int((k + kc - 1) / kc);
  const int64_t sa = ta ? kc * lda : kc, sb = tb ? kc : kc * ldb;
  TNX_TRY(gemm_fp64_class(df, ta, tb, m, n, kc, 1.0, A, lda, sa, B, ldb, sb, 0.0, part, n, m * n, nsplit, st, k));
  int64_t blocks = (m * n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  splitk_reduce_kernel<<<unsigned(blocks < 1 ? 1 : blocks), 256, 0, st>>>(part, nsplit, m, n, alpha, beta, C, ldc);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

// ---------------------------------------------------------------------------------
// MPO step. The MPO tensor (at most 32 x 32 x 2 x 2 here) is staged in shared memory;
// each thread owns one (a', c) [left form] or (a, c') [right form] fibre and produces
// all dr*d (dl*d) outputs from its dl*d (dr*d) inputs.
// ---------------------------------------------------------------------------------
namespace {
constexpr int WMAX = 64;  // max dl*d and dr*d handled per thread

__global__ void wcontract_left_kernel(const double* __restrict__ T1, const double* __restrict__ W,
                                      double* __restrict__ T2, int64_t chi_l, int d, int64_t chi_r,
                                      int dl, int dr) {
  extern __shared__ double ws[];
  const int wn = dl * dr * d * d;
  for (int i = threadIdx.x; i < wn; i += blockDim.x) ws[i] = W[i];
  __syncthreads();
  const int64_t total = chi_l * chi_r;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t ap = idx / chi_r, c = idx % chi_r;
    double in[WMAX];
    // T1[(w,a'),(s,c)] at ((w*chi_l + a')*d + s)*chi_r + c
    for (int w = 0; w < dl; ++w)
      for (int s = 0; s < d; ++s) in[w * d + s] = T1[((w * chi_l + ap) * d + s) * chi_r + c];
    // T2[(a',s'),(c,v)] at ((a'*d + s')*chi_r + c)*dr + v
    for (int sp = 0; sp < d; ++sp) {
      double* out = T2 + ((ap * d + sp) * chi_r + c) * dr;
      for (int v = 0; v < dr; ++v) {
        double acc = 0.0;
        for (int w = 0; w < dl; ++w)
          for (int s = 0; s < d; ++s) acc = fma(in[w * d + s], ws[((w * dr + v) * d + s) * d + sp], acc);
        out[v] = acc;
      }
    }
  }
}

__global__ void wcontract_right_kernel(const double* __restrict__ T1, const double* __restrict__ W,
                                       double* __restrict__ T2, int64_t chi_l, int d, int64_t chi_r,
                                       int dl, int dr) {
  extern __shared__ double ws[];
  const int wn = dl * dr * d * d;
  for (int i = threadIdx.x; i < wn; i += blockDim.x) ws[i] = W[i];
  __syncthreads();
  const int64_t total = chi_l * chi_r;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t a = idx / chi_r, cp = idx % chi_r;
    double in[WMAX];
    // T1[(a,s),(v,c')] at ((a*d + s)*dr + v)*chi_r + c'
    for (int s = 0; s < d; ++s)
      for (int v = 0; v < dr; ++v) in[v * d + s] = T1[((a * d + s) * dr + v) * chi_r + cp];
    // T2[(a,w),(s',c')] at ((a*dl + w)*d + s')*chi_r + c'
    for (int w = 0; w < dl; ++w)
      for (int sp = 0; sp < d; ++sp) {
        double acc = 0.0;
        for (int v = 0; v < dr; ++v)
          for (int s = 0; s < d; ++s) acc = fma(in[v * d + s], ws[((w * dr + v) * d + s) * d + sp], acc);
        T2[((a * dl + w) * d + sp) * chi_r + cp] = acc;
      }
  }
}

inline unsigned grid_for(int64_t total, int threads) {
  int64_t b = (total + threads - 1) / threads;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}
}  // namespace

int wcontract_left(const double* T1, const double* W, double* T2, int64_t chi_l, int64_t d,
                   int64_t chi_r, int64_t dl, int64_t dr, cudaStream_t st) {
  TNX_CHECK_SHAPE(dl * d <= WMAX && dr * d <= WMAX, "MPO bond too large (dl*d, dr*d <= %d)", WMAX);
  size_t smem = size_t(dl * dr * d * d) * sizeof(double);
  wcontract_left_kernel<<<grid_for(chi_l * chi_r, 128), 128, smem, st>>>(T1, W, T2, chi_l, (int)d, chi_r,
                                                                          (int)dl, (int)dr);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

int wcontract_right(const double* T1, const double* W, double* T2, int64_t chi_l, int64_t d,
                    int64_t chi_r, int64_t dl, int64_t dr, cudaStream_t st) {
  TNX_CHECK_SHAPE(dl * d <= WMAX && dr * d <= WMAX, "MPO bond too large (dl*d, dr*d <= %d)", WMAX);
  size_t smem = size_t(dl * dr * d * d) * sizeof(double);
  wcontract_right_kernel<<<grid_for(chi_l * chi_r, 128), 128, smem, st>>>(T1, W, T2, chi_l, (int)d, chi_r,
                                                                           (int)dl, (int)dr);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

int64_t matvec1_scratch_elems(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr) {
  int64_t a = dl * chi_l * d * chi_r, b = chi_l * d * chi_r * dr;
  return a > b ? a : b;
}

bool use_oz(int64_t m, int64_t n, int64_t k) {
  // the tensor-core FP64-class GEMM pays five launches of operand slicing: large products only
  return m >= 256 && n >= 64 && k >= 128 && double(m) * double(n) * double(k) >= double(1 << 27);
}

int gemm_fp64_class_oz(bool df, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                       int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* oz_ws,
                       size_t oz_bytes, cudaStream_t st) {
  if (df && oz_ws && use_oz(m, n, k) && oz_bytes >= gemm_oz_workspace_bytes(m, n, k)) {
    // FP64-class engine, autotuned per shape: 0 tcgen05 Ozaki GEMM, 1 double-FP32 SIMT GEMM
    auto run = [&](int v) -> int {
      if (v == 0) return gemm_oz(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, oz_ws, oz_bytes, st);
      return gemm_fp64_class(true, ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1, st);
    };
    const TuneKey key{2, int64_t(ta) * 2 + int64_t(tb), m, n, k, 0};
    return autotuned(key, 2, 0, beta == 0.0, st, run);
  }
  return gemm_fp64_class(df, ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1, st);
}

size_t matvec1_oz_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr) {
  size_t a = use_oz(dl * chi_l, d * chi_r, chi_l) ? gemm_oz_workspace_bytes(dl * chi_l, d * chi_r, chi_l) : 0;
  size_t b = use_oz(chi_l * d, chi_r, chi_r * dr) ? gemm_oz_workspace_bytes(chi_l * d, chi_r, chi_r * dr) : 0;
  return a > b ? a : b;
}

int matvec1_f64(const double* L, const double* W, const double* R, const double* x, double* y,
                int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, double* T1,
                double* T2, cudaStream_t st, bool df, void* oz_ws, size_t oz_bytes) {
  // T1[(w,a'),(s,c)] = sum_a L[a,(w,a')] x[a,(s,c)]
  TNX_TRY(gemm_fp64_class_oz(df, true, false, dl * chi_l, d * chi_r, chi_l, 1.0, L, dl * chi_l, x, d * chi_r, 0.0,
                             T1, d * chi_r, oz_ws, oz_bytes, st));
  TNX_TRY(wcontract_left(T1, W, T2, chi_l, d, chi_r, dl, dr, st));
  // y[(a',s'),c'] = sum_{(c,v)} T2[(a',s'),(c,v)] R[(c,v),c']
  TNX_TRY(gemm_fp64_class_oz(df, false, false, chi_l * d, chi_r, chi_r * dr, 1.0, T2, chi_r * dr, R, chi_r, 0.0, y,
                             chi_r, oz_ws, oz_bytes, st));
  return TNX_OK;
}

// ---------------------------------------------------------------------------------
// diag(H_eff) and dense H_eff
// ---------------------------------------------------------------------------------
namespace {
__global__ void diag1_kernel(const double* __restrict__ L, const double* __restrict__ W,
                             const double* __restrict__ R, double* __restrict__ diag, int64_t chi_l,
                             int d, int64_t chi_r, int dl, int dr) {
  const int64_t total = chi_l * d * chi_r;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t a = idx / (d * chi_r);
    const int s = int((idx / chi_r) % d);
    const int64_t c = idx % chi_r;
    double acc = 0.0;
    for (int w = 0; w < dl; ++w) {
      const double lw = L[(a * dl + w) * chi_l + a];
      for (int v = 0; v < dr; ++v)
        acc = fma(lw * W[((w * dr + v) * d + s) * d + s], R[(c * dr + v) * chi_r + c], acc);
    }
    diag[idx] = acc;
  }
}

__global__ void full_matrix1_kernel(const double* __restrict__ L, const double* __restrict__ W,
                                    const double* __restrict__ R, double* __restrict__ H,
                                    int64_t chi_l, int d, int64_t chi_r, int dl, int dr) {
  const int64_t n = chi_l * d * chi_r;
  const int64_t total = n * n;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t row = idx / n, col = idx % n;
    const int64_t a = row / (d * chi_r), c = row % chi_r;
    const int s = int((row / chi_r) % d);
    const int64_t ap = col / (d * chi_r), cp = col % chi_r;
    const int sp = int((col / chi_r) % d);
    double acc = 0.0;
    for (int w = 0; w < dl; ++w) {
      const double lw = L[(a * dl + w) * chi_l + ap];
      if (lw == 0.0) continue;
      for (int v = 0; v < dr; ++v)
        acc = fma(lw * W[((w * dr + v) * d + s) * d + sp], R[(c * dr + v) * chi_r + cp], acc);
    }
    H[idx] = acc;
  }
}
}  // namespace

}  // namespace tnx

using namespace tnx;

static int check_site(const void* L, const void* W, const void* R, int64_t chi_l, int64_t d,
                      int64_t chi_r, int64_t dl, int64_t dr) {
  TNX_CHECK_ARG(L && W && R, "null L/W/R pointer");
  TNX_CHECK_ARG(chi_l > 0 && d > 0 && chi_r > 0 && dl > 0 && dr > 0,
                "non-positive dimension (chi_l=%lld d=%lld chi_r=%lld dl=%lld dr=%lld)",
                (long long)chi_l, (long long)d, (long long)chi_r, (long long)dl, (long long)dr);
  TNX_CHECK_SHAPE(dl * d <= 64 && dr * d <= 64, "MPO bond too large: dl*d=%lld dr*d=%lld (max 64)",
                  (long long)(dl * d), (long long)(dr * d));
  return TNX_OK;
}

extern "C" {

size_t tnx_matvec1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                   int precision) {
  if (precision == TNX_BF16X3 && mixed_supported(chi_l, d, chi_r, dl, dr))
    return matvec1_bf16x3_scratch_bytes(chi_l, d, chi_r, dl, dr);
  const size_t t = 2 * align_up(size_t(matvec1_scratch_elems(chi_l, d, chi_r, dl, dr)) * sizeof(double));
  return precision == TNX_FP64 ? t : t + align_up(matvec1_oz_bytes(chi_l, d, chi_r, dl, dr));
}

int tnx_matvec1(const double* L, const double* W, const double* R, const double* x, double* y,
                int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, int precision,
                void* workspace, size_t workspace_bytes, void* stream) {
  TNX_TRY(check_site(L, W, R, chi_l, d, chi_r, dl, dr));
  TNX_CHECK_ARG(x && y, "null x/y pointer");
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  size_t need = tnx_matvec1_workspace_bytes(chi_l, d, chi_r, dl, dr, precision);
  if (workspace_bytes < need || (need && !workspace)) {
    set_error("tnx_matvec1: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  // sites with a bond below 16 (the chain ends) are too small for the tensor-core tiles and
  // always run the FP64 kernels
  if (precision == TNX_BF16X3 && mixed_supported(chi_l, d, chi_r, dl, dr))
    return matvec1_bf16x3(L, W, R, x, y, chi_l, d, chi_r, dl, dr, workspace, workspace_bytes, st);
  Arena ar(workspace, workspace_bytes);
  const int64_t ne = matvec1_scratch_elems(chi_l, d, chi_r, dl, dr);
  double* T1 = ar.take<double>(ne);
  double* T2 = ar.take<double>(ne);
  const size_t ozb = precision == TNX_DF64 ? matvec1_oz_bytes(chi_l, d, chi_r, dl, dr) : 0;
  void* oz = ozb ? static_cast<void*>(ar.take<char>(ozb)) : nullptr;
  return matvec1_f64(L, W, R, x, y, chi_l, d, chi_r, dl, dr, T1, T2, st, precision == TNX_DF64, oz, ozb);
}

int tnx_diag1(const double* L, const double* W, const double* R, double* diag, int64_t chi_l,
              int64_t d, int64_t chi_r, int64_t dl, int64_t dr, void* stream) {
  TNX_TRY(check_site(L, W, R, chi_l, d, chi_r, dl, dr));
  TNX_CHECK_ARG(diag, "null diag pointer");
  int64_t total = chi_l * d * chi_r;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  diag1_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(L, W, R, diag, chi_l, (int)d, chi_r,
                                                                (int)dl, (int)dr);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

int tnx_full_matrix1(const double* L, const double* W, const double* R, double* H, int64_t chi_l,
                     int64_t d, int64_t chi_r, int64_t dl, int64_t dr, void* stream) {
  TNX_TRY(check_site(L, W, R, chi_l, d, chi_r, dl, dr));
  TNX_CHECK_ARG(H, "null H pointer");
  int64_t n = chi_l * d * chi_r;
  TNX_CHECK_SHAPE(n <= 8192, "dense effective Hamiltonian limited to 8192 rows (got %lld)", (long long)n);
  int64_t blocks = (n * n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  full_matrix1_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(L, W, R, H, chi_l, (int)d, chi_r,
                                                                       (int)dl, (int)dr);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

// FP64-class scratch of the environment update's two GEMMs (tensor-core path)
static size_t env_oz_bytes(int direction, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr) {
  int64_t g[2][3];
  if (direction == 1) {
    int64_t a[2][3] = {{dl * chi_l, d * chi_r, chi_l}, {chi_r * dr, chi_r, chi_l * d}};
    memcpy(g, a, sizeof(g));
  } else {
    int64_t a[2][3] = {{chi_l * d, dr * chi_r, chi_r}, {chi_l * dl, chi_l, d * chi_r}};
    memcpy(g, a, sizeof(g));
  }
  size_t out = 0;
  for (auto& x : g)
    if (use_oz(x[0], x[1], x[2])) {
      const size_t b = gemm_oz_workspace_bytes(x[0], x[1], x[2]);
      out = b > out ? b : out;
    }
  return out;
}

size_t tnx_env_update_workspace_bytes(int direction, int64_t chi_l, int64_t d, int64_t chi_r,
                                      int64_t dl, int64_t dr, int precision) {
  const size_t t = 2 * align_up(size_t(matvec1_scratch_elems(chi_l, d, chi_r, dl, dr)) * sizeof(double));
  if (!use_df64(precision)) return t;
  return t + align_up(env_oz_bytes(direction == -1 ? -1 : 1, chi_l, d, chi_r, dl, dr));
}

int tnx_env_update(int direction, const double* E_in, const double* A, const double* W,
                   double* E_out, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                   int precision, void* workspace, size_t workspace_bytes, void* stream) {
  TNX_TRY(check_site(E_in, W, A, chi_l, d, chi_r, dl, dr));
  TNX_CHECK_ARG(E_out, "null E_out pointer");
  TNX_CHECK_ARG(direction == 1 || direction == -1, "direction must be +1 or -1 (got %d)", direction);
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  const bool df = use_df64(precision);
  size_t need = tnx_env_update_workspace_bytes(direction, chi_l, d, chi_r, dl, dr, precision);
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_env_update: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  Arena ar(workspace, workspace_bytes);
  const int64_t ne = matvec1_scratch_elems(chi_l, d, chi_r, dl, dr);
  double* T1 = ar.take<double>(ne);
  double* T2 = ar.take<double>(ne);
  const size_t ozb = df ? env_oz_bytes(direction, chi_l, d, chi_r, dl, dr) : 0;
  void* oz = ozb ? static_cast<void*>(ar.take<char>(ozb)) : nullptr;
  if (direction == 1) {
    // T1[(w,a'),(s,c)] = sum_a L[a,(w,a')] A[a,(s,c)]
    TNX_TRY(gemm_fp64_class_oz(df, true, false, dl * chi_l, d * chi_r, chi_l, 1.0, E_in, dl * chi_l, A, d * chi_r,
                               0.0, T1, d * chi_r, oz, ozb, st));
    TNX_TRY(wcontract_left(T1, W, T2, chi_l, d, chi_r, dl, dr, st));
    // L'[(c,v),c'] = sum_{(a',s')} T2[(a',s'),(c,v)] A[(a',s'),c']
    TNX_TRY(gemm_fp64_class_oz(df, true, false, chi_r * dr, chi_r, chi_l * d, 1.0, T2, chi_r * dr, A, chi_r, 0.0,
                               E_out, chi_r, oz, ozb, st));
  } else {
    // T1[(a,s),(v,c')] = sum_c A[(a,s),c] R[c,(v,c')]
    TNX_TRY(gemm_fp64_class_oz(df, false, false, chi_l * d, dr * chi_r, chi_r, 1.0, A, chi_r, E_in, dr * chi_r,
                               0.0, T1, dr * chi_r, oz, ozb, st));
    TNX_TRY(wcontract_right(T1, W, T2, chi_l, d, chi_r, dl, dr, st));
    // R'[(a,w),a'] = sum_{(s',c')} T2[(a,w),(s',c')] A[a',(s',c')]
    TNX_TRY(gemm_fp64_class_oz(df, false, true, chi_l * dl, chi_l, d * chi_r, 1.0, T2, d * chi_r, A, d * chi_r,
                               0.0, E_out, chi_l, oz, ozb, st));
  }
  return TNX_OK;
}

int tnx_gemm_f64(int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                 const double* A, int64_t lda, int64_t stride_a, const double* B, int64_t ldb,
                 int64_t stride_b, double beta, double* C, int64_t ldc, int64_t stride_c,
                 int64_t batch, void* stream) {
  TNX_CHECK_ARG(A && B && C, "null pointer");
  TNX_CHECK_ARG(m >= 0 && n >= 0 && k >= 0 && batch >= 0, "negative size");
  return gemm_f64(trans_a != 0, trans_b != 0, m, n, k, alpha, A, lda, stride_a, B, ldb, stride_b, beta,
                  C, ldc, stride_c, batch, as_stream(stream));
}

}  // extern "C"
