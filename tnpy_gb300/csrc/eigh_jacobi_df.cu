// Dense symmetric eigensolver for small matrices (n <= 64) in double-FP32 arithmetic: an
// FP64-class form of the batched Jacobi behind tSDRG's dense block spectra (np.linalg.eigh at
// tnpy/tsdrg.py:584), selected by eigh_batched(..., precision="df64").
//
// One CTA per matrix, the matrix and the rotation accumulator V held in shared memory as
// (hi, lo) float pairs, parallel cyclic Jacobi with the round-robin ordering of the FP64
// kernel (eigh_jacobi.cu). On this part a dependent FP64 FMA takes ~64 cycles and FP64
// square root / division several hundred, against ~5 cycles for FP32, so:
//   * the rotation angle comes from FP32 arithmetic on the leading parts (the difference
//     a_qq - a_pp taken in double-FP32 first, so that close diagonal entries keep a relative
//     angle error of ~1e-7); the Jacobi iteration converges with such angles: the ~1e-7 of a_pq
//     that an approximate angle leaves stays in the matrix (it is not zeroed as exact-angle
//     Jacobi does) and the next sweep rotates it away;
//   * the rotation is made orthogonal in double-FP32: c = 1 / sqrt(1 + t^2) by an rsqrtf seed and
//     two Newton steps, s = t c, so c^2 + s^2 = 1 to the format's ~2^-47 and V stays orthonormal;
//   * the updates of A and V (two products and a sum per element) run in double-FP32.
// Off-diagonal entries below 1e-13 ||A||_F (or 1e-13 sqrt|a_pp a_qq|) are left alone, about the
// rounding the rotations accumulate, so that a sweep can end without rotations. Output as the FP64
// kernel: the lowest `keep` eigenvalues ascending and their vectors, as FP64.
#include <cuda_runtime.h>

#include <atomic>

#include "tnx_internal.cuh"
#include "qr_panel_df.cuh"

namespace tnx {
namespace {

using qrdf::df2;

constexpr int EJD_THREADS = 512;
constexpr int EJD_MAX = 64;
constexpr int EJD_MAX_SWEEPS = 40;

__device__ __forceinline__ int rr_player_df(int j, int r, int np) {
  return j == 0 ? 0 : 1 + (j - 1 + r) % (np - 1);
}

__global__ void __launch_bounds__(EJD_THREADS) jacobi_eigh_df_kernel(
    const double* __restrict__ A_all, const int64_t* __restrict__ offsets, const int* __restrict__ sizes,
    int max_size, int keep, double* __restrict__ evals, double* __restrict__ evecs) {
  extern __shared__ df2 sm[];
  const int b = blockIdx.x;
  const int n = sizes[b];
  const double* Ain = A_all + offsets[b];
  // [n][ld] each, ld = n + 1: the column sweeps of a round (32 rows of one column per warp) then
  // fall on distinct banks instead of one
  const int ld = n + 1;
  df2* A = sm;
  df2* V = sm + EJD_MAX * (EJD_MAX + 1);
  __shared__ df2 sc[EJD_MAX / 2], ss[EJD_MAX / 2];
  __shared__ int sp[EJD_MAX / 2], sq[EJD_MAX / 2];
  __shared__ float red[EJD_THREADS / 32];
  __shared__ int s_rot;
  __shared__ float s_fro;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (n <= 0) return;

  float fro = 0.f;
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e % n;
    df2 v;
    split_df(Ain[size_t(i) * n + j], v.h, v.l);
    A[i * ld + j] = v;
    V[i * ld + j] = {i == j ? 1.f : 0.f, 0.f};
    fro = fmaf(v.h, v.h, fro);
  }
  for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
  if ((tid & 31) == 0) red[tid >> 5] = fro;
  __syncthreads();
  if (tid == 0) {
    float t = 0.f;
    for (int w = 0; w < nt / 32; ++w) t += red[w];
    s_fro = sqrtf(t);
  }
  __syncthreads();
  // off-diagonal entries below 1e-13 ||A||_F are left alone: the rotations' double-FP32 rounding
  // (~2^-47 per operation) accumulates to about that over the sweeps, and an entry that small
  // moves the eigenvalues by ~1e-26 ||A||^2 / gap
  const float abs_floor = 1e-30f + 1e-13f * s_fro;

  if (n > 1) {
    const int np = n + (n & 1);
    const int npairs = np / 2;
    for (int sweep = 0; sweep < EJD_MAX_SWEEPS; ++sweep) {
      if (tid == 0) s_rot = 0;
      __syncthreads();
      for (int r = 0; r < np - 1; ++r) {
        for (int k = tid; k < npairs; k += nt) {
          int p = rr_player_df(k, r, np), q = rr_player_df(np - 1 - k, r, np);
          if (p > q) {
            const int t = p;
            p = q;
            q = t;
          }
          df2 c = {1.f, 0.f}, s = {0.f, 0.f};
          if (q < n) {
            const df2 apq = A[p * ld + q], app = A[p * ld + p], aqq = A[q * ld + q];
            const float a = fabsf(apq.h);
            if (a > abs_floor && a > 1e-13f * sqrtf(fabsf(app.h * aqq.h))) {
              const df2 dqp = qrdf::add(aqq, qrdf::neg(app));
              const float theta = dqp.h / (2.f * apq.h);
              float t;
              if (fabsf(theta) > 1e18f) {
                t = 0.5f / theta;  // theta^2 would overflow; t = 1 / (2 theta) to ~theta^-2
              } else {
                t = copysignf(1.f, theta) / (fabsf(theta) + sqrtf(fmaf(theta, theta, 1.f)));
              }
              const df2 tt = {t, 0.f};
              c = qrdf::rsqrt_df(qrdf::add({1.f, 0.f}, qrdf::mul(tt, tt)));
              s = qrdf::mul(tt, c);
              s_rot = 1;
            }
          }
          sp[k] = p;
          sq[k] = q;
          sc[k] = c;
          ss[k] = s;
        }
        __syncthreads();
        // A <- A P (columns p, q of every row)
        for (int e = tid; e < npairs * n; e += nt) {
          const int k = e / n, i = e % n;
          const df2 s = ss[k];
          if (s.h == 0.f) continue;
          const int p = sp[k], q = sq[k];
          const df2 c = sc[k];
          const df2 aip = A[i * ld + p], aiq = A[i * ld + q];
          A[i * ld + p] = qrdf::fms(qrdf::mul(c, aip), s, aiq);
          A[i * ld + q] = qrdf::add(qrdf::mul(s, aip), qrdf::mul(c, aiq));
        }
        __syncthreads();
        // A <- P^T A (rows p, q of every column); V <- V P
        for (int e = tid; e < npairs * n; e += nt) {
          const int k = e / n, j = e % n;
          const df2 s = ss[k];
          if (s.h == 0.f) continue;
          const int p = sp[k], q = sq[k];
          const df2 c = sc[k];
          const df2 apj = A[p * ld + j], aqj = A[q * ld + j];
          A[p * ld + j] = qrdf::fms(qrdf::mul(c, apj), s, aqj);
          A[q * ld + j] = qrdf::add(qrdf::mul(s, apj), qrdf::mul(c, aqj));
          const df2 vjp = V[j * ld + p], vjq = V[j * ld + q];
          V[j * ld + p] = qrdf::fms(qrdf::mul(c, vjp), s, vjq);
          V[j * ld + q] = qrdf::add(qrdf::mul(s, vjp), qrdf::mul(c, vjq));
        }
        // (a_pq is not set to zero after the rotation: the FP32 angle leaves ~1e-7 of it, which
        // belongs to the matrix and is rotated away in the next sweep)
        __syncthreads();
      }
      if (s_rot == 0) break;
      __syncthreads();
    }
  }
  // ascending order: rank of each diagonal entry (ties broken by index)
  double* ev_out = evals + size_t(b) * keep;
  double* vec_out = evecs + size_t(b) * max_size * keep;
  for (int i = tid; i < n; i += nt) {
    const double di = join_df(A[i * ld + i].h, A[i * ld + i].l);
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double dj = join_df(A[j * ld + j].h, A[j * ld + j].l);
      rank += (dj < di) || (dj == di && j < i);
    }
    if (rank < keep) {
      ev_out[rank] = di;
      for (int row = 0; row < n; ++row) vec_out[size_t(row) * keep + rank] = join_df(V[row * ld + i].h, V[row * ld + i].l);
    }
  }
}

}  // namespace
}  // namespace tnx

using namespace tnx;

extern "C" {

int tnx_eigh_batched_df64(double* A, const int64_t* offsets, const int* sizes, int batch, int max_size, int keep,
                          double* evals, double* evecs, void* stream) {
  TNX_CHECK_ARG(A && offsets && sizes && evals && evecs, "null pointer");
  TNX_CHECK_ARG(batch >= 0 && max_size > 0 && keep > 0 && keep <= max_size, "bad batch/max_size/keep (%d, %d, %d)",
                batch, max_size, keep);
  TNX_CHECK_SHAPE(max_size <= EJD_MAX, "double-FP32 eigh: matrices up to %d (got %d)", EJD_MAX, max_size);
  if (batch == 0) return TNX_OK;
  const size_t smem = size_t(2) * EJD_MAX * (EJD_MAX + 1) * sizeof(df2);
  static std::atomic<bool> attr{false};
  if (!attr.load()) {
    TNX_CUDA(cudaFuncSetAttribute(jacobi_eigh_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    attr.store(true);
  }
  cudaStream_t st = as_stream(stream);
  profile_mark(KF_EIGH, st, true);
  jacobi_eigh_df_kernel<<<batch, EJD_THREADS, smem, st>>>(A, offsets, sizes, max_size, keep, evals, evecs);
  profile_mark(KF_EIGH, st, false);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

}  // extern "C"
