// Double-FP32 ("df64") GEMM: FP64 in, FP64 out, arithmetic on the FP32 pipe.
//
// GB300 issues FP64 at ~2 FMA/clock/SM but FP32 at 128 FMA/clock/SM. Each FP64 operand is
// split into a float pair (hi, lo) by integer operations (split_df); a product is formed as
//   p = hi_a*hi_b, e = fma(hi_a, hi_b, -p) + hi_a*lo_b + lo_a*hi_b   (error-free + cross terms)
// and accumulated with an error-free two-sum into a (hi, lo) float pair. About 11 FP32
// operations per product give ~2^-48 relative accuracy per product, i.e. FP64-class
// environments, residuals and gauge moves at several times the native FP64 rate.
//
// Tiling: 64 x 128 output tile per CTA, 16-deep K slab, 256 threads, 4 x 8 outputs per
// thread at stride 16 (conflict-free shared-memory reads), operands staged as float pairs;
// the next slab's global loads are issued into registers before the current slab's products.
// One such tile is ~0.5M double-FP32 products, tens of microseconds on one SM: products whose
// large-tile grid would not fill two waves of the GPU (the narrow QR panel updates, small
// split-K slices) use 32 x 32 tiles of 64 threads instead, eight times as many CTAs.
#include <cuda_runtime.h>

#include <cstdlib>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

constexpr int DK = 16;

__device__ __forceinline__ void df_fma(float ah, float al, float bh, float bl, float& ch, float& cl) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  const float s = ch + p;
  const float bv = s - ch;
  const float err = (ch - (s - bv)) + (p - bv);
  ch = s;
  cl += err + e;
}

// BM x BN output tile, NT threads: thread (tx, ty) = (tid % 16, tid / 16) owns rows ty + TY i
// and columns tx + 16 j
template <bool TA, bool TB, int BM, int BN, int NT>
__global__ void __launch_bounds__(NT) gemm_df64_kernel(int64_t M, int64_t N, int64_t K, double alpha,
                                                     const double* __restrict__ A, int64_t lda, int64_t sa,
                                                     const double* __restrict__ B, int64_t ldb, int64_t sb,
                                                     double beta, double* __restrict__ C, int64_t ldc, int64_t sc,
                                                     int64_t k_total, const int* __restrict__ bmask) {
  constexpr int DM = BM, DN = BN, DT = NT, TY = NT / 16;
  constexpr int RI = DM / TY, RJ = DN / 16;  // outputs per thread
  static_assert(NT % 16 == 0 && DM % TY == 0 && DN % 16 == 0 && (DM * DK) % NT == 0 && (DN * DK) % NT == 0,
                "df64 GEMM tile");
  __shared__ float Ah[DK][DM + 4], Al[DK][DM + 4];
  __shared__ float Bh[DK][DN + 4], Bl[DK][DN + 4];
  const int64_t bz = blockIdx.z;
  if (bmask && !bmask[bz]) return;  // a batch entry the caller masked out
  A += bz * sa;
  B += bz * sb;
  C += bz * sc;
  if (k_total > 0) {
    const int64_t rem = k_total - bz * K;
    K = rem < K ? rem : K;
  }
  const int64_t m0 = int64_t(blockIdx.y) * DM, n0 = int64_t(blockIdx.x) * DN;
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  float ch[RI][RJ], cl[RI][RJ];
#pragma unroll
  for (int i = 0; i < RI; ++i)
#pragma unroll
    for (int j = 0; j < RJ; ++j) ch[i][j] = cl[i][j] = 0.f;

  constexpr int LA = (DM * DK) / DT, LB = (DN * DK) / DT;  // slab elements per thread
  double pa[LA], pb[LB];
  // global -> registers for the slab at k0 (zero outside the matrix)
  auto fetch = [&](int64_t k0) {
#pragma unroll
    for (int r = 0; r < LA; ++r) {
      const int e = tid + r * DT;
      const int mm = TA ? e % DM : e / DK, kk = TA ? e / DM : e % DK;
      const int64_t gm = m0 + mm, gk = k0 + kk;
      pa[r] = (gm < M && gk < K) ? (TA ? A[gk * lda + gm] : A[gm * lda + gk]) : 0.0;
    }
#pragma unroll
    for (int r = 0; r < LB; ++r) {
      const int e = tid + r * DT;
      const int nn = TB ? e / DK : e % DN, kk = TB ? e % DK : e / DN;
      const int64_t gn = n0 + nn, gk = k0 + kk;
      pb[r] = (gn < N && gk < K) ? (TB ? B[gn * ldb + gk] : B[gk * ldb + gn]) : 0.0;
    }
  };
  // registers -> shared memory as (hi, lo) float pairs
  auto stage = [&]() {
#pragma unroll
    for (int r = 0; r < LA; ++r) {
      const int e = tid + r * DT;
      const int mm = TA ? e % DM : e / DK, kk = TA ? e / DM : e % DK;
      split_df(pa[r], Ah[kk][mm], Al[kk][mm]);
    }
#pragma unroll
    for (int r = 0; r < LB; ++r) {
      const int e = tid + r * DT;
      const int nn = TB ? e / DK : e % DN, kk = TB ? e % DK : e / DN;
      split_df(pb[r], Bh[kk][nn], Bl[kk][nn]);
    }
  };
  // software pipeline: the global loads of slab k0 + DK are in flight while slab k0 is multiplied
  fetch(0);
  stage();
  __syncthreads();
  for (int64_t k0 = 0; k0 < K; k0 += DK) {
    const bool more = k0 + DK < K;
    if (more) fetch(k0 + DK);
#pragma unroll 2
    for (int kk = 0; kk < DK; ++kk) {
      float ah[RI], al[RI], bh[RJ], bl[RJ];
#pragma unroll
      for (int i = 0; i < RI; ++i) {
        ah[i] = Ah[kk][ty + TY * i];
        al[i] = Al[kk][ty + TY * i];
      }
#pragma unroll
      for (int j = 0; j < RJ; ++j) {
        bh[j] = Bh[kk][tx + 16 * j];
        bl[j] = Bl[kk][tx + 16 * j];
      }
#pragma unroll
      for (int i = 0; i < RI; ++i)
#pragma unroll
        for (int j = 0; j < RJ; ++j) df_fma(ah[i], al[i], bh[j], bl[j], ch[i][j], cl[i][j]);
    }
    __syncthreads();
    if (more) {
      stage();
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < RI; ++i) {
    const int64_t gm = m0 + ty + TY * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < RJ; ++j) {
      const int64_t gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      double v = alpha * (double(ch[i][j]) + double(cl[i][j]));
      if (beta != 0.0) v = fma(beta, C[gm * ldc + gn], v);
      C[gm * ldc + gn] = v;
    }
  }
}

}  // namespace

int gemm_df64(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
              int64_t sa, const double* B, int64_t ldb, int64_t sb, double beta, double* C, int64_t ldc, int64_t sc,
              int64_t batch, cudaStream_t st, int64_t k_total, const int* bmask) {
  if (m <= 0 || n <= 0 || batch <= 0) return TNX_OK;
  if (k <= 0) return gemm_f64(ta, tb, m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, batch, st);
  TNX_CHECK_SHAPE(batch <= 65535, "gemm_df64: batch %lld > 65535", (long long)batch);
  // TNX_DF64_SMALL_WAVES (tuning, default 2): large-tile waves below which 32 x 32 tiles are used
  static const int small_waves = [] {
    const char* e = getenv("TNX_DF64_SMALL_WAVES");
    return e ? atoi(e) : 2;
  }();
  const int64_t big = ((n + 127) / 128) * ((m + 63) / 64) * batch;
  const bool small_rule = big < int64_t(small_waves) * 152;
  // variant 0: 64 x 128 tiles, 256 threads; variant 1: 32 x 32 tiles, 64 threads
  auto launch = [&](int v) -> int {
    const bool small = v == 1;
    const int64_t bm = small ? 32 : 64, bn = small ? 32 : 128;
    dim3 grid((unsigned)((n + bn - 1) / bn), (unsigned)((m + bm - 1) / bm), (unsigned)batch);
    TNX_CHECK_SHAPE(grid.y <= 65535, "gemm_df64: m too large");
    auto go = [&](auto kernel, int nt) {
      kernel<<<grid, nt, 0, st>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, k_total, bmask);
    };
    if (small) {
      if (!ta && !tb) go(gemm_df64_kernel<false, false, 32, 32, 64>, 64);
      else if (ta && !tb) go(gemm_df64_kernel<true, false, 32, 32, 64>, 64);
      else if (!ta && tb) go(gemm_df64_kernel<false, true, 32, 32, 64>, 64);
      else go(gemm_df64_kernel<true, true, 32, 32, 64>, 64);
    } else {
      if (!ta && !tb) go(gemm_df64_kernel<false, false, 64, 128, 256>, 256);
      else if (ta && !tb) go(gemm_df64_kernel<true, false, 64, 128, 256>, 256);
      else if (!ta && tb) go(gemm_df64_kernel<false, true, 64, 128, 256>, 256);
      else go(gemm_df64_kernel<true, true, 64, 128, 256>, 256);
    }
    TNX_LAUNCH_CHECK();
    return TNX_OK;
  };
  profile_mark(KF_F64_GEMM, st, true);
  const TuneKey key{1, int64_t(ta) * 2 + int64_t(tb), m, n, k_total > 0 ? k_total : k, batch};
  // a masked call skips some batch entries: its timing would not represent the shape
  TNX_TRY(autotuned(key, 2, small_rule ? 1 : 0, beta == 0.0 && !bmask, st, launch));
  profile_mark(KF_F64_GEMM, st, false);
  profile_work(KF_F64_GEMM, 2.0 * double(m) * n * (k_total > 0 ? k_total : k * batch),
               8.0 * (double(m) * k + double(k) * n + double(m) * n) * batch);
  return TNX_OK;
}

int gemm_fp64_class(bool df, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                    int64_t lda, int64_t sa, const double* B, int64_t ldb, int64_t sb, double beta, double* C,
                    int64_t ldc, int64_t sc, int64_t batch, cudaStream_t st, int64_t k_total, const int* bmask) {
  if (df)
    return gemm_df64(ta, tb, m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, batch, st, k_total, bmask);
  return gemm_f64(ta, tb, m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, batch, st, k_total, bmask);
}

}  // namespace tnx

using namespace tnx;

extern "C" int tnx_gemm_df64(int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                             int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                             void* stream) {
  TNX_CHECK_ARG(A && B && C, "null pointer");
  TNX_CHECK_ARG(m >= 0 && n >= 0 && k >= 0, "negative size");
  return gemm_df64(trans_a != 0, trans_b != 0, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1,
                   as_stream(stream), 0);
}
