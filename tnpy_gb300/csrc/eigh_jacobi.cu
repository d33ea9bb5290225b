// Dense symmetric eigensolver, one CTA per matrix: parallel cyclic Jacobi (round-robin
// ordering, n/2 disjoint rotations per round), FP64.
//
// Used for the Davidson Rayleigh-Ritz problem (size <= max_basis), the dense
// effective-Hamiltonian path of FiniteDMRG.one_site_solver (tnpy/finite_dmrg.py:108-110,
// linalg.eigh at tnpy/linalg.py:42-61, N < 200) and tSDRG blocks (np.linalg.eigh at
// tnpy/tsdrg.py:584). Jacobi is chosen for these small problems because it needs no
// tridiagonal stage, reaches full FP64 accuracy and keeps every rotation of a round
// independent, so all threads of the CTA work on one round at a time.
#include <cuda_runtime.h>

#include <atomic>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

constexpr int EJ_THREADS = 512;
constexpr int EJ_MAX_SWEEPS = 40;

// round-robin (circle method) position j of round r for np (even) players
__device__ __forceinline__ int rr_player(int j, int r, int np) {
  return j == 0 ? 0 : 1 + (j - 1 + r) % (np - 1);
}

// A: matrix b at A + offsets[b], leading dimension lds[b] (or sizes[b] when lds == null).
// work: per matrix 2*max_size^2 doubles (copy of A and the rotation accumulator V).
__global__ void __launch_bounds__(EJ_THREADS) jacobi_eigh_kernel(
    const double* __restrict__ A_all, const int64_t* __restrict__ offsets, const int* __restrict__ sizes,
    const int* __restrict__ lds, int n_uniform, int ld_uniform, int max_size, int keep,
    double* __restrict__ evals, double* __restrict__ evecs, double* __restrict__ work) {
  const int b = blockIdx.x;
  const int n = sizes ? sizes[b] : n_uniform;
  const int lda = lds ? lds[b] : (sizes ? n : ld_uniform);
  const double* Ain = A_all + (offsets ? offsets[b] : int64_t(b) * ld_uniform * n_uniform);
  double* A = work + size_t(b) * 2 * size_t(max_size) * max_size;
  double* V = A + size_t(max_size) * max_size;
  const int tid = threadIdx.x, nt = blockDim.x;

  __shared__ double sc[512], ss[512];
  __shared__ int sp[512], sq[512];
  __shared__ double red[EJ_THREADS / 32];
  __shared__ int s_rot;
  __shared__ double s_fro;

  if (n <= 0) return;
  // copy A (ld = n) and V = I
  double fro = 0.0;
  for (int e = tid; e < n * n; e += nt) {
    int i = e / n, j = e % n;
    double v = Ain[size_t(i) * lda + j];
    A[e] = v;
    V[e] = (i == j) ? 1.0 : 0.0;
    fro += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
  if ((tid & 31) == 0) red[tid >> 5] = fro;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int w = 0; w < nt / 32; ++w) t += red[w];
    s_fro = sqrt(t);
  }
  __syncthreads();
  // off-diagonal entries below the rounding noise of the rotations (~eps*||A||) are left alone,
  // so that a sweep can end without any rotation
  const double abs_floor = 1e-300 + 2e-16 * s_fro;

  if (n > 1) {
    const int np = n + (n & 1);
    const int npairs = np / 2;
    for (int sweep = 0; sweep < EJ_MAX_SWEEPS; ++sweep) {
      if (tid == 0) s_rot = 0;
      __syncthreads();
      for (int r = 0; r < np - 1; ++r) {
        // rotation parameters for every pair of this round
        for (int k = tid; k < npairs; k += nt) {
          int p = rr_player(k, r, np), q = rr_player(np - 1 - k, r, np);
          if (p > q) { int t = p; p = q; q = t; }
          double c = 1.0, s = 0.0;
          if (q < n) {
            const double apq = A[p * n + q];
            const double app = A[p * n + p], aqq = A[q * n + q];
            if (fabs(apq) > abs_floor && fabs(apq) > 1e-16 * sqrt(fabs(app * aqq))) {
              const double theta = (aqq - app) / (2.0 * apq);
              const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(1.0 + theta * theta));
              c = 1.0 / sqrt(1.0 + t * t);
              s = t * c;
              s_rot = 1;
            }
          }
          sp[k] = p; sq[k] = q; sc[k] = c; ss[k] = s;
        }
        __syncthreads();
        // A <- A P (columns p, q of every row)
        for (int e = tid; e < npairs * n; e += nt) {
          int k = e / n, i = e % n;
          double s = ss[k];
          if (s == 0.0) continue;
          int p = sp[k], q = sq[k];
          double c = sc[k];
          double aip = A[i * n + p], aiq = A[i * n + q];
          A[i * n + p] = c * aip - s * aiq;
          A[i * n + q] = s * aip + c * aiq;
        }
        __syncthreads();
        // A <- P^T A (rows p, q of every column); V <- V P
        for (int e = tid; e < npairs * n; e += nt) {
          int k = e / n, j = e % n;
          double s = ss[k];
          if (s == 0.0) continue;
          int p = sp[k], q = sq[k];
          double c = sc[k];
          double apj = A[p * n + j], aqj = A[q * n + j];
          A[p * n + j] = c * apj - s * aqj;
          A[q * n + j] = s * apj + c * aqj;
          double vjp = V[j * n + p], vjq = V[j * n + q];
          V[j * n + p] = c * vjp - s * vjq;
          V[j * n + q] = s * vjp + c * vjq;
        }
        __syncthreads();
        for (int k = tid; k < npairs; k += nt)
          if (ss[k] != 0.0) {
            A[sp[k] * n + sq[k]] = 0.0;
            A[sq[k] * n + sp[k]] = 0.0;
          }
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
    const double di = A[i * n + i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double dj = A[j * n + j];
      rank += (dj < di) || (dj == di && j < i);
    }
    if (rank < keep) {
      ev_out[rank] = di;
      for (int row = 0; row < n; ++row) vec_out[size_t(row) * keep + rank] = V[row * n + i];
    }
  }
}

}  // namespace

int eigh_small_f64_ld(const double* A, const int64_t* offsets, const int* sizes, const int* lds,
                      int batch, int max_size, int keep, double* evals, double* evecs, double* work,
                      cudaStream_t st) {
  if (batch <= 0) return TNX_OK;
  jacobi_eigh_kernel<<<batch, EJ_THREADS, 0, st>>>(A, offsets, sizes, lds, 0, 0, max_size, keep, evals,
                                                   evecs, work);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

int eigh_small_f64_uniform(const double* A, int n, int ld, int keep, double* evals, double* evecs,
                           double* work, cudaStream_t st) {
  jacobi_eigh_kernel<<<1, EJ_THREADS, 0, st>>>(A, nullptr, nullptr, nullptr, n, ld, n, keep, evals, evecs,
                                               work);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

int eigh_small_f64(double* A, const int64_t* offsets, const int* sizes, int batch, int max_size,
                   int keep, double* evals, double* evecs, double* work, cudaStream_t st) {
  return eigh_small_f64_ld(A, offsets, sizes, nullptr, batch, max_size, keep, evals, evecs, work, st);
}

}  // namespace tnx

using namespace tnx;

extern "C" {

size_t tnx_eigh_batched_workspace_bytes(int batch, int max_size, int keep) {
  (void)keep;
  if (batch <= 0 || max_size <= 0) return 0;
  return align_up(size_t(batch) * 2 * size_t(max_size) * max_size * sizeof(double));
}

int tnx_eigh_batched(double* A, const int64_t* offsets, const int* sizes, int batch, int max_size,
                     int keep, double* evals, double* evecs, void* workspace, size_t workspace_bytes,
                     void* stream) {
  TNX_CHECK_ARG(A && offsets && sizes && evals && evecs, "null pointer");
  TNX_CHECK_ARG(batch >= 0 && max_size > 0 && keep > 0 && keep <= max_size,
                "bad batch/max_size/keep (%d, %d, %d)", batch, max_size, keep);
  TNX_CHECK_SHAPE(max_size <= 1024, "eigh: matrices larger than 1024 are not supported (got %d)",
                  max_size);
  size_t need = align_up(size_t(batch) * 2 * size_t(max_size) * max_size * sizeof(double));
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_eigh_batched: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  if (batch == 1 && keep == 1 && max_size <= 64)  // one small matrix, lowest pair: one-warp path
    return rr_lowest_f64(A, max_size, max_size, evals, evecs, as_stream(stream));
  return eigh_small_f64(A, offsets, sizes, batch, max_size, keep, evals, evecs,
                        static_cast<double*>(workspace), as_stream(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Lowest eigenpair of a small symmetric matrix (n <= 64) with one warp.
//
// GB300 issues FP64 at ~2 FMA/clock/SM, so an FP64 Jacobi on one SM costs ~n^3 * sweeps
// FP64 clocks (~100 us at n = 24). Here the Jacobi sweeps run in FP32 (64x the issue
// rate), and the lowest eigenpair is then refined in FP64 against the FP64 matrix:
//   s <- s - sum_{j != 0} v_j (v_j . r) / (lambda_j - theta),  r = A s - theta s,
// which contracts the error by ~(FP32 eigenvector error) per step; three steps reach
// FP64 accuracy for a non-degenerate lowest eigenvalue, and theta = s^T A s is FP64.
// Used for the Davidson Rayleigh-Ritz problem and the dense effective Hamiltonians
// of the chain ends.
// ---------------------------------------------------------------------------------------
namespace tnx {
namespace {

constexpr int RW_MAX = 64;

constexpr int RR_T = 128;  // threads of the Rayleigh-Ritz kernel

// Lowest eigenpair of a small symmetric matrix (n <= 64): parallel-ordered cyclic Jacobi in
// FP32 (the rotation angles of one round by one thread per pair, the row and column updates
// spread over all threads), then three FP64 correction steps of the lowest Ritz vector against
// the FP32 eigenbasis, s <- s - sum_j v_j (v_j . r) / (l_j - theta), and the FP64 Rayleigh
// quotient. FP32 rounding keeps regenerating off-diagonal entries at ~6e-8 |A|_F, so the sweeps
// stop once every off-diagonal entry is below 1e-6 |A|_F; the FP64 steps take it from there.
// Batched form: block b solves the matrix at A + b sA into eval[b sE], evec + b sV, and returns at
// once when active is given and active[b] == 0.
__global__ void __launch_bounds__(RR_T) rr_lowest_warp_kernel(const double* __restrict__ A, int n, int ld,
                                                            double* __restrict__ eval, double* __restrict__ evec,
                                                            int64_t sA, int64_t sE, int64_t sV,
                                                            const int* __restrict__ active) {
  if (active && !active[blockIdx.x]) return;
  A += int64_t(blockIdx.x) * sA;
  eval += int64_t(blockIdx.x) * sE;
  evec += int64_t(blockIdx.x) * sV;
  extern __shared__ double sm_d[];
  double* Ad = sm_d;                                      // n x n FP64
  float* Af = reinterpret_cast<float*>(Ad + n * n);       // n x (n+1) FP32
  float* Vf = Af + n * (n + 1);                           // n x (n+1) FP32
  double* s = reinterpret_cast<double*>(Vf + n * (n + 1) + ((n * (n + 1)) & 1));  // n FP64 (8-byte aligned)
  double* r = s + n;                                      // n
  double* f = r + n;                                      // n correction coefficients
  __shared__ float cs[32], ss[32];
  __shared__ int pp[32], qq[32];
  __shared__ float red[RR_T / 32];
  __shared__ double redd[RR_T / 32];
  __shared__ int s_any, s_imin;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nf = n + 1;
  float fro = 0.f;
  for (int e = tid; e < n * n; e += RR_T) {
    const int i = e / n, j = e % n;
    const double v = A[int64_t(i) * ld + j];
    Ad[e] = v;
    Af[i * nf + j] = float(v);
    Vf[i * nf + j] = (i == j) ? 1.f : 0.f;
    fro += float(v) * float(v);
  }
  for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
  if (lane == 0) red[warp] = fro;
  __syncthreads();
  fro = 0.f;
  for (int w = 0; w < RR_T / 32; ++w) fro += red[w];
  fro = sqrtf(fro);
  const float thresh = 1e-6f * fro;
  if (n > 1) {
    const int np = n + (n & 1), npairs = np / 2;
    if (tid == 0) s_any = 0;
    __syncthreads();
    for (int sweep = 0; sweep < 30; ++sweep) {
      for (int rnd = 0; rnd < np - 1; ++rnd) {
        if (tid < npairs) {
          int p = tid == 0 ? 0 : 1 + (tid - 1 + rnd) % (np - 1);
          int q = 1 + (np - 1 - tid - 1 + rnd) % (np - 1);
          if (p > q) { int t = p; p = q; q = t; }
          float c = 1.f, sn = 0.f;
          if (q < n) {
            const float apq = Af[p * nf + q], app = Af[p * nf + p], aqq = Af[q * nf + q];
            if (fabsf(apq) > thresh) {
              const float th = (aqq - app) / (2.f * apq);
              const float t = (th >= 0.f ? 1.f : -1.f) / (fabsf(th) + sqrtf(1.f + th * th));
              c = 1.f / sqrtf(1.f + t * t);
              sn = t * c;
              s_any = 1;
            }
          }
          pp[tid] = p; qq[tid] = q; cs[tid] = c; ss[tid] = sn;
        }
        __syncthreads();
        // A <- A J: columns p, q (pairs touch disjoint columns)
        for (int e = tid; e < npairs * n; e += RR_T) {
          const int k = e / n, i = e % n;
          const float sn = ss[k];
          if (sn == 0.f) continue;
          const int p = pp[k], q = qq[k];
          const float c = cs[k];
          const float a = Af[i * nf + p], b = Af[i * nf + q];
          Af[i * nf + p] = c * a - sn * b;
          Af[i * nf + q] = sn * a + c * b;
        }
        __syncthreads();
        // A <- J^T A: rows p, q (disjoint rows); V <- V J
        for (int e = tid; e < npairs * n; e += RR_T) {
          const int k = e / n, j = e % n;
          const float sn = ss[k];
          if (sn == 0.f) continue;
          const int p = pp[k], q = qq[k];
          const float c = cs[k];
          const float a = Af[p * nf + j], b = Af[q * nf + j];
          Af[p * nf + j] = c * a - sn * b;
          Af[q * nf + j] = sn * a + c * b;
          const float va = Vf[j * nf + p], vb = Vf[j * nf + q];
          Vf[j * nf + p] = c * va - sn * vb;
          Vf[j * nf + q] = sn * va + c * vb;
        }
        __syncthreads();
        if (tid < npairs && ss[tid] != 0.f) {
          Af[pp[tid] * nf + qq[tid]] = 0.f;
          Af[qq[tid] * nf + pp[tid]] = 0.f;
        }
        __syncthreads();
      }
      // every thread reads the flag before thread 0 clears it for the next sweep
      const int any = s_any;
      __syncthreads();
      if (!any) break;
      if (tid == 0) s_any = 0;
      __syncthreads();
    }
  }
  // lowest FP32 eigenvalue
  if (tid == 0) {
    int imin = 0;
    float dmin = Af[0];
    for (int i = 1; i < n; ++i)
      if (Af[i * nf + i] < dmin) { dmin = Af[i * nf + i]; imin = i; }
    s_imin = imin;
  }
  __syncthreads();
  const int imin = s_imin;
  for (int i = tid; i < n; i += RR_T) s[i] = double(Vf[i * nf + imin]);
  __syncthreads();
  const double floor = 1e-6 * (double(fro) + 1e-300);
  double theta = 0.0;
  for (int step = 0; step < 4; ++step) {
    // normalise s (n <= 64 entries: summed by every warp redundantly), r = A s, theta = s . r
    double nn = 0.0;
    for (int i = lane; i < n; i += 32) nn += s[i] * s[i];
    for (int o = 16; o > 0; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
    __syncthreads();
    const double inv = 1.0 / sqrt(nn);
    for (int i = tid; i < n; i += RR_T) s[i] *= inv;
    __syncthreads();
    double th = 0.0;
    for (int i = tid; i < n; i += RR_T) {
      double acc = 0.0;
      for (int j = 0; j < n; ++j) acc = fma(Ad[i * n + j], s[j], acc);
      r[i] = acc;
      th = fma(acc, s[i], th);
    }
    for (int o = 16; o > 0; o >>= 1) th += __shfl_xor_sync(0xffffffffu, th, o);
    if (lane == 0) redd[warp] = th;
    __syncthreads();
    th = 0.0;
    for (int w = 0; w < RR_T / 32; ++w) th += redd[w];
    theta = th;
    if (step == 3) break;
    for (int i = tid; i < n; i += RR_T) r[i] -= theta * s[i];
    __syncthreads();
    // f_j = (v_j . r) / (l_j - theta), one warp per j; (near-)degenerate partners keep f_j = 0
    for (int j = warp; j < n; j += RR_T / 32) {
      double dot = 0.0;
      for (int i = lane; i < n; i += 32) dot = fma(double(Vf[i * nf + j]), r[i], dot);
      for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
      const double den = double(Af[j * nf + j]) - theta;
      if (lane == 0) f[j] = (j != imin && fabs(den) >= floor) ? dot / den : 0.0;
    }
    __syncthreads();
    for (int i = tid; i < n; i += RR_T) {
      double acc = s[i];
      for (int j = 0; j < n; ++j) acc = fma(-f[j], double(Vf[i * nf + j]), acc);
      s[i] = acc;
    }
    __syncthreads();
  }
  if (tid == 0) eval[0] = theta;
  for (int i = tid; i < n; i += RR_T) evec[i] = s[i];
}

}  // namespace

size_t rr_lowest_smem(int n) {
  return size_t(n) * n * 8 + 2 * size_t(n) * (n + 1) * 4 + 8 + 3 * size_t(n) * 8;
}

int rr_lowest_f64(const double* A, int n, int ld, double* eval, double* evec, cudaStream_t st) {
  return rr_lowest_f64_batched(A, n, ld, 0, eval, 0, evec, 0, 1, nullptr, st);
}

int rr_lowest_f64_batched(const double* A, int n, int ld, int64_t sA, double* eval, int64_t sE, double* evec,
                          int64_t sV, int batch, const int* active, cudaStream_t st) {
  if (n > RW_MAX) {
    set_error("rr_lowest_f64: n=%d > %d", n, RW_MAX);
    return TNX_ERR_SHAPE;
  }
  if (batch <= 0) return TNX_OK;
  static std::atomic<bool> attr{false};  // idempotent setup; threads may race to it
  const size_t smem = rr_lowest_smem(RW_MAX);
  if (!attr.load()) {
    TNX_CUDA(cudaFuncSetAttribute(rr_lowest_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    attr.store(true);
  }
  profile_mark(KF_EIGH, st, true);
  rr_lowest_warp_kernel<<<batch, RR_T, rr_lowest_smem(n), st>>>(A, n, ld, eval, evec, sA, sE, sV, active);
  profile_mark(KF_EIGH, st, false);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

}  // namespace tnx
