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
  return eigh_small_f64(A, offsets, sizes, batch, max_size, keep, evals, evecs,
                        static_cast<double*>(workspace), as_stream(stream));
}

}  // extern "C"
