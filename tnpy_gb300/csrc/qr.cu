// Householder QR (FP64) and the one-site gauge move of FiniteDMRG.sweep.
//
// Reference: linalg.qr (tnpy/linalg.py:26-39); the gauge move replaces the SVD split of
// MatrixProductState.split_tensor (tnpy/matrix_product_state.py:187-225) as called through
// Environment.split_tensor (:359-365). One-site DMRG never truncates there (cutoff = the
// current bond), so any orthonormal factor Q with Q R = psi gives the same state; Q and R
// differ from the SVD's U and S V^T by an orthogonal change of gauge on the bond, which
// leaves energies, environments (up to that gauge) and the next local problem unchanged.
//
// Blocked right-looking Householder on a column-major copy: each 32-column panel is
// factored by one CTA (reflectors + the compact-WY T factor), the trailing matrix is
// updated with three FP64 GEMMs (W = V^T C, W = T^T W, C -= V W), and Q is formed by
// applying the panels backwards to [I; 0].
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "tnx_internal.cuh"

namespace cg = cooperative_groups;

namespace tnx {
namespace {

constexpr int QB = 32;        // panel width
constexpr int QT = 512;       // threads of the panel kernel
constexpr int QC = 8;         // CTAs of the cluster panel kernel
constexpr int QCT = 256;      // threads per CTA of the cluster panel kernel
constexpr int QC_ROWS = 512;  // panel rows held per CTA (shared memory)

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Factor panel columns [j0, j0+nb) of the column-major m x n matrix F (ld = m), rows >= j0.
// On exit: R entries on/above the diagonal, reflector v_j below the diagonal (v_j[j] = 1
// implicit), tau[j], and T (nb x nb, column-major, upper triangular) with
// H_j0 ... H_{j0+nb-1} = I - V T V^T.
__global__ void __launch_bounds__(QT) panel_kernel(double* __restrict__ F, int64_t m, int64_t j0, int nb,
                                                  double* __restrict__ tau, double* __restrict__ T) {
  __shared__ double red[QT / 32][QB + 1];
  __shared__ double wv[QB];
  __shared__ double s_beta, s_tau, s_scale;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarp = QT / 32;
  for (int jj = 0; jj < nb; ++jj) {
    const int64_t j = j0 + jj;
    double* col = F + j * m;
    // sigma = ||col[j+1:]||^2
    double part = 0.0;
    for (int64_t i = j + 1 + tid; i < m; i += QT) part = fma(col[i], col[i], part);
    part = warp_sum(part);
    if (lane == 0) red[warp][0] = part;
    __syncthreads();
    if (tid == 0) {
      double sigma = 0.0;
      for (int w = 0; w < nwarp; ++w) sigma += red[w][0];
      const double alpha = col[j];
      if (sigma == 0.0) {
        s_tau = 0.0;
        s_beta = alpha;
        s_scale = 0.0;
      } else {
        const double nrm = sqrt(alpha * alpha + sigma);
        const double beta = alpha >= 0.0 ? -nrm : nrm;
        s_tau = (beta - alpha) / beta;
        s_beta = beta;
        s_scale = 1.0 / (alpha - beta);
      }
    }
    __syncthreads();
    const double tj = s_tau;
    if (tj != 0.0)
      for (int64_t i = j + 1 + tid; i < m; i += QT) col[i] *= s_scale;
    if (tid == 0) {
      col[j] = s_beta;
      tau[jj] = tj;
    }
    __syncthreads();
    // apply H_j = I - tau v v^T to the panel columns jj+1 .. nb-1
    const int rem = nb - jj - 1;
    if (tj != 0.0 && rem > 0) {
      double acc[QB];
#pragma unroll
      for (int c = 0; c < QB; ++c) acc[c] = 0.0;
      for (int64_t i = j + tid; i < m; i += QT) {
        const double vi = (i == j) ? 1.0 : col[i];
#pragma unroll
        for (int c = 0; c < QB; ++c)
          if (c < rem) acc[c] = fma(vi, F[(j + 1 + c) * m + i], acc[c]);
      }
#pragma unroll
      for (int c = 0; c < QB; ++c) {
        if (c < rem) {
          double v = warp_sum(acc[c]);
          if (lane == 0) red[warp][c] = v;
        }
      }
      __syncthreads();
      if (tid < rem) {
        double s = 0.0;
        for (int w = 0; w < nwarp; ++w) s += red[w][tid];
        wv[tid] = tj * s;
      }
      __syncthreads();
      for (int64_t i = j + tid; i < m; i += QT) {
        const double vi = (i == j) ? 1.0 : col[i];
        for (int c = 0; c < rem; ++c) F[(j + 1 + c) * m + i] -= wv[c] * vi;
      }
    }
    __syncthreads();
  }
  // T factor: T[jj][jj] = tau_jj, T[0:jj, jj] = -tau_jj T[0:jj,0:jj] (V[:,0:jj]^T v_jj)
  // Gram entries G[a][b] = v_a . v_b for a < b
  __shared__ double G[QB][QB + 1];
  for (int pair = warp; pair < nb * nb; pair += nwarp) {
    const int a = pair / nb, b = pair % nb;
    if (a >= b) continue;
    const int64_t ja = j0 + a, jb = j0 + b;
    double s = 0.0;
    for (int64_t i = jb + lane; i < m; i += 32) {
      const double va = F[ja * m + i];              // i >= jb > ja: stored part of v_a
      const double vb = (i == jb) ? 1.0 : F[jb * m + i];
      s = fma(va, vb, s);
    }
    s = warp_sum(s);
    if (lane == 0) G[a][b] = s;
  }
  __syncthreads();
  if (tid == 0) {
    for (int b = 0; b < nb; ++b) {
      const double tb = tau[b];
      for (int a = 0; a < b; ++a) {
        double s = 0.0;
        for (int c = a; c < b; ++c) s += T[c * QB + a] * G[c][b];  // T[a][c] * G[c][b]
        T[b * QB + a] = -tb * s;
      }
      T[b * QB + b] = tb;
      for (int a = b + 1; a < QB; ++a) T[b * QB + a] = 0.0;
    }
    for (int b = nb; b < QB; ++b)
      for (int a = 0; a < QB; ++a) T[b * QB + a] = 0.0;
  }
}

// Cluster form of panel_kernel: the panel's rows are split over QC CTAs of one thread-block
// cluster, each holding its rows in shared memory. Per column, the partial norms and the
// partial dot products of the reflector with the remaining columns are exchanged through
// distributed shared memory with two cluster barriers, so the FP64 work of a panel is
// spread over QC SMs instead of one. Every CTA combines the partials in the same order, so
// all CTAs compute bitwise-identical reflector coefficients.
__global__ void __cluster_dims__(QC, 1, 1) __launch_bounds__(QCT)
    panel_cluster_kernel(double* __restrict__ F, int64_t m, int64_t j0, int nb, double* __restrict__ tau,
                         double* __restrict__ T) {
  cg::cluster_group cluster = cg::this_cluster();
  const int q = int(cluster.block_rank());
  extern __shared__ double pl[];  // [QB][QC_ROWS] column-major panel rows of this CTA
  __shared__ double sig[2], alph[2], dots[2][QB];
  __shared__ double gram[QB][QB + 1];
  __shared__ double s_tau[QB];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = QCT / 32;
  const int64_t mp = m - j0;
  const int64_t rpc = (mp + QC - 1) / QC;
  const int64_t r0 = int64_t(q) * rpc;                          // first panel row of this CTA
  const int rows = int(r0 >= mp ? 0 : (mp - r0 < rpc ? mp - r0 : rpc));
  for (int e = tid; e < nb * rows; e += QCT) {
    const int c = e / rows, r = e % rows;
    pl[c * QC_ROWS + r] = F[(j0 + c) * m + j0 + r0 + r];
  }
  __syncthreads();
  for (int jj = 0; jj < nb; ++jj) {
    const int par = jj & 1;
    const int64_t jrow = jj;  // pivot row in panel coordinates
    // -- partial sigma over rows > pivot; the owner of the pivot row publishes alpha
    double part = 0.0;
    for (int r = tid; r < rows; r += QCT) {
      const int64_t gr = r0 + r;
      if (gr > jrow) {
        const double x = pl[jj * QC_ROWS + r];
        part = fma(x, x, part);
      }
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    __shared__ double red[NW];
    if (lane == 0) red[warp] = part;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < NW; ++w) t += red[w];
      sig[par] = t;
      if (jrow >= r0 && jrow < r0 + rows) alph[par] = pl[jj * QC_ROWS + (jrow - r0)];
    }
    cluster.sync();
    const int owner = int(jrow / rpc);
    // one warp gathers the QC partial norms and alpha over DSMEM and publishes them locally
    __shared__ double s_sigma, s_alpha;
    if (warp == 0) {
      double v = lane < QC ? *cluster.map_shared_rank(&sig[par], lane) : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) {
        // fixed-order sum would differ from the tree sum across CTAs only if they used
        // different orders; every CTA runs this same reduction, so results are identical
        s_sigma = v;
        s_alpha = *cluster.map_shared_rank(&alph[par], owner);
      }
    }
    __syncthreads();
    const double sigma = s_sigma;
    const double alpha = s_alpha;
    double tj, beta, scale;
    if (sigma == 0.0) {
      tj = 0.0;
      beta = alpha;
      scale = 0.0;
    } else {
      const double nrm = sqrt(alpha * alpha + sigma);
      beta = alpha >= 0.0 ? -nrm : nrm;
      tj = (beta - alpha) / beta;
      scale = 1.0 / (alpha - beta);
    }
    // -- reflector v in place (v_pivot = 1 implicit; the pivot slot keeps beta = R_jj)
    if (tj != 0.0)
      for (int r = tid; r < rows; r += QCT)
        if (r0 + r > jrow) pl[jj * QC_ROWS + r] *= scale;
    if (tid == 0) {
      s_tau[jj] = tj;
      if (jrow >= r0 && jrow < r0 + rows) pl[jj * QC_ROWS + (jrow - r0)] = beta;
    }
    __syncthreads();
    // -- partial dots of v with the remaining columns (warp per column, lanes over rows)
    const int rem = nb - jj - 1;
    for (int c = warp; c < rem; c += NW) {
      double acc = 0.0;
      if (tj != 0.0)
        for (int r = lane; r < rows; r += 32) {
          const int64_t gr = r0 + r;
          if (gr < jrow) continue;
          const double vi = gr == jrow ? 1.0 : pl[jj * QC_ROWS + r];
          acc = fma(vi, pl[(jj + 1 + c) * QC_ROWS + r], acc);
        }
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) dots[par][c] = acc;
    }
    cluster.sync();
    if (tj != 0.0 && rem > 0) {
      __shared__ double wv[QB];
      if (tid < rem) {
        double t = 0.0;
        for (int qq = 0; qq < QC; ++qq) t += *cluster.map_shared_rank(&dots[par][tid], qq);
        wv[tid] = tj * t;
      }
      __syncthreads();
      for (int e = tid; e < rem * rows; e += QCT) {
        const int c = e / rows, r = e % rows;
        const int64_t gr = r0 + r;
        if (gr < jrow) continue;
        const double vi = gr == jrow ? 1.0 : pl[jj * QC_ROWS + r];
        pl[(jj + 1 + c) * QC_ROWS + r] -= wv[c] * vi;
      }
    }
    __syncthreads();
  }
  // -- partial Gram of the reflectors, G[a][b] = v_a . v_b (a < b), reduced on rank 0
  for (int pr = warp; pr < nb * nb; pr += NW) {
    const int a = pr / nb, b = pr % nb;
    if (a >= b) continue;
    double acc = 0.0;
    for (int r = lane; r < rows; r += 32) {
      const int64_t gr = r0 + r;
      if (gr < b) continue;
      const double va = pl[a * QC_ROWS + r];  // gr >= b > a: stored part of v_a
      const double vb = gr == b ? 1.0 : pl[b * QC_ROWS + r];
      acc = fma(va, vb, acc);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) gram[a][b] = acc;
  }
  cluster.sync();
  __shared__ double G[QB][QB + 1];
  if (q == 0) {
    // sum the partial Gram matrices of all CTAs, one (a, b) pair per thread
    for (int pr = tid; pr < nb * nb; pr += QCT) {
      const int a = pr / nb, b = pr % nb;
      if (a >= b) continue;
      double t = 0.0;
      for (int qq = 0; qq < QC; ++qq) t += cluster.map_shared_rank(&gram[0][0], qq)[a * (QB + 1) + b];
      G[a][b] = t;
    }
    __syncthreads();
  }
  if (q == 0 && tid == 0) {
    for (int b = 0; b < nb; ++b) {
      const double tb = s_tau[b];
      tau[b] = tb;
      for (int a = 0; a < b; ++a) {
        double t = 0.0;
        for (int c = a; c < b; ++c) t += T[c * QB + a] * G[c][b];
        T[b * QB + a] = -tb * t;
      }
      T[b * QB + b] = tb;
      for (int a = b + 1; a < QB; ++a) T[b * QB + a] = 0.0;
    }
    for (int b = nb; b < QB; ++b)
      for (int a = 0; a < QB; ++a) T[b * QB + a] = 0.0;
  }
  // write the factored rows back; the last barrier keeps every CTA's shared memory alive
  // until rank 0 has read the Gram partials
  for (int e = tid; e < nb * rows; e += QCT) {
    const int c = e / rows, r = e % rows;
    F[(j0 + c) * m + j0 + r0 + r] = pl[c * QC_ROWS + r];
  }
  cluster.sync();
}

// dst (row-major rows x cols) <-> col-major transposed copy
__global__ void transpose_kernel(const double* __restrict__ src, int64_t rows, int64_t cols,
                                 double* __restrict__ dst) {
  __shared__ double tile[32][33];
  const int64_t r0 = int64_t(blockIdx.y) * 32, c0 = int64_t(blockIdx.x) * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[k][threadIdx.x] = src[r * cols + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[c * rows + r] = tile[threadIdx.x][k];
  }
}

// Q (column-major m x n) = [I; 0]
__global__ void eye_kernel(double* __restrict__ Q, int64_t m, int64_t n) {
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < m * n;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = e / m, r = e % m;
    Q[e] = (r == c) ? 1.0 : 0.0;
  }
}

// R (row-major n x n) = upper triangle of F (column-major, ld m)
__global__ void extract_r_kernel(const double* __restrict__ F, int64_t m, int64_t n, double* __restrict__ R) {
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < n * n;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = e / n, c = e % n;
    R[e] = (r <= c) ? F[c * m + r] : 0.0;
  }
}

// V panel (column-major (m-j0) x nb, ld m) with the implicit unit diagonal and zeros above
__global__ void panel_v_kernel(const double* __restrict__ F, int64_t m, int64_t j0, int nb,
                               double* __restrict__ Vp) {
  const int64_t mp = m - j0;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < mp * nb;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = e / mp, r = e % mp;
    double v;
    if (r < c) v = 0.0;
    else if (r == c) v = 1.0;
    else v = F[(j0 + c) * m + j0 + r];
    Vp[c * mp + r] = v;
  }
}

unsigned blocks_for(int64_t total) {
  int64_t b = (total + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  return unsigned(b < 1 ? 1 : b);
}

struct QrWs {
  double *F, *Qc, *tau, *T, *Vp, *W1, *W2, *part;
};
constexpr int QR_SPLIT_MAX = 16;
inline int qr_nsplit(int64_t k) {
  int64_t s = (k + 255) / 256;
  return int(s < 1 ? 1 : (s > QR_SPLIT_MAX ? QR_SPLIT_MAX : s));
}

size_t qr_layout(int64_t m, int64_t n, void* base, QrWs* w) {
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += align_up(bytes); return o; };
  const int64_t np = (n + QB - 1) / QB;
  size_t oF = take(m * n * 8), oQ = take(m * n * 8), otau = take(np * QB * 8), oT = take(np * QB * QB * 8),
         oV = take(m * QB * 8), oW1 = take(n * QB * 8), oW2 = take(n * QB * 8),
         oP = take(size_t(QR_SPLIT_MAX) * n * QB * 8);
  if (w && base) {
    char* b = static_cast<char*>(base);
    w->F = reinterpret_cast<double*>(b + oF);
    w->Qc = reinterpret_cast<double*>(b + oQ);
    w->tau = reinterpret_cast<double*>(b + otau);
    w->T = reinterpret_cast<double*>(b + oT);
    w->Vp = reinterpret_cast<double*>(b + oV);
    w->W1 = reinterpret_cast<double*>(b + oW1);
    w->W2 = reinterpret_cast<double*>(b + oW2);
    w->part = reinterpret_cast<double*>(b + oP);
  }
  return off;
}

}  // namespace

// Factor the column-major m x n matrix in w.F (m >= n) and form Q (column-major) in w.Qc.
int qr_colmajor(int64_t m, int64_t n, QrWs& w, cudaStream_t st, bool df = false) {
  const int64_t np = (n + QB - 1) / QB;
  for (int64_t p = 0; p < np; ++p) {
    const int64_t j0 = p * QB;
    const int nb = int(n - j0 < QB ? n - j0 : QB);
    if (m - j0 <= int64_t(QC) * QC_ROWS) {
      static bool attr = false;
      const size_t smem = size_t(QB) * QC_ROWS * sizeof(double);
      if (!attr) {
        TNX_CUDA(cudaFuncSetAttribute(panel_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        attr = true;
      }
      profile_mark(KF_QR_PANEL, st, true);
      panel_cluster_kernel<<<QC, QCT, smem, st>>>(w.F, m, j0, nb, w.tau + p * QB, w.T + p * QB * QB);
      profile_mark(KF_QR_PANEL, st, false);
    } else {
      profile_mark(KF_QR_PANEL, st, true);
      panel_kernel<<<1, QT, 0, st>>>(w.F, m, j0, nb, w.tau + p * QB, w.T + p * QB * QB);
      profile_mark(KF_QR_PANEL, st, false);
    }
    TNX_LAUNCH_CHECK();
    const int64_t mp = m - j0, nc = n - j0 - nb;
    if (nc > 0) {
      panel_v_kernel<<<blocks_for(mp * nb), 256, 0, st>>>(w.F, m, j0, nb, w.Vp);
      TNX_LAUNCH_CHECK();
      double* C = w.F + (j0 + nb) * m + j0;  // column-major mp x nc, ld m
      // W1^T (nc x nb) = C^T V  (thin output, long K: split over K)
      TNX_TRY(gemm_f64_splitk(false, true, nc, nb, mp, 1.0, C, m, w.Vp, mp, 0.0, w.W1, nb, qr_nsplit(mp), w.part,
                              st, df));
      // W2^T = W1^T T   (T column-major nb x nb with ld QB == row-major T^T)
      TNX_TRY(gemm_fp64_class(df, false, true, nc, nb, nb, 1.0, w.W1, nb, 0, w.T + p * QB * QB, QB, 0, 0.0, w.W2,
                              nb, 0, 1, st));
      // C^T -= W2^T V^T
      TNX_TRY(gemm_fp64_class(df, false, false, nc, mp, nb, -1.0, w.W2, nb, 0, w.Vp, mp, 0, 1.0, C, m, 0, 1, st));
    }
  }
  // Q = H_0 H_1 ... [I; 0]: apply panels last to first to the columns >= j0
  eye_kernel<<<blocks_for(m * n), 256, 0, st>>>(w.Qc, m, n);
  TNX_LAUNCH_CHECK();
  for (int64_t p = np - 1; p >= 0; --p) {
    const int64_t j0 = p * QB;
    const int nb = int(n - j0 < QB ? n - j0 : QB);
    const int64_t mp = m - j0, nq = n - j0;
    panel_v_kernel<<<blocks_for(mp * nb), 256, 0, st>>>(w.F, m, j0, nb, w.Vp);
    TNX_LAUNCH_CHECK();
    double* Qs = w.Qc + j0 * m + j0;  // column-major mp x nq, ld m
    // W1^T (nq x nb) = Qs^T V
    TNX_TRY(gemm_f64_splitk(false, true, nq, nb, mp, 1.0, Qs, m, w.Vp, mp, 0.0, w.W1, nb, qr_nsplit(mp), w.part,
                            st, df));
    // W2^T = W1^T T^T  -> B = T^T: op(B)[k][n] = T[n][k] = Tcm[k*QB + n] -> row-major, ld QB
    TNX_TRY(gemm_fp64_class(df, false, false, nq, nb, nb, 1.0, w.W1, nb, 0, w.T + p * QB * QB, QB, 0, 0.0, w.W2,
                            nb, 0, 1, st));
    // Qs^T -= W2^T V^T
    TNX_TRY(gemm_fp64_class(df, false, false, nq, mp, nb, -1.0, w.W2, nb, 0, w.Vp, mp, 0, 1.0, Qs, m, 0, 1, st));
  }
  return TNX_OK;
}

}  // namespace tnx

using namespace tnx;

extern "C" {

size_t tnx_qr_workspace_bytes(int64_t m, int64_t n) { return qr_layout(m, n, nullptr, nullptr); }

int tnx_qr(const double* M, int64_t m, int64_t n, double* Q, double* R, void* workspace,
           size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(M && Q && R, "null pointer");
  TNX_CHECK_ARG(m > 0 && n > 0, "non-positive size");
  TNX_CHECK_SHAPE(m >= n, "tnx_qr needs m >= n (got %lld x %lld)", (long long)m, (long long)n);
  QrWs w;
  size_t need = qr_layout(m, n, workspace, &w);
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_qr: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  dim3 tb(32, 8);
  transpose_kernel<<<dim3(unsigned((n + 31) / 32), unsigned((m + 31) / 32)), tb, 0, st>>>(M, m, n, w.F);
  TNX_LAUNCH_CHECK();
  TNX_TRY(qr_colmajor(m, n, w, st));
  // Q row-major m x n = transpose of the column-major n x m view
  transpose_kernel<<<dim3(unsigned((m + 31) / 32), unsigned((n + 31) / 32)), tb, 0, st>>>(w.Qc, n, m, Q);
  TNX_LAUNCH_CHECK();
  extract_r_kernel<<<blocks_for(n * n), 256, 0, st>>>(w.F, m, n, R);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

size_t tnx_gauge_move_workspace_bytes(int direction, int64_t chi_l, int64_t d, int64_t chi_r,
                                      int64_t chi_other) {
  int64_t m = direction == 1 ? chi_l * d : d * chi_r;
  int64_t n = direction == 1 ? chi_r : chi_l;
  int64_t nb_elems = direction == 1 ? chi_r * d * chi_other : chi_other * d * chi_l;
  return qr_layout(m, n, nullptr, nullptr) + align_up(n * n * 8) + align_up(nb_elems * 8);
}

int tnx_gauge_move(int direction, double* A_site, double* A_nb, int64_t chi_l, int64_t d, int64_t chi_r,
                   int64_t chi_other, int precision, void* workspace, size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  const bool df = use_df64(precision);
  TNX_CHECK_ARG(A_site && A_nb, "null pointer");
  TNX_CHECK_ARG(direction == 1 || direction == -1, "direction must be +1 or -1");
  TNX_CHECK_ARG(chi_l > 0 && d > 0 && chi_r > 0 && chi_other > 0, "non-positive size");
  const int64_t m = direction == 1 ? chi_l * d : d * chi_r;
  const int64_t n = direction == 1 ? chi_r : chi_l;
  TNX_CHECK_SHAPE(m >= n, "gauge move needs the split bond (%lld) <= the fused dimension (%lld)",
                  (long long)n, (long long)m);
  size_t need = tnx_gauge_move_workspace_bytes(direction, chi_l, d, chi_r, chi_other);
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_gauge_move: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  QrWs w;
  size_t qbytes = qr_layout(m, n, workspace, &w);
  double* Rb = reinterpret_cast<double*>(static_cast<char*>(workspace) + qbytes);
  double* tmp = reinterpret_cast<double*>(static_cast<char*>(workspace) + qbytes + align_up(n * n * 8));
  cudaStream_t st = as_stream(stream);
  dim3 tb(32, 8);
  if (direction == 1) {
    // psi (chi_l d x chi_r) row-major -> column-major
    transpose_kernel<<<dim3(unsigned((n + 31) / 32), unsigned((m + 31) / 32)), tb, 0, st>>>(A_site, m, n, w.F);
    TNX_LAUNCH_CHECK();
    TNX_TRY(qr_colmajor(m, n, w, st, df));
    transpose_kernel<<<dim3(unsigned((m + 31) / 32), unsigned((n + 31) / 32)), tb, 0, st>>>(w.Qc, n, m, A_site);
    TNX_LAUNCH_CHECK();
    extract_r_kernel<<<blocks_for(n * n), 256, 0, st>>>(w.F, m, n, Rb);
    TNX_LAUNCH_CHECK();
    // A_next (chi_r x d chi_other) <- R A_next
    const int64_t nc = d * chi_other;
    TNX_TRY(gemm_fp64_class(df, false, false, n, nc, n, 1.0, Rb, n, 0, A_nb, nc, 0, 0.0, tmp, nc, 0, 1, st));
    TNX_CUDA(cudaMemcpyAsync(A_nb, tmp, n * nc * 8, cudaMemcpyDeviceToDevice, st));
  } else {
    // psi (chi_l x d chi_r) row-major == psi^T (d chi_r x chi_l) column-major
    TNX_CUDA(cudaMemcpyAsync(w.F, A_site, m * n * 8, cudaMemcpyDeviceToDevice, st));
    TNX_TRY(qr_colmajor(m, n, w, st, df));
    // Q column-major (d chi_r x chi_l) == Q^T row-major (chi_l x d chi_r)
    TNX_CUDA(cudaMemcpyAsync(A_site, w.Qc, m * n * 8, cudaMemcpyDeviceToDevice, st));
    extract_r_kernel<<<blocks_for(n * n), 256, 0, st>>>(w.F, m, n, Rb);
    TNX_LAUNCH_CHECK();
    // A_prev (chi_other d x chi_l) <- A_prev R^T
    const int64_t mr = chi_other * d;
    TNX_TRY(gemm_fp64_class(df, false, true, mr, n, n, 1.0, A_nb, n, 0, Rb, n, 0, 0.0, tmp, n, 0, 1, st));
    TNX_CUDA(cudaMemcpyAsync(A_nb, tmp, mr * n * 8, cudaMemcpyDeviceToDevice, st));
  }
  return TNX_OK;
}

}  // extern "C"
