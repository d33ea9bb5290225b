// Householder QR (FP64, or FP64-class in double-FP32) and the one-site gauge move of
// FiniteDMRG.sweep.
//
// Reference: linalg.qr (tnpy/linalg.py:26-39); the gauge move replaces the SVD split of
// MatrixProductState.split_tensor (tnpy/matrix_product_state.py:187-225) as called through
// Environment.split_tensor (:359-365). One-site DMRG never truncates there (cutoff = the
// current bond), so any orthonormal factor Q with Q R = psi gives the same state; Q and R
// differ from the SVD's U and S V^T by an orthogonal change of gauge on the bond, which
// leaves energies, environments (up to that gauge) and the next local problem unchanged.
//
// Blocked right-looking Householder on a column-major copy: each 64- (or 32-) column panel
// is factored by one thread-block cluster holding the panel in shared memory (reflectors +
// the compact-WY T factor; FP64 here, double-FP32 in qr_panel_df.cuh for the FP64-class
// modes; one-CTA kernel for panels too tall for a cluster), the trailing matrix is updated
// with three FP64 / double-FP32 GEMMs (W = V^T C, W = T^T W, C -= V W) with look-ahead (the
// next panel's columns first, the rest on a second stream). Q is formed by applying the panels
// backwards to [I; 0], or, in the FP64-class modes at large bonds, from the compact WY form of
// all reflectors with four FP64-class tensor-core GEMMs (form_q_wy).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>

#include "tnx_internal.cuh"
#include "qr_panel_df.cuh"

namespace cg = cooperative_groups;

namespace tnx {
namespace {

constexpr int QB = 32;        // panel width of the one-CTA panel kernel
constexpr int QT = 512;       // threads of the panel kernel

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

// Cluster form of the panel factorisation: the panel's rows are split over CL CTAs of one
// thread-block cluster, each holding its rows in shared memory. Column jj costs ONE cluster
// barrier: before it, every CTA publishes in its exchange slot the partial dot products of
// column jj (below its pivot) with every column c >= jj (c = jj gives the norm), the pivot
// row jj (its owner only) and the partial dot products v_a . v_{jj-1} that extend the
// compact-WY T factor by one column (LAPACK dlarft recurrence, forward/columnwise). After the
// barrier each CTA sums the CL partials in rank order, so all CTAs derive bitwise-identical
// beta, tau and v^T x_c = x_c[jj] + scale * sum_{i>jj} x_jj[i] x_c[i] without a second
// exchange, update their rows, and compute the next column's partials in the same pass.
// Slots are double-buffered, so the barrier of step jj also orders the reads of step jj-1.
//
// Each step: one thread derives the column's scalars; phase A forms v = scale * x_jj and the
// updated column jj+1 once per row (FP64 arithmetic is scarce on this part); phase B (before
// the barrier arrives) updates columns c > jj+1 and forms the partial dots; phase C (between
// arrive and wait) stores v and column jj+1 and extends T on rank 0.
constexpr int PT = 256;  // threads per CTA of the cluster panel kernel

__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
  asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory");
}

template <int NB, int CL>
__global__ void __launch_bounds__(PT) panel_cl_kernel(double* __restrict__ F, int64_t m, int64_t j0, int nb,
                                                      int ld, double* __restrict__ tau_out,
                                                      double* __restrict__ T_out) {
  constexpr int TPC = PT / NB;  // threads per panel column, interleaved over rows
  cg::cluster_group cluster = cg::this_cluster();
  const int q = int(cluster.block_rank());
  extern __shared__ double pl[];  // [NB][ld] column-major panel rows of this CTA, then vr[ld], vnr[ld]
  double* vr = pl + NB * ld;      // reflector of the current column over this CTA's rows
  double* vnr = vr + ld;          // next column after the current reflector
  __shared__ double slot[2][3 * NB];  // s[NB] partial dots, piv[NB] pivot row, z[NB] T dots
  __shared__ double S[NB], P[NB], Z[NB], taus[NB], sc[4];
  __shared__ double Ts[NB][NB + 1];  // T factor, rank 0 only, row a held by thread a
  const int tid = threadIdx.x, ci = tid / TPC, h = tid % TPC;
  const int64_t mp = m - j0;
  const int64_t rpc = (mp + CL - 1) / CL;
  const int64_t r0 = int64_t(q) * rpc;  // first panel row of this CTA
  const int rows = int(r0 >= mp ? 0 : (mp - r0 < rpc ? mp - r0 : rpc));
  for (int e = tid; e < nb * rows; e += PT) {
    const int c = e / rows, r = e % rows;
    pl[c * ld + r] = F[(j0 + c) * m + j0 + r0 + r];
  }
  __syncthreads();
  // partials of pivot 0: s[c] = sum_{row > 0} x_0 x_c, pivot row 0 from rank 0
  {
    double acc = 0.0;
    if (ci < nb) {
      const double* xc = pl + ci * ld;
      const int rs = r0 > 0 ? 0 : 1;
      for (int i = rs / TPC; i * TPC < rows; ++i) {
        const int r = i * TPC + h;
        if (r >= rs && r < rows) acc = fma(pl[r], xc[r], acc);
      }
    }
#pragma unroll
    for (int o = TPC / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (ci < nb && h == 0) {
      slot[0][ci] = acc;
      if (r0 == 0 && rows > 0) slot[0][NB + ci] = pl[ci * ld];
    }
  }
  cluster_arrive_release();
  cluster_wait_acquire();
  for (int jj = 0; jj < nb; ++jj) {
    const int par = jj & 1;
    const int owner = int(jj / rpc);
    if (tid < NB) {
      const int c = tid;
      if (c >= jj && c < nb) {
        double t = 0.0;
#pragma unroll
        for (int qq = 0; qq < CL; ++qq) t += cluster.map_shared_rank(&slot[par][0], qq)[c];
        S[c] = t;
        P[c] = cluster.map_shared_rank(&slot[par][NB], owner)[c];
      }
    } else if (tid < 2 * NB && q == 0) {
      const int a = tid - NB;
      if (a < jj - 1) {
        double t = 0.0;
#pragma unroll
        for (int qq = 0; qq < CL; ++qq) t += cluster.map_shared_rank(&slot[par][2 * NB], qq)[a];
        Z[a] = t;
      }
    }
    __syncthreads();
    // column scalars once (FP64 sqrt and divisions are slow on this part's FP64 pipe)
    if (tid == 0) {
      const double sigma = S[jj], alpha = P[jj];
      double tj = 0.0, beta = alpha, scale = 0.0;
      if (sigma != 0.0) {
        const double nrm = sqrt(alpha * alpha + sigma);
        beta = alpha >= 0.0 ? -nrm : nrm;
        tj = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      sc[0] = tj;
      sc[1] = beta;
      sc[2] = scale;
      sc[3] = jj + 1 < nb ? tj * (P[jj + 1] + scale * S[jj + 1]) : 0.0;  // w of column jj+1
      taus[jj] = tj;
    }
    __syncthreads();
    const double tj = sc[0], beta = sc[1], scale = sc[2], wn = sc[3];
    const bool has_next = jj + 1 < nb;
    double* nxt = slot[par ^ 1];
    double* xj = pl + jj * ld;
    double* xn = pl + (jj + 1) * ld;
    const int64_t lj = jj - r0;  // local row of pivot jj (outside [0, rows) if another CTA holds it)
    // ---- phase A: v_jj = scale * x_jj below the pivot (1 at it) and the updated column jj+1,
    // once per row
    for (int r = int(lj > 0 ? lj : 0) + tid; r < rows; r += PT) {
      const double v = r == lj ? 1.0 : scale * xj[r];
      vr[r] = v;
      if (has_next) vnr[r] = xn[r] - wn * v;
    }
    __syncthreads();
    // ---- phase B: update columns c > jj+1, partial dots of column jj+1 with c >= jj+1 below
    // pivot jj+1 (norm at c = jj+1), pivot row jj+1, T dots v_c . v_jj for c < jj
    double acc = 0.0;
    if (ci < nb && ci != jj) {
      double* xc = pl + ci * ld;
      const int64_t ln = lj + 1;
      const bool own_ln = ln >= 0 && ln < rows && ln % TPC == h;
      if (ci == jj + 1) {
        if (own_ln) nxt[NB + ci] = vnr[ln];
        const int rs = int(lj + 2 > 0 ? lj + 2 : 0);
        for (int i = rs / TPC; i * TPC < rows; ++i) {
          const int r = i * TPC + h;
          if (r >= rs && r < rows) acc = fma(vnr[r], vnr[r], acc);
        }
      } else if (ci > jj) {
        const double wc = tj * (P[ci] + scale * S[ci]);
        if (lj >= 0 && lj < rows && lj % TPC == h) xc[lj] -= wc;  // v_jj[jj] = 1
        if (own_ln) {
          const double val = xc[ln] - wc * vr[ln];
          xc[ln] = val;
          nxt[NB + ci] = val;  // pivot row of step jj+1
        }
        const int rs = int(lj + 2 > 0 ? lj + 2 : 0);
        for (int i = rs / TPC; i * TPC < rows; ++i) {
          const int r = i * TPC + h;
          if (r < rs || r >= rows) continue;
          const double val = xc[r] - wc * vr[r];
          xc[r] = val;
          acc = fma(vnr[r], val, acc);
        }
      } else {
        const int rs = int(lj > 0 ? lj : 0);
        for (int i = rs / TPC; i * TPC < rows; ++i) {
          const int r = i * TPC + h;
          if (r >= rs && r < rows) acc = fma(xc[r], vr[r], acc);
        }
      }
    }
#pragma unroll
    for (int o = TPC / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (ci < nb && ci != jj && h == 0) {
      if (ci > jj) nxt[ci] = acc;
      else nxt[2 * NB + ci] = acc;
    }
    cluster_arrive_release();
    __syncthreads();
    // ---- phase C: store v_jj and beta, the updated column jj+1, extend T by column jj-1
    {
      for (int r = int(lj > 0 ? lj : 0) + tid; r < rows; r += PT) {
        xj[r] = r == lj ? beta : vr[r];
        if (has_next) xn[r] = vnr[r];
      }
      if (q == 0 && jj >= 1 && tid < jj) {
        const int k = jj - 1, a = tid;
        if (a == k) {
          Ts[k][k] = taus[k];
        } else {
          double t = 0.0;
          for (int c = a; c < k; ++c) t = fma(Ts[a][c], Z[c], t);
          Ts[a][k] = -taus[k] * t;
        }
      }
    }
    // the next gather rewrites S, P and Z, which phase C of other threads still reads
    __syncthreads();
    cluster_wait_acquire();
  }
  // last T column from the final exchange
  if (q == 0 && tid >= NB && tid < 2 * NB) {
    const int a = tid - NB;
    if (a < nb - 1) {
      double t = 0.0;
#pragma unroll
      for (int qq = 0; qq < CL; ++qq) t += cluster.map_shared_rank(&slot[nb & 1][2 * NB], qq)[a];
      Z[a] = t;
    }
  }
  __syncthreads();
  if (q == 0 && tid < nb) {
    const int k = nb - 1, a = tid;
    if (a == k) {
      Ts[k][k] = taus[k];
    } else {
      double t = 0.0;
      for (int c = a; c < k; ++c) t = fma(Ts[a][c], Z[c], t);
      Ts[a][k] = -taus[k] * t;
    }
  }
  __syncthreads();
  if (q == 0) {
    for (int e = tid; e < NB * NB; e += PT) {
      const int b = e / NB, a = e % NB;  // T_out column-major, ld NB
      T_out[e] = (a <= b && b < nb) ? Ts[a][b] : 0.0;
    }
    for (int b = tid; b < NB; b += PT) tau_out[b] = b < nb ? taus[b] : 0.0;
  }
  for (int e = tid; e < nb * rows; e += PT) {
    const int c = e / rows, r = e % rows;
    F[(j0 + c) * m + j0 + r0 + r] = pl[c * ld + r];
  }
  // no CTA leaves while rank 0 may still read its slots
  cluster_arrive_release();
  cluster_wait_acquire();
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

// Two scratch sets (Vp / W1 / W2 / part): set 0 for the caller's stream, set 1 for the
// look-ahead stream of the factorisation.
struct QrWs {
  double *F, *Qc, *tau, *T, *Vp, *W1, *W2, *part;
  double *Vp2, *W1b, *W2b, *partb;
};
constexpr int QBMAX = 64;  // widest panel
constexpr int QR_SPLIT_MAX = 16;
inline int qr_nsplit(int64_t k) {
  int64_t s = (k + 127) / 128;
  return int(s < 1 ? 1 : (s > QR_SPLIT_MAX ? QR_SPLIT_MAX : s));
}
// K split of an m x n product with a long K into slices of >= 64 for up to `cap` partial
// doubles: narrow products (the next panel's update) get more, shorter slices
inline int qr_nsplit_cap(int64_t k, int64_t m, int64_t n, int64_t cap) {
  int64_t s = (k + 63) / 64;
  const int64_t c = cap / (m * n);
  if (s > c) s = c;
  if (s > 64) s = 64;
  return int(s < 1 ? 1 : s);
}

// sized for QBMAX-wide panels, which also covers QB-wide ones
size_t qr_layout(int64_t m, int64_t n, void* base, QrWs* w) {
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += align_up(bytes); return o; };
  const int64_t np = (n + QBMAX - 1) / QBMAX;
  size_t oF = take(m * n * 8), oQ = take(m * n * 8), otau = take(np * QBMAX * 8),
         oT = take(np * QBMAX * QBMAX * 8), oV = take(m * QBMAX * 8), oW1 = take(n * QBMAX * 8),
         oW2 = take(n * QBMAX * 8), oP = take(size_t(QR_SPLIT_MAX) * n * QBMAX * 8), oV2 = take(m * QBMAX * 8),
         oW1b = take(n * QBMAX * 8), oW2b = take(n * QBMAX * 8), oPb = take(size_t(QR_SPLIT_MAX) * n * QBMAX * 8);
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
    w->Vp2 = reinterpret_cast<double*>(b + oV2);
    w->W1b = reinterpret_cast<double*>(b + oW1b);
    w->W2b = reinterpret_cast<double*>(b + oW2b);
    w->partb = reinterpret_cast<double*>(b + oPb);
  }
  return off;
}

// Leading dimension of a CTA's panel rows: a multiple of 16 doubles plus the threads per column,
// so the TPC row-interleaved threads of 16 / TPC neighbouring columns hit distinct banks.
inline int panel_ld(int64_t rpc, int tpc) { return int((rpc + 15) / 16 * 16 + tpc); }

// One-time attribute setup of a cluster panel instantiation: largest dynamic shared memory it
// may use and whether a cluster of CL CTAs with that much shared memory can be scheduled.
struct PanelKernelInfo {
  bool ok = false;
  size_t max_dyn = 0;
};

// DF selects the double-FP32 panel (FP64-class modes), otherwise the FP64 one
using PanelFn = void (*)(double*, int64_t, int64_t, int, int, double*, double*);
template <int NB, int CL, bool DF>
PanelFn panel_fn() {
  if constexpr (DF) return qrdf::panel_df_kernel<NB, CL>;
  else return panel_cl_kernel<NB, CL>;
}
template <bool DF>
constexpr int panel_threads() {
  return DF ? qrdf::DPT : PT;
}

template <int NB, int CL, bool DF>
const PanelKernelInfo& panel_info() {
  static PanelKernelInfo info;
  static std::once_flag once;
  std::call_once(once, [] {
    PanelFn k = panel_fn<NB, CL, DF>();
    cudaFuncAttributes fa{};
    int dev = 0, optin = 0;
    if (cudaFuncGetAttributes(&fa, k) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    const size_t dyn = size_t(optin) > fa.sharedSizeBytes ? size_t(optin) - fa.sharedSizeBytes : 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dyn)) != cudaSuccess ||
        (CL > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)) {
      cudaGetLastError();
      return;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CL;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(CL);
    cfg.blockDim = dim3(panel_threads<DF>());
    cfg.dynamicSmemBytes = dyn;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, k, &cfg) != cudaSuccess) {
      cudaGetLastError();
      clusters = 0;
    }
    info.max_dyn = dyn;
    info.ok = clusters > 0;
  });
  return info;
}

template <int NB, int CL, bool DF>
int launch_panel(double* F, int64_t m, int64_t j0, int nb, double* tau, double* T, cudaStream_t st) {
  const int64_t rpc = (m - j0 + CL - 1) / CL;
  const int ld = panel_ld(rpc, panel_threads<DF>() / NB);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(panel_threads<DF>());
  cfg.dynamicSmemBytes = size_t(NB + 2) * ld * sizeof(double);
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  TNX_CUDA(cudaLaunchKernelEx(&cfg, panel_fn<NB, CL, DF>(), F, m, j0, nb, ld, tau, T));
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

// Panel plan of one QR: width nb (64 or 32), cluster size cl (16 or 8; 0 = one-CTA panel,
// for panels too tall for a cluster's shared memory) and arithmetic (df: the double-FP32 panel
// of the FP64-class modes). Wider panels give the trailing-update GEMMs a longer K; 16-CTA
// clusters (where the device schedules them) spread the panel over twice the SMs of the
// portable 8. TNX_QR_CLUSTER=8 or 16 restricts the cluster size, TNX_QR_PANEL=fp64 keeps
// FP64 panels in the FP64-class modes and TNX_QR_NB=32 selects 32-column double-FP32 panels
// (tuning).
struct PanelPlan {
  int nb, cl;
  bool df;
};

template <int NB, int CL, bool DF>
bool panel_fits(int64_t m) {
  const PanelKernelInfo& info = panel_info<NB, CL, DF>();
  const int64_t rpc = (m + CL - 1) / CL;
  return info.ok && size_t(NB + 2) * panel_ld(rpc, panel_threads<DF>() / NB) * sizeof(double) <= info.max_dyn;
}

PanelPlan plan_panels(int64_t m, bool df) {
  static const int only = [] {
    const char* e = getenv("TNX_QR_CLUSTER");
    return e ? atoi(e) : 0;
  }();
  static const bool fp64_panels = [] {
    const char* e = getenv("TNX_QR_PANEL");
    return e && std::string(e) == "fp64";
  }();
  static const int nb_only = [] {
    const char* e = getenv("TNX_QR_NB");
    return e ? atoi(e) : 0;
  }();
  const bool c8 = only == 0 || only == 8, c16 = only == 0 || only == 16;
  if (df && !fp64_panels) {
    if (nb_only == 32 && c16 && panel_fits<32, 16, true>(m)) return {32, 16, true};
    if (c16 && panel_fits<64, 16, true>(m)) return {64, 16, true};
    if (c8 && panel_fits<64, 8, true>(m)) return {64, 8, true};
  }
  if (c16 && panel_fits<64, 16, false>(m)) return {64, 16, false};
  if (c8 && panel_fits<64, 8, false>(m)) return {64, 8, false};
  if (c16 && panel_fits<32, 16, false>(m)) return {32, 16, false};
  if (c8 && panel_fits<32, 8, false>(m)) return {32, 8, false};
  return {QB, 0, false};
}

int factor_panel(const PanelPlan& pp, double* F, int64_t m, int64_t j0, int nb, double* tau, double* T,
                 cudaStream_t st) {
  profile_mark(KF_QR_PANEL, st, true);
  int rc = TNX_OK;
  if (pp.cl == 0) {
    panel_kernel<<<1, QT, 0, st>>>(F, m, j0, nb, tau, T);
    TNX_LAUNCH_CHECK();
  } else if (pp.df) {
    rc = pp.nb == 32   ? launch_panel<32, 16, true>(F, m, j0, nb, tau, T, st)
         : pp.cl == 16 ? launch_panel<64, 16, true>(F, m, j0, nb, tau, T, st)
                       : launch_panel<64, 8, true>(F, m, j0, nb, tau, T, st);
  } else if (pp.nb == 64) {
    rc = pp.cl == 16 ? launch_panel<64, 16, false>(F, m, j0, nb, tau, T, st)
                     : launch_panel<64, 8, false>(F, m, j0, nb, tau, T, st);
  } else {
    rc = pp.cl == 16 ? launch_panel<32, 16, false>(F, m, j0, nb, tau, T, st)
                     : launch_panel<32, 8, false>(F, m, j0, nb, tau, T, st);
  }
  profile_mark(KF_QR_PANEL, st, false);
  // algorithmic work of a Householder panel of nb columns over the m - j0 remaining rows:
  // 2 (m - j0) nb^2 - 2 nb^3 / 3 flops, plus nb^2 (m - j0) for the T factor
  const double mr = double(m - j0), b = double(nb);
  profile_work(KF_QR_PANEL, 3.0 * mr * b * b - 2.0 * b * b * b / 3.0, 8.0 * mr * b * 2.0);
  return rc;
}

// ---- next-panel update in double-FP32, three short launches (FP64-class modes) ----------
//
// The update of the next panel's columns by H_p sits on the factorisation's critical path
// between two panels. As three general GEMM launches (split-K V^T C with its reduction, T^T W,
// C -= V W) it is latency-bound at 64 x 64 x (m - j0); these kernels spread each phase over
// all rows of the GPU instead: NR_ROWS-row chunks of V^T C per CTA, a fixed-order reduction of
// the chunk partials fused with T^T W, and the rank-nb update per row chunk.
constexpr int NR_ROWS = 16;   // rows of V and C per CTA in the partial and update kernels
constexpr int NR_T = 512;     // threads of those kernels

// part[c][b][a] = sum over rows r of chunk c of V[r][a] C[r][b]  (a < nb, b < nc <= 64; df2)
__global__ void __launch_bounds__(NR_T) nar_partial_kernel(const double* __restrict__ Vp, int64_t mp, int nb,
                                                           const double* __restrict__ C, int64_t ldc, int nc,
                                                           qrdf::df2* __restrict__ part) {
  __shared__ qrdf::df2 Vs[NR_ROWS][64], Cs[NR_ROWS][64];
  const int tid = threadIdx.x;
  const int64_t r0 = int64_t(blockIdx.x) * NR_ROWS;
#pragma unroll
  for (int e = tid; e < NR_ROWS * 64; e += NR_T) {
    const int r = e % NR_ROWS, c = e / NR_ROWS;
    const int64_t gr = r0 + r;
    qrdf::df2 v = {0.f, 0.f}, x = {0.f, 0.f};
    if (gr < mp) {
      if (c < nb) split_df(Vp[int64_t(c) * mp + gr], v.h, v.l);
      if (c < nc) split_df(C[int64_t(c) * ldc + gr], x.h, x.l);
    }
    Vs[r][c] = v;
    Cs[r][c] = x;
  }
  __syncthreads();
  constexpr int PJ = 64 * 64 / NR_T, PS = NR_T / 64;  // outputs per thread, their column stride
  const int a = tid & 63, bq = tid >> 6;              // outputs (a, bq + PS j)
  qrdf::df2 acc[PJ];
#pragma unroll
  for (int j = 0; j < PJ; ++j) acc[j] = {0.f, 0.f};
#pragma unroll 4
  for (int r = 0; r < NR_ROWS; ++r) {
    const qrdf::df2 v = Vs[r][a];
#pragma unroll
    for (int j = 0; j < PJ; ++j) qrdf::acc(acc[j], v, Cs[r][bq + PS * j]);
  }
  qrdf::df2* out = part + int64_t(blockIdx.x) * 64 * 64;
#pragma unroll
  for (int j = 0; j < PJ; ++j) out[(bq + PS * j) * 64 + a] = qrdf::norm(acc[j]);
}

// W2[a][b] = sum_{k <= a} T(k, a) W[k][b] with W[k][b] = sum over chunks c of part[c][b][k]; one
// CTA of 256 threads per column b: thread (g, k) sums the chunks c = g (mod 4) in order
// (coalesced loads, four in flight), the four group sums are added in group order, and T
// (column-major, ld NB, upper triangular) is staged in shared memory by all threads at once
constexpr int NRED_T = 256;
__global__ void __launch_bounds__(NRED_T) nar_reduce_kernel(const qrdf::df2* __restrict__ part, int nchunk, int nb,
                                                            const double* __restrict__ T, int NB,
                                                            qrdf::df2* __restrict__ W2) {
  __shared__ qrdf::df2 Wg[4][64];
  __shared__ double Ts[64][65];
  const int b = blockIdx.x, tid = threadIdx.x, k = tid & 63, g = tid >> 6;
#pragma unroll
  for (int i = 0; i < 64 * 64 / NRED_T; ++i) {
    const int e = tid + i * NRED_T, col = e / 64, row = e % 64;  // T(row, col)
    Ts[col][row] = (row < nb && col < nb) ? T[col * NB + row] : 0.0;
  }
  const qrdf::df2* pb = part + b * 64 + k;
  qrdf::df2 s = {0.f, 0.f};
  int c = g;
  for (; c + 12 < nchunk; c += 16) {
    const qrdf::df2 p0 = pb[int64_t(c) * 4096], p1 = pb[int64_t(c + 4) * 4096], p2 = pb[int64_t(c + 8) * 4096],
                    p3 = pb[int64_t(c + 12) * 4096];
    s = qrdf::add(s, p0);
    s = qrdf::add(s, p1);
    s = qrdf::add(s, p2);
    s = qrdf::add(s, p3);
  }
  for (; c < nchunk; c += 4) s = qrdf::add(s, pb[int64_t(c) * 4096]);
  Wg[g][k] = s;
  __syncthreads();
  if (tid < 64) {
    Wg[0][k] = qrdf::add(qrdf::add(Wg[0][k], Wg[1][k]), qrdf::add(Wg[2][k], Wg[3][k]));
  }
  __syncthreads();
  if (tid < 64) {
    const int a = tid;
    qrdf::df2 t = {0.f, 0.f};
    if (a < nb)
      for (int kk = 0; kk <= a; ++kk) {
        qrdf::df2 tk;
        split_df(Ts[a][kk], tk.h, tk.l);
        qrdf::acc(t, tk, Wg[0][kk]);
      }
    W2[a * 64 + b] = qrdf::norm(t);
  }
}

// C[r][b] -= sum_a V[r][a] W2[a][b] for the rows of one chunk
__global__ void __launch_bounds__(NR_T) nar_update_kernel(const double* __restrict__ Vp, int64_t mp, int nb,
                                                          const qrdf::df2* __restrict__ W2, double* __restrict__ C,
                                                          int64_t ldc, int nc) {
  __shared__ qrdf::df2 Ws[64][65], Vs[NR_ROWS][65];
  const int tid = threadIdx.x;
  const int64_t r0 = int64_t(blockIdx.x) * NR_ROWS;
#pragma unroll
  for (int i = 0; i < 64 * 64 / NR_T; ++i) {
    const int e = tid + i * NR_T;
    Ws[e / 64][e % 64] = W2[e];
  }
#pragma unroll
  for (int e = tid; e < NR_ROWS * 64; e += NR_T) {
    const int r = e % NR_ROWS, c = e / NR_ROWS;
    const int64_t gr = r0 + r;
    qrdf::df2 v = {0.f, 0.f};
    if (gr < mp && c < nb) split_df(Vp[int64_t(c) * mp + gr], v.h, v.l);
    Vs[r][c] = v;
  }
  __syncthreads();
  constexpr int UJ = NR_ROWS * 64 / NR_T, US = NR_T / NR_ROWS;  // outputs per thread, column stride
  const int r = tid % NR_ROWS, bq = tid / NR_ROWS;              // outputs (r, bq + US j)
  qrdf::df2 acc[UJ];
#pragma unroll
  for (int j = 0; j < UJ; ++j) acc[j] = {0.f, 0.f};
  for (int a = 0; a < nb; ++a) {
    const qrdf::df2 v = Vs[r][a];
#pragma unroll
    for (int j = 0; j < UJ; ++j) qrdf::acc(acc[j], v, Ws[a][bq + US * j]);
  }
  const int64_t gr = r0 + r;
  if (gr < mp)
#pragma unroll
    for (int j = 0; j < UJ; ++j) {
      const int b = bq + US * j;
      if (b < nc) {
        const qrdf::df2 s = qrdf::norm(acc[j]);
        C[int64_t(b) * ldc + gr] -= join_df(s.h, s.l);
      }
    }
}

// C -= V T^T V^T C for a block of nc <= 64 columns (the next panel), double-FP32 arithmetic;
// part holds ceil(mp / NR_ROWS) * 64 * 64 float pairs, W2 64 * 64
int apply_panel_narrow(int64_t m, int64_t mp, int nb, int NB, const double* Vp, const double* Tp, double* C, int nc,
                       qrdf::df2* W2, qrdf::df2* part, cudaStream_t st) {
  const int nchunk = int((mp + NR_ROWS - 1) / NR_ROWS);
  profile_mark(KF_F64_GEMM, st, true);
  nar_partial_kernel<<<nchunk, NR_T, 0, st>>>(Vp, mp, nb, C, m, nc, part);
  TNX_LAUNCH_CHECK();
  nar_reduce_kernel<<<nc, NRED_T, 0, st>>>(part, nchunk, nb, Tp, NB, W2);
  TNX_LAUNCH_CHECK();
  nar_update_kernel<<<nchunk, NR_T, 0, st>>>(Vp, mp, nb, W2, C, m, nc);
  TNX_LAUNCH_CHECK();
  profile_mark(KF_F64_GEMM, st, false);
  profile_work(KF_F64_GEMM, 4.0 * double(mp) * nb * nc + 2.0 * double(nb) * nb * nc,
               8.0 * (2.0 * mp * nb + 2.0 * mp * nc));
  return TNX_OK;
}

// C -= V T^T V^T C for the mp x nc column-major block C (ld m): the trailing update of one
// panel (V: mp x nb column-major in Vp, T: column-major ld NB)
// With `oz` (FP64-class modes, large trailing blocks) the two large products run on the Ozaki
// GEMM: V^T C split over K (QR_OZ_SPLIT ranges), C^T -= W2^T V^T with K = nb.
constexpr int QR_OZ_SPLIT = 16;
inline bool bulk_on_oz(int64_t mp, int64_t nc) { return mp >= 256 && nc >= 128; }
size_t bulk_oz_bytes(int64_t m, int64_t n) {
  return std::max(gemm_oz_ex_workspace_bytes(QBMAX, n, m, 1, QR_OZ_SPLIT), gemm_oz_ex_workspace_bytes(n, m, QBMAX, 1, 1));
}

int apply_panel_t(int64_t m, int64_t mp, int nb, int NB, const double* Vp, const double* Tp, double* C, int64_t nc,
                  double* W1, double* W2, double* part, int64_t part_cap, cudaStream_t st, bool df,
                  void* oz = nullptr, size_t ozb = 0) {
  if (nc <= 0) return TNX_OK;
  const bool on_oz = df && oz && bulk_on_oz(mp, nc);
  // Row-major views: C (column-major mp x nc, ld m) is C^T (nc x mp, ld m), V is V^T (nb x mp).
  // W1 (nb x nc) = V^T C  (short output rows, long K: split over K; finer for narrow C)
  if (on_oz) {
    TNX_TRY(gemm_oz_ex(false, true, nb, nc, mp, 1.0, Vp, mp, 0, C, m, 0, 0.0, W1, nc, 0, 1, QR_OZ_SPLIT, nullptr, oz,
                       ozb, st));
  } else {
    const int ns = nc <= NB ? qr_nsplit_cap(mp, nb, nc, part_cap) : qr_nsplit(mp);
    TNX_TRY(gemm_f64_splitk(false, true, nb, nc, mp, 1.0, Vp, mp, C, m, 0.0, W1, nc, ns, part, st, df));
  }
  // W2 = T^T W1   (T column-major with ld NB is T^T row-major)
  TNX_TRY(gemm_fp64_class(df, false, false, nb, nc, nb, 1.0, Tp, NB, 0, W1, nc, 0, 0.0, W2, nc, 0, 1, st));
  // C -= V W2, i.e. C^T -= W2^T V^T
  if (on_oz) {
    TNX_TRY(gemm_oz_ex(true, false, nc, mp, nb, -1.0, W2, nc, 0, Vp, mp, 0, 1.0, C, m, 0, 1, 1, nullptr, oz, ozb, st));
  } else {
    TNX_TRY(gemm_fp64_class(df, true, false, nc, mp, nb, -1.0, W2, nc, 0, Vp, mp, 0, 1.0, C, m, 0, 1, st));
  }
  return TNX_OK;
}

// Look-ahead stream and its two events, one set per host thread and device, created on first use
// and kept for the thread's lifetime.
// `hi` (the highest stream priority) carries the factorisation's critical path (panels and the
// next panel's update), `aux` (a middle priority) the bulk trailing updates, `wy` (the lowest)
// the compact-WY bookkeeping of the FP64-class gauge move: when several have blocks waiting,
// the SMs that free up go to the critical path first (a 16-CTA panel cluster needs 16 free SMs
// of one GPC at once).
struct LookAhead {
  cudaStream_t aux = nullptr, hi = nullptr, wy = nullptr;
  cudaEvent_t ev_v = nullptr, ev_r = nullptr, ev_h = nullptr, ev_w = nullptr;
};

int look_ahead(LookAhead** out) {
  constexpr int MAXDEV = 64;
  thread_local LookAhead la[MAXDEV];
  int dev = 0;
  TNX_CUDA(cudaGetDevice(&dev));
  TNX_CHECK_ARG(dev >= 0 && dev < MAXDEV, "device index %d out of range", dev);
  LookAhead& l = la[dev];
  if (!l.aux) {
    int least = 0, greatest = 0;
    TNX_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    TNX_CUDA(cudaStreamCreateWithPriority(&l.hi, cudaStreamNonBlocking, greatest));
    TNX_CUDA(cudaStreamCreateWithPriority(&l.aux, cudaStreamNonBlocking, (least + greatest) / 2));
    TNX_CUDA(cudaStreamCreateWithPriority(&l.wy, cudaStreamNonBlocking, least));
    TNX_CUDA(cudaEventCreateWithFlags(&l.ev_v, cudaEventDisableTiming));
    TNX_CUDA(cudaEventCreateWithFlags(&l.ev_r, cudaEventDisableTiming));
    TNX_CUDA(cudaEventCreateWithFlags(&l.ev_h, cudaEventDisableTiming));
    TNX_CUDA(cudaEventCreateWithFlags(&l.ev_w, cudaEventDisableTiming));
  }
  *out = &l;
  return TNX_OK;
}

}  // namespace

// ---- Q from the compact WY form of all n reflectors (FP64-class modes, large QRs) ----------
//
// H_0 H_1 ... H_{n-1} = I - V Tf V^T with V (m x n, unit lower trapezoidal) and Tf (n x n, upper
// triangular). Tf grows by one panel per factorisation step, on the look-ahead stream while the
// next panels are factored (dlarft's recurrence applied a panel at a time):
//   Tf[0:j0, p] = -Tf[0:j0, 0:j0] (V[:, 0:j0]^T V_p) T_p,   Tf[p, p] = T_p,
// so that only the last panel's column block is left when the factorisation ends. Then
//   Q = [I; 0] - V (Tf V_top^T),   V_top = rows 0..n-1 of V,
// two FP64-class GEMMs on the tensor cores (Ozaki). The backward accumulation this replaces is
// 16 steps of narrow K = 64 products on the FP32 pipe after the factorisation.
struct WyWs {
  double *V, *S, *Tf, *X, *Y;  // S: the n x 64 block V^T V_p of the current step, Y: S T_p
  double* part;                // split-K scratch of the V^T V_p products
  void* oz;                    // Ozaki scratch of the WY stream (and of X and Q after it)
  size_t oz_bytes;
  void* oz_bulk;               // Ozaki scratch of the bulk trailing updates (look-ahead stream)
  size_t oz_bulk_bytes;
};

inline bool wy_applies(int64_t m, int64_t n, bool df) { return df && use_oz(n, n, m) && n >= 256; }

size_t wy_oz_bytes(int64_t m, int64_t n) {
  size_t b = gemm_oz_workspace_bytes(n, n, n);  // X
  auto mx = [&](size_t x) { b = x > b ? x : b; };
  mx(gemm_oz_ex_workspace_bytes(n, QBMAX, m, 1, QR_OZ_SPLIT));  // V[:, 0:j0]^T V_p
  mx(gemm_oz_ex_workspace_bytes(n, QBMAX, n, 1, QR_OZ_SPLIT));  // Tf Y
  mx(gemm_oz_workspace_bytes(m, n, n));  // Q, row-major output
  mx(gemm_oz_workspace_bytes(n, m, n));  // Q, column-major output
  return b;
}

size_t wy_layout(int64_t m, int64_t n, void* base, WyWs* w) {
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += align_up(bytes); return o; };
  const size_t oV = take(size_t(m) * n * 8), oS = take(size_t(n) * n * 8), oT = take(size_t(n) * n * 8),
               oX = take(size_t(n) * n * 8), oY = take(size_t(n) * n * 8 / 4),
               oP = take(size_t(QR_SPLIT_MAX) * n * QBMAX * 8), obz = wy_oz_bytes(m, n), oZ = take(obz),
               obb = bulk_oz_bytes(m, n), oB = take(obb);
  if (w && base) {
    char* b = static_cast<char*>(base);
    w->V = reinterpret_cast<double*>(b + oV);
    w->S = reinterpret_cast<double*>(b + oS);
    w->Tf = reinterpret_cast<double*>(b + oT);
    w->X = reinterpret_cast<double*>(b + oX);
    w->Y = reinterpret_cast<double*>(b + oY);
    w->part = reinterpret_cast<double*>(b + oP);
    w->oz = b + oZ;
    w->oz_bytes = obz;
    w->oz_bulk = b + oB;
    w->oz_bulk_bytes = obb;
  }
  return off;
}

// V column block p (full height, ld m: zero above the diagonal, unit diagonal) from F
__global__ void v_block_kernel(const double* __restrict__ F, int64_t m, int64_t j0, int nb, double* __restrict__ V) {
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < m * nb; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = j0 + e / m, r = e % m;
    V[c * m + r] = r < c ? 0.0 : (r == c ? 1.0 : F[c * m + r]);
  }
}

// Tf diagonal block p (row-major, ld n) = T_p (column-major, ld NB), zero below its diagonal
__global__ void t_block_kernel(const double* __restrict__ Tp, int NB, int nb, double* __restrict__ Tf, int64_t n,
                               int64_t j0) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nb * nb; e += gridDim.x * blockDim.x) {
    const int a = e / nb, b = e % nb;
    Tf[(j0 + a) * n + j0 + b] = a <= b ? Tp[b * NB + a] : 0.0;
  }
}

// Append panel p (columns j0 .. j0+nb) to V and Tf: V's column block, then
// Tf[0:j0, j0:j0+nb] = -Tf[0:j0, 0:j0] (V[:, 0:j0]^T V_p) T_p and the diagonal block T_p.
// part: split-K scratch of at least QR_SPLIT_MAX * n * QBMAX doubles.
int wy_append_panel(int64_t m, int64_t n, int NB, int64_t j0, int nb, const double* F, const double* Tp,
                    const WyWs& y, double* part, cudaStream_t st) {
  v_block_kernel<<<blocks_for(m * nb), 256, 0, st>>>(F, m, j0, nb, y.V);
  TNX_LAUNCH_CHECK();
  t_block_kernel<<<(nb * nb + 255) / 256, 256, 0, st>>>(Tp, NB, nb, y.Tf, n, j0);
  TNX_LAUNCH_CHECK();
  if (j0 == 0) return TNX_OK;
  // S (j0 x nb, ld nb) = V[:, 0:j0]^T V_p over rows >= j0, where V_p is nonzero
  // (op(A)(i, k) = V(j0 + k, i); op(B)(k, j) = V(j0 + k, j0 + j))
  const int64_t K = m - j0;
  const bool on_oz = j0 >= 256;
  if (on_oz) {
    TNX_TRY(gemm_oz_ex(false, true, j0, nb, K, 1.0, y.V + j0, m, 0, y.V + j0 * m + j0, m, 0, 0.0, y.S, nb, 0, 1,
                       QR_OZ_SPLIT, nullptr, y.oz, y.oz_bytes, st));
  } else {
    TNX_TRY(gemm_f64_splitk(false, true, j0, nb, K, 1.0, y.V + j0, m, y.V + j0 * m + j0, m, 0.0, y.S, nb,
                            qr_nsplit_cap(K, j0, nb, int64_t(QR_SPLIT_MAX) * n * QBMAX), part, st, true));
  }
  // Y (j0 x nb, ld nb) = S T_p   (op(B)(k, j) = T_p(k, j) = Tp[j NB + k])
  TNX_TRY(gemm_fp64_class(true, false, true, j0, nb, nb, 1.0, y.S, nb, 0, Tp, NB, 0, 0.0, y.Y, nb, 0, 1, st));
  // Tf[0:j0, j0:j0+nb] = -Tf[0:j0, 0:j0] Y  (K = j0 long, nb = 64 wide: split over K)
  if (on_oz) {
    TNX_TRY(gemm_oz_ex(false, false, j0, nb, j0, -1.0, y.Tf, n, 0, y.Y, nb, 0, 0.0, y.Tf + j0, n, 0, 1, QR_OZ_SPLIT,
                       nullptr, y.oz, y.oz_bytes, st));
  } else {
    TNX_TRY(gemm_f64_splitk(false, false, j0, nb, j0, -1.0, y.Tf, n, y.Y, nb, 0.0, y.Tf + j0, n,
                            qr_nsplit_cap(j0, j0, nb, int64_t(QR_SPLIT_MAX) * n * QBMAX), y.part, st, true));
  }
  return TNX_OK;
}

// Factor the column-major m x n matrix in w.F (m >= n) and form Q (column-major) in w.Qc.
//
// Factorisation with look-ahead: after panel p is factored, a high-priority stream updates only
// the next panel's columns with H_p and factors panel p+1, while the low-priority look-ahead
// stream applies H_p to all columns beyond panel p+1 (the bulk of the flops); the 16 SMs of a
// panel no longer leave the rest of the GPU idle. Panel p+2's columns (part of that bulk) are
// used only after the look-ahead stream's update of step p has completed. V is double-buffered
// between the streams; both join the caller's stream at the end.
int qr_colmajor(int64_t m, int64_t n, QrWs& w, cudaStream_t st, bool df = false, bool form_q = true,
                const WyWs* wy = nullptr) {
  const PanelPlan pp = plan_panels(m, df);
  const int NB = pp.nb;
  const int64_t np = (n + NB - 1) / NB;
  const int64_t part_cap = int64_t(QR_SPLIT_MAX) * n * QBMAX;  // doubles of each split-K scratch
  LookAhead* la = nullptr;
  TNX_TRY(look_ahead(&la));
  cudaStream_t cs = la->hi;  // critical path
  // both streams start after everything queued on the caller's stream
  TNX_CUDA(cudaEventRecord(la->ev_r, st));
  TNX_CUDA(cudaStreamWaitEvent(la->aux, la->ev_r, 0));
  TNX_CUDA(cudaStreamWaitEvent(cs, la->ev_r, 0));
  if (wy) {
    TNX_CUDA(cudaStreamWaitEvent(la->wy, la->ev_r, 0));
    TNX_CUDA(cudaMemsetAsync(wy->Tf, 0, size_t(n) * n * 8, la->wy));
  }
  TNX_TRY(factor_panel(pp, w.F, m, 0, int(n < NB ? n : NB), w.tau, w.T, cs));
  for (int64_t p = 0; p < np; ++p) {
    const int64_t j0 = p * NB;
    const int nb = int(n - j0 < NB ? n - j0 : NB);
    double* Tp = w.T + p * NB * NB;  // column-major nb x nb, ld NB
    const int64_t mp = m - j0, nc = n - j0 - nb;
    if (nc <= 0) break;
    double* Vp = (p & 1) ? w.Vp2 : w.Vp;
    panel_v_kernel<<<blocks_for(mp * nb), 256, 0, cs>>>(w.F, m, j0, nb, Vp);
    TNX_LAUNCH_CHECK();
    const int nb1 = int(nc < NB ? nc : NB);  // next panel
    const int64_t rest = nc - nb1;
    double* Cn = w.F + (j0 + nb) * m + j0;
    if (rest > 0 || wy) TNX_CUDA(cudaEventRecord(la->ev_v, cs));  // V_p, T_p ready; panel p+2's columns updated
    if (rest > 0) {
      TNX_CUDA(cudaStreamWaitEvent(la->aux, la->ev_v, 0));
      TNX_TRY(apply_panel_t(m, mp, nb, NB, Vp, Tp, Cn + int64_t(nb1) * m, rest, w.W1b, w.W2b, w.partb, part_cap,
                            la->aux, df, wy ? wy->oz_bulk : nullptr, wy ? wy->oz_bulk_bytes : 0));
      TNX_CUDA(cudaEventRecord(la->ev_r, la->aux));  // panel p+2's columns updated by H_p
    }
    // panel p joins the compact WY form on the lowest-priority stream, off the critical path
    if (wy) {
      TNX_CUDA(cudaStreamWaitEvent(la->wy, la->ev_v, 0));
      TNX_TRY(wy_append_panel(m, n, NB, j0, nb, w.F, Tp, *wy, wy->part, la->wy));
    }
    const bool narrow = df && n >= 64 && (mp + NR_ROWS - 1) / NR_ROWS * 64 * 64 <= part_cap;
    if (narrow) {
      TNX_TRY(apply_panel_narrow(m, mp, nb, NB, Vp, Tp, Cn, nb1, reinterpret_cast<qrdf::df2*>(w.W2),
                                 reinterpret_cast<qrdf::df2*>(w.part), cs));
    } else {
      TNX_TRY(apply_panel_t(m, mp, nb, NB, Vp, Tp, Cn, nb1, w.W1, w.W2, w.part, part_cap, cs, df));
    }
    TNX_TRY(factor_panel(pp, w.F, m, j0 + nb, nb1, w.tau + (p + 1) * NB, w.T + (p + 1) * NB * NB, cs));
    // the next step reads panel p+2's columns and rewrites the other V buffer
    if (rest > 0) TNX_CUDA(cudaStreamWaitEvent(cs, la->ev_r, 0));
  }
  // join both streams back into the caller's (also when they received no work: keeps stream
  // capture balanced)
  TNX_CUDA(cudaEventRecord(la->ev_r, la->aux));
  TNX_CUDA(cudaStreamWaitEvent(st, la->ev_r, 0));
  TNX_CUDA(cudaEventRecord(la->ev_h, cs));
  TNX_CUDA(cudaStreamWaitEvent(st, la->ev_h, 0));
  if (wy) {  // the WY stream's work so far, then the last panel
    TNX_CUDA(cudaEventRecord(la->ev_w, la->wy));
    TNX_CUDA(cudaStreamWaitEvent(st, la->ev_w, 0));
    const int64_t j0 = (np - 1) * NB;
    TNX_TRY(wy_append_panel(m, n, NB, j0, int(n - j0), w.F, w.T + (np - 1) * NB * NB, *wy, wy->part, st));
  }
  if (!form_q) return TNX_OK;
  // Q = H_0 H_1 ... [I; 0]: apply panels last to first to the columns >= j0
  eye_kernel<<<blocks_for(m * n), 256, 0, st>>>(w.Qc, m, n);
  TNX_LAUNCH_CHECK();
  for (int64_t p = np - 1; p >= 0; --p) {
    const int64_t j0 = p * NB;
    const int nb = int(n - j0 < NB ? n - j0 : NB);
    const int64_t mp = m - j0, nq = n - j0;
    const double* Tp = w.T + p * NB * NB;
    panel_v_kernel<<<blocks_for(mp * nb), 256, 0, st>>>(w.F, m, j0, nb, w.Vp);
    TNX_LAUNCH_CHECK();
    double* Qs = w.Qc + j0 * m + j0;  // column-major mp x nq, ld m
    // W1 (nb x nq) = V^T Qs
    TNX_TRY(gemm_f64_splitk(false, true, nb, nq, mp, 1.0, w.Vp, mp, Qs, m, 0.0, w.W1, nq, qr_nsplit(mp), w.part,
                            st, df));
    // W2 = T W1   (op(A) = T: the row-major view of column-major T is T^T, so transpose it)
    TNX_TRY(gemm_fp64_class(df, true, false, nb, nq, nb, 1.0, Tp, NB, 0, w.W1, nq, 0, 0.0, w.W2, nq, 0, 1, st));
    // Qs -= V W2
    TNX_TRY(gemm_fp64_class(df, true, false, nq, mp, nb, -1.0, w.W2, nq, 0, w.Vp, mp, 0, 1.0, Qs, m, 0, 1, st));
  }
  return TNX_OK;
}

// FP64-class product on the Ozaki GEMM without the autotuner (the gauge move runs the Q
// formation and the R A product concurrently, which would distort a first-call timing); the
// autotuned path where the Ozaki GEMM does not apply
int gemm_oz_direct(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
                   const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* oz, size_t ozb,
                   cudaStream_t st) {
  if (oz && use_oz(m, n, k) && ozb >= gemm_oz_workspace_bytes(m, n, k))
    return gemm_oz(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, oz, ozb, st);
  return gemm_fp64_class_oz(true, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, oz, ozb, st);
}

// Q (m x n) from V and Tf (built during the factorisation): row-major (ld n) when q_rowmajor,
// otherwise column-major (ld m)
int form_q_wy(int64_t m, int64_t n, const WyWs& y, double* Q, bool q_rowmajor, cudaStream_t st) {
  // X = Tf V_top^T  (op(B)(k, j) = V(j, k) = V[k m + j])
  TNX_TRY(gemm_oz_direct(false, false, n, n, n, 1.0, y.Tf, n, y.V, m, 0.0, y.X, n, y.oz, y.oz_bytes, st));
  if (q_rowmajor) {
    // Q = [I; 0] - V X  (op(A)(i, k) = V(i, k) = V[k m + i])
    eye_kernel<<<blocks_for(m * n), 256, 0, st>>>(Q, n, m);
    TNX_LAUNCH_CHECK();
    TNX_TRY(gemm_oz_direct(true, false, m, n, n, -1.0, y.V, m, y.X, n, 1.0, Q, n, y.oz, y.oz_bytes, st));
  } else {
    // Q^T = [I, 0] - X^T V^T  (row-major n x m)
    eye_kernel<<<blocks_for(m * n), 256, 0, st>>>(Q, m, n);
    TNX_LAUNCH_CHECK();
    TNX_TRY(gemm_oz_direct(true, false, n, m, n, -1.0, y.X, n, y.V, m, 1.0, Q, m, y.oz, y.oz_bytes, st));
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

// slices of the R * neighbour product on the tensor cores (FP64-class modes)
static size_t gauge_oz_bytes(int direction, int64_t chi_l, int64_t d, int64_t chi_r, int64_t chi_other) {
  const int64_t n = direction == 1 ? chi_r : chi_l;
  const int64_t gm = direction == 1 ? n : chi_other * d, gn = direction == 1 ? d * chi_other : n;
  return use_oz(gm, gn, n) ? gemm_oz_workspace_bytes(gm, gn, n) : 0;
}

size_t tnx_gauge_move_workspace_bytes(int direction, int64_t chi_l, int64_t d, int64_t chi_r,
                                      int64_t chi_other) {
  int64_t m = direction == 1 ? chi_l * d : d * chi_r;
  int64_t n = direction == 1 ? chi_r : chi_l;
  int64_t nb_elems = direction == 1 ? chi_r * d * chi_other : chi_other * d * chi_l;
  return qr_layout(m, n, nullptr, nullptr) + align_up(n * n * 8) + align_up(nb_elems * 8) +
         align_up(gauge_oz_bytes(direction, chi_l, d, chi_r, chi_other)) +
         (wy_applies(m, n, true) ? wy_layout(m, n, nullptr, nullptr) : 0);
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
  const int64_t nb_elems = direction == 1 ? chi_r * d * chi_other : chi_other * d * chi_l;
  const size_t ozb = df ? gauge_oz_bytes(direction, chi_l, d, chi_r, chi_other) : 0;
  char* after_tmp = reinterpret_cast<char*>(tmp) + align_up(nb_elems * 8);
  void* oz = ozb ? static_cast<void*>(after_tmp) : nullptr;
  // Q from the compact WY form on the tensor cores (FP64-class modes, large bonds)
  const bool wy = wy_applies(m, n, df);
  WyWs wys{};
  if (wy) wy_layout(m, n, after_tmp + align_up(gauge_oz_bytes(direction, chi_l, d, chi_r, chi_other)), &wys);
  cudaStream_t st = as_stream(stream);
  dim3 tb(32, 8);
  if (direction == 1) {
    // psi (chi_l d x chi_r) row-major -> column-major
    transpose_kernel<<<dim3(unsigned((n + 31) / 32), unsigned((m + 31) / 32)), tb, 0, st>>>(A_site, m, n, w.F);
    TNX_LAUNCH_CHECK();
    TNX_TRY(qr_colmajor(m, n, w, st, df, !wy, wy ? &wys : nullptr));
    const int64_t nc = d * chi_other;
    if (wy) {
      // A_next (chi_r x d chi_other) <- R A_next on the look-ahead stream while Q forms on the
      // caller's stream
      LookAhead* la = nullptr;
      TNX_TRY(look_ahead(&la));
      TNX_CUDA(cudaEventRecord(la->ev_r, st));
      TNX_CUDA(cudaStreamWaitEvent(la->aux, la->ev_r, 0));
      extract_r_kernel<<<blocks_for(n * n), 256, 0, la->aux>>>(w.F, m, n, Rb);
      TNX_LAUNCH_CHECK();
      TNX_TRY(gemm_oz_direct(false, false, n, nc, n, 1.0, Rb, n, A_nb, nc, 0.0, tmp, nc, oz, ozb, la->aux));
      TNX_CUDA(cudaMemcpyAsync(A_nb, tmp, n * nc * 8, cudaMemcpyDeviceToDevice, la->aux));
      TNX_TRY(form_q_wy(m, n, wys, A_site, true, st));
      TNX_CUDA(cudaEventRecord(la->ev_v, la->aux));
      TNX_CUDA(cudaStreamWaitEvent(st, la->ev_v, 0));
    } else {
      transpose_kernel<<<dim3(unsigned((m + 31) / 32), unsigned((n + 31) / 32)), tb, 0, st>>>(w.Qc, n, m, A_site);
      TNX_LAUNCH_CHECK();
      extract_r_kernel<<<blocks_for(n * n), 256, 0, st>>>(w.F, m, n, Rb);
      TNX_LAUNCH_CHECK();
      // A_next (chi_r x d chi_other) <- R A_next
      TNX_TRY(gemm_fp64_class_oz(df, false, false, n, nc, n, 1.0, Rb, n, A_nb, nc, 0.0, tmp, nc, oz, ozb, st));
      TNX_CUDA(cudaMemcpyAsync(A_nb, tmp, n * nc * 8, cudaMemcpyDeviceToDevice, st));
    }
  } else {
    // psi (chi_l x d chi_r) row-major == psi^T (d chi_r x chi_l) column-major
    TNX_CUDA(cudaMemcpyAsync(w.F, A_site, m * n * 8, cudaMemcpyDeviceToDevice, st));
    TNX_TRY(qr_colmajor(m, n, w, st, df, !wy, wy ? &wys : nullptr));
    const int64_t mr = chi_other * d;
    // Q column-major (d chi_r x chi_l) == Q^T row-major (chi_l x d chi_r)
    if (wy) {
      // A_prev (chi_other d x chi_l) <- A_prev R^T on the look-ahead stream while Q forms on the
      // caller's stream
      LookAhead* la = nullptr;
      TNX_TRY(look_ahead(&la));
      TNX_CUDA(cudaEventRecord(la->ev_r, st));
      TNX_CUDA(cudaStreamWaitEvent(la->aux, la->ev_r, 0));
      extract_r_kernel<<<blocks_for(n * n), 256, 0, la->aux>>>(w.F, m, n, Rb);
      TNX_LAUNCH_CHECK();
      TNX_TRY(gemm_oz_direct(false, true, mr, n, n, 1.0, A_nb, n, Rb, n, 0.0, tmp, n, oz, ozb, la->aux));
      TNX_CUDA(cudaMemcpyAsync(A_nb, tmp, mr * n * 8, cudaMemcpyDeviceToDevice, la->aux));
      TNX_TRY(form_q_wy(m, n, wys, A_site, false, st));
      TNX_CUDA(cudaEventRecord(la->ev_v, la->aux));
      TNX_CUDA(cudaStreamWaitEvent(st, la->ev_v, 0));
    } else {
      TNX_CUDA(cudaMemcpyAsync(A_site, w.Qc, m * n * 8, cudaMemcpyDeviceToDevice, st));
      extract_r_kernel<<<blocks_for(n * n), 256, 0, st>>>(w.F, m, n, Rb);
      TNX_LAUNCH_CHECK();
      // A_prev (chi_other d x chi_l) <- A_prev R^T
      TNX_TRY(gemm_fp64_class_oz(df, false, true, mr, n, n, 1.0, A_nb, n, Rb, n, 0.0, tmp, n, oz, ozb, st));
      TNX_CUDA(cudaMemcpyAsync(A_nb, tmp, mr * n * 8, cudaMemcpyDeviceToDevice, st));
    }
  }
  return TNX_OK;
}

}  // extern "C"
