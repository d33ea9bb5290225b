// Many independent chains swept in lockstep: every kernel of a site update spans all chains.
//
// Replaces the per-chain loop of FiniteDMRG.run (tnpy/finite_dmrg.py:214-257) run once per
// chain (independent disorder realisations of the same shape: equal n, bond dimensions, MPO
// bond and physical dimension). Chain c's tensors sit at a fixed stride from chain 0's in
// stacked arrays ([B][...] per site), so that
//   * the one-site matvec is two strided-batched GEMMs (FP64 or double-FP32, tile autotuned)
//     around one batched MPO contraction;
//   * the Davidson eigensolver expands every chain's basis in the same launches: block-per-chain
//     Gram-Schmidt (two classical passes), batched Rayleigh-Ritz (one CTA per chain), Ritz
//     vector, residual and diagonal-preconditioned correction, and a convergence kernel that
//     clears a chain's bit in the active mask once its residual meets the tolerance; masked
//     chains keep their converged pair and are skipped by every vector kernel. The host reads
//     one counter (active chains) per expansion;
//   * the gauge move is one Householder QR per chain held in shared memory (one CTA per chain)
//     followed by a batched GEMM that pushes R into the neighbour;
//   * the environment update is the batched form of tnx_env_update.
#include <cuda_runtime.h>

#include <cmath>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

constexpr int BT = 256;
constexpr int BWMAX = 64;   // max dl*d and dr*d of the batched MPO contraction
constexpr int BMB = 64;     // largest basis of the batched Davidson

inline unsigned bgrid(int64_t total, int threads, int64_t cap) {
  int64_t b = (total + threads - 1) / threads;
  if (b > cap) b = cap;
  return unsigned(b < 1 ? 1 : b);
}

// ---- batched MPO contraction (blockIdx.y = chain) ---------------------------------------
__global__ void bw_left_kernel(const double* __restrict__ T1, int64_t sT1, const double* __restrict__ W, int64_t sW,
                               double* __restrict__ T2, int64_t sT2, int64_t chi_l, int d, int64_t chi_r, int dl,
                               int dr, const int* __restrict__ mask = nullptr) {
  extern __shared__ double ws[];
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  T1 += b * sT1;
  W += b * sW;
  T2 += b * sT2;
  const int wn = dl * dr * d * d;
  for (int i = threadIdx.x; i < wn; i += blockDim.x) ws[i] = W[i];
  __syncthreads();
  const int64_t total = chi_l * chi_r;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t ap = idx / chi_r, c = idx % chi_r;
    double in[BWMAX];
    for (int w = 0; w < dl; ++w)
      for (int s = 0; s < d; ++s) in[w * d + s] = T1[((w * chi_l + ap) * d + s) * chi_r + c];
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

__global__ void bw_right_kernel(const double* __restrict__ T1, int64_t sT1, const double* __restrict__ W, int64_t sW,
                                double* __restrict__ T2, int64_t sT2, int64_t chi_l, int d, int64_t chi_r, int dl,
                                int dr) {
  extern __shared__ double ws[];
  const int b = blockIdx.y;
  T1 += b * sT1;
  W += b * sW;
  T2 += b * sT2;
  const int wn = dl * dr * d * d;
  for (int i = threadIdx.x; i < wn; i += blockDim.x) ws[i] = W[i];
  __syncthreads();
  const int64_t total = chi_l * chi_r;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t a = idx / chi_r, cp = idx % chi_r;
    double in[BWMAX];
    for (int s = 0; s < d; ++s)
      for (int v = 0; v < dr; ++v) in[v * d + s] = T1[((a * d + s) * dr + v) * chi_r + cp];
    for (int w = 0; w < dl; ++w)
      for (int sp = 0; sp < d; ++sp) {
        double acc = 0.0;
        for (int v = 0; v < dr; ++v)
          for (int s = 0; s < d; ++s) acc = fma(in[v * d + s], ws[((w * dr + v) * d + s) * d + sp], acc);
        T2[((a * dl + w) * d + sp) * chi_r + cp] = acc;
      }
  }
}

__global__ void bdiag_kernel(const double* __restrict__ L, int64_t sL, const double* __restrict__ W, int64_t sW,
                             const double* __restrict__ R, int64_t sR, double* __restrict__ diag, int64_t sD,
                             int64_t chi_l, int d, int64_t chi_r, int dl, int dr) {
  const int b = blockIdx.y;
  L += b * sL;
  W += b * sW;
  R += b * sR;
  diag += b * sD;
  const int64_t total = chi_l * d * chi_r;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t a = idx / (d * chi_r);
    const int s = int((idx / chi_r) % d);
    const int64_t c = idx % chi_r;
    double acc = 0.0;
    for (int w = 0; w < dl; ++w) {
      const double lw = L[(a * dl + w) * chi_l + a];
      for (int v = 0; v < dr; ++v) acc = fma(lw * W[((w * dr + v) * d + s) * d + s], R[(c * dr + v) * chi_r + c], acc);
    }
    diag[idx] = acc;
  }
}

__global__ void bfull_kernel(const double* __restrict__ L, int64_t sL, const double* __restrict__ W, int64_t sW,
                             const double* __restrict__ R, int64_t sR, double* __restrict__ H, int64_t chi_l, int d,
                             int64_t chi_r, int dl, int dr) {
  const int b = blockIdx.y;
  L += b * sL;
  W += b * sW;
  R += b * sR;
  const int64_t n = chi_l * d * chi_r;
  H += int64_t(b) * n * n;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < n * n;
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
      for (int v = 0; v < dr; ++v) acc = fma(lw * W[((w * dr + v) * d + s) * d + sp], R[(c * dr + v) * chi_r + cp], acc);
    }
    H[idx] = acc;
  }
}

// ---- Davidson vector kernels -------------------------------------------------------------
__device__ __forceinline__ double bsum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < int(blockDim.x >> 5); ++i) t += sh[i];
  return t;  // every thread
}

// out[b*so + j*ostr] (and out2[b*so + j*o2str]) = V_b[j] . w_b, grid (k, B)
__global__ void __launch_bounds__(BT) bdots_kernel(const double* __restrict__ V, int64_t sV, int64_t n,
                                                  const double* __restrict__ w, int64_t sw, double* __restrict__ out,
                                                  int64_t so, int ostr, double* __restrict__ out2, int o2str,
                                                  const int* __restrict__ active) {
  __shared__ double sh[BT / 32];
  const int j = blockIdx.x, b = blockIdx.y;
  if (active && !active[b]) return;
  const double* v = V + b * sV + int64_t(j) * n;
  const double* x = w + b * sw;
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += BT) acc = fma(v[i], x[i], acc);
  acc = bsum(acc, sh);
  if (threadIdx.x == 0) {
    out[b * so + int64_t(j) * ostr] = acc;
    if (out2) out2[b * so + int64_t(j) * o2str] = acc;
  }
}

// w_b -= sum_{j<k} h_b[j] V_b[j]; nrm2[b] = |w_b|^2 (k = 0: the norm only), grid (B)
__global__ void __launch_bounds__(BT) bupdate_kernel(const double* __restrict__ V, int64_t sV, int64_t n, int k,
                                                    const double* __restrict__ h, int64_t sh_, double* __restrict__ w,
                                                    int64_t sw, double* __restrict__ nrm2, const int* __restrict__ active) {
  __shared__ double sh[BT / 32];
  __shared__ double hs[BMB];
  const int b = blockIdx.x;
  if (active && !active[b]) return;
  if (threadIdx.x < k) hs[threadIdx.x] = h[b * sh_ + threadIdx.x];
  __syncthreads();
  const double* vb = V + b * sV;
  double* x = w + b * sw;
  double acc2 = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += BT) {
    double a = x[i];
    for (int j = 0; j < k; ++j) a = fma(-hs[j], vb[int64_t(j) * n + i], a);
    x[i] = a;
    acc2 = fma(a, a, acc2);
  }
  acc2 = bsum(acc2, sh);
  if (threadIdx.x == 0) nrm2[b] = acc2;
}

// w_b *= 1/sqrt(nrm2[b]); a direction that vanished against the basis (|w|^2 <= 1e-26 |t|^2
// before orthogonalisation) retires the chain (its Ritz pair is as good as the basis allows)
__global__ void __launch_bounds__(BT) bscale_kernel(double* __restrict__ w, int64_t sw, int64_t n,
                                                   const double* __restrict__ nrm2, const double* __restrict__ nrm2_0,
                                                   int* __restrict__ active) {
  const int b = blockIdx.y;
  if (!active[b]) return;
  const double q = nrm2[b];
  if (!(q > 1e-26 * nrm2_0[b]) || !(q > 0.0)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) active[b] = 0;
    return;
  }
  const double s = 1.0 / sqrt(q);
  double* x = w + b * sw;
  for (int64_t i = int64_t(blockIdx.x) * BT + threadIdx.x; i < n; i += int64_t(gridDim.x) * BT) x[i] *= s;
}

__global__ void bcopy_kernel(const double* __restrict__ src, int64_t ss, double* __restrict__ dst, int64_t sd,
                             int64_t n, const int* __restrict__ active) {
  const int b = blockIdx.y;
  if (active && !active[b]) return;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    dst[b * sd + i] = src[b * ss + i];
}

// x = V s, ax = AV s, r = ax - theta x, t = r / (diag - theta), rn2 = |r|^2; grid (B)
__global__ void __launch_bounds__(BT) britz_kernel(const double* __restrict__ V, const double* __restrict__ AV,
                                                  int64_t sV, int64_t n, int k, const double* __restrict__ evecs,
                                                  int64_t sE, const double* __restrict__ theta,
                                                  const double* __restrict__ diag, int64_t sD, double* __restrict__ x,
                                                  double* __restrict__ ax, double* __restrict__ t, int64_t sX,
                                                  double* __restrict__ rn2, const int* __restrict__ active) {
  __shared__ double sh[BT / 32];
  __shared__ double ss[BMB];
  const int b = blockIdx.x;
  if (!active[b]) return;
  if (threadIdx.x < k) ss[threadIdx.x] = evecs[b * sE + threadIdx.x];
  __syncthreads();
  const double th = theta[b];
  const double* vb = V + b * sV;
  const double* ab = AV + b * sV;
  const double* db = diag + b * sD;
  double* xb = x + b * sX;
  double* axb = ax + b * sX;
  double* tb = t + b * sX;
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += BT) {
    double xv = 0.0, av = 0.0;
    for (int j = 0; j < k; ++j) {
      xv = fma(ss[j], vb[int64_t(j) * n + i], xv);
      av = fma(ss[j], ab[int64_t(j) * n + i], av);
    }
    const double r = av - th * xv;
    xb[i] = xv;
    axb[i] = av;
    double den = db[i] - th;
    if (fabs(den) < 1e-2) den = den >= 0.0 ? 1e-2 : -1e-2;
    tb[i] = r / den;
    acc = fma(r, r, acc);
  }
  acc = bsum(acc, sh);
  if (threadIdx.x == 0) rn2[b] = acc;
}

// retire chains whose residual meets tol * max(1, |theta|); count the rest (one block)
__global__ void bcheck_kernel(const double* __restrict__ theta, const double* __restrict__ rn2, double tol, int B,
                              int* __restrict__ active, int* __restrict__ count) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    if (!active[b]) continue;
    const double r = sqrt(fmax(rn2[b], 0.0));
    if (r <= tol * fmax(1.0, fabs(theta[b]))) {
      active[b] = 0;
    } else {
      atomicAdd(&cnt, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) count[0] = cnt;
}

// GD+1 restart of every active chain (one CTA per chain), to the Ritz vector x = V s and the
// previous step's Ritz vector orthogonalised against it, s' = [s_prev; 0] - (s . s_prev) s (V is
// orthonormal, so on the coefficients). When s_prev lies along s, the basis vector least aligned
// with x takes its place, s' = e_j - s_j s, so every chain restarts to two vectors. Writes
// xp = V s', axp = AV s' and the off-diagonal / second diagonal entry of the 2 x 2 projected
// matrix [s s']^T H_k [s s'] into Hm (the caller sets Hm[0][0] = theta).
__global__ void __launch_bounds__(BT) brestart_plus_kernel(const double* __restrict__ V, const double* __restrict__ AV,
                                                          int64_t sV, int64_t n, int k, double* __restrict__ Hm,
                                                          int64_t sH, int mb, const double* __restrict__ evecs,
                                                          const double* __restrict__ evecs_prev, int64_t sE,
                                                          double* __restrict__ xp, double* __restrict__ axp,
                                                          int64_t sX, const int* __restrict__ active) {
  __shared__ double s[BMB], sp[BMB];
  __shared__ double h01, h11;
  const int b = blockIdx.x;
  if (!active[b]) return;
  if (threadIdx.x == 0) {
    const double* sc = evecs + b * sE;
    const double* so = evecs_prev + b * sE;
    double dot = 0.0;
    for (int j = 0; j < k; ++j) s[j] = sc[j];
    for (int j = 0; j < k - 1; ++j) dot += s[j] * so[j];
    double nrm = 0.0;
    for (int j = 0; j < k; ++j) {
      sp[j] = (j < k - 1 ? so[j] : 0.0) - dot * s[j];
      nrm += sp[j] * sp[j];
    }
    if (!(nrm > 1e-12)) {
      int jm = 0;
      for (int j = 1; j < k; ++j)
        if (fabs(s[j]) < fabs(s[jm])) jm = j;
      nrm = 0.0;
      for (int j = 0; j < k; ++j) {
        sp[j] = (j == jm ? 1.0 : 0.0) - s[jm] * s[j];
        nrm += sp[j] * sp[j];
      }
    }
    nrm = sqrt(nrm);
    for (int j = 0; j < k; ++j) sp[j] /= nrm;
    const double* H = Hm + b * sH;
    double a01 = 0.0, a11 = 0.0;
    for (int i = 0; i < k; ++i) {
      double hsp = 0.0;
      for (int j = 0; j < k; ++j) hsp += H[int64_t(i) * mb + j] * sp[j];
      a01 += s[i] * hsp;
      a11 += sp[i] * hsp;
    }
    h01 = a01;
    h11 = a11;
  }
  __syncthreads();
  const double* vb = V + b * sV;
  const double* ab = AV + b * sV;
  double* xb = xp + b * sX;
  double* axb = axp + b * sX;
  for (int64_t i = threadIdx.x; i < n; i += BT) {
    double xv = 0.0, av = 0.0;
    for (int j = 0; j < k; ++j) {
      xv = fma(sp[j], vb[int64_t(j) * n + i], xv);
      av = fma(sp[j], ab[int64_t(j) * n + i], av);
    }
    xb[i] = xv;
    axb[i] = av;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double* H = Hm + b * sH;
    H[1] = h01;
    H[mb] = h01;
    H[mb + 1] = h11;
  }
}

// Hm_b[0][0] = theta_b for active chains
__global__ void bset_theta_kernel(double* __restrict__ Hm, int64_t sH, const double* __restrict__ theta, int B,
                                  const int* __restrict__ active) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x)
    if (active[b]) Hm[b * sH] = theta[b];
}

__global__ void bsqrt_kernel(const double* __restrict__ in, double* __restrict__ out, int B) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) out[b] = sqrt(fmax(in[b], 0.0));
}

__global__ void bfill_kernel(int* __restrict__ a, int B, int v) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) a[b] = v;
}

// ---- batched Householder QR in shared memory (one CTA per chain) ---------------------------
// M (m x n, m >= n) = Q R. trans = 0: M is the row-major m x n matrix at A_b; trans = 1: M is
// the transpose of the row-major n x m matrix at A_b. Q (m x n) overwrites A_b in the same
// layout (trans = 1 writes Q^T); R (n x n, upper triangular, row-major) goes to R_b.
// Shared memory: the panel a and the Q accumulator q, column-major, 2 m n doubles.
constexpr int QT = 256;

__global__ void __launch_bounds__(QT) bqr_kernel(double* __restrict__ A, int64_t sA, int m, int n, int trans,
                                                double* __restrict__ Rout, int64_t sR) {
  extern __shared__ double smq[];
  double* a = smq;          // m x n column-major: a[j*m + i]
  double* q = smq + m * n;  // m x n column-major
  __shared__ double tau[128];
  const int b = blockIdx.x;
  double* Ab = A + b * sA;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = QT / 32;
  for (int e = tid; e < m * n; e += QT) {
    const int j = e / m, i = e % m;
    a[e] = trans ? Ab[int64_t(j) * m + i] : Ab[int64_t(i) * n + j];
    q[e] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    double* cj = a + j * m;
    if (warp == 0) {
      double sg = 0.0;
      for (int i = j + 1 + lane; i < m; i += 32) sg = fma(cj[i], cj[i], sg);
      const double alpha = cj[j];  // every lane reads it before the shuffles below
      for (int o = 16; o > 0; o >>= 1) sg += __shfl_xor_sync(0xffffffffu, sg, o);
      double t = 0.0, scale = 0.0, beta = alpha;
      if (sg > 0.0) {
        const double nrm = sqrt(fma(alpha, alpha, sg));
        beta = alpha >= 0.0 ? -nrm : nrm;
        t = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      for (int i = j + 1 + lane; i < m; i += 32) cj[i] *= scale;
      __syncwarp();
      if (lane == 0) {
        cj[j] = beta;
        tau[j] = t;
      }
    }
    __syncthreads();
    const double tj = tau[j];
    if (tj != 0.0) {
      for (int c = j + 1 + warp; c < n; c += nw) {
        double* cc = a + c * m;
        const double top = cc[j];  // read by every lane before lane 0 rewrites it
        double w = 0.0;
        for (int i = j + 1 + lane; i < m; i += 32) w = fma(cj[i], cc[i], w);
        for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
        w = tj * (w + top);
        if (lane == 0) cc[j] -= w;
        for (int i = j + 1 + lane; i < m; i += 32) cc[i] = fma(-w, cj[i], cc[i]);
      }
    }
    __syncthreads();
  }
  // Q = H_0 H_1 ... H_{n-1} I[:, :n], applied from the last reflector
  for (int j = n - 1; j >= 0; --j) {
    const double tj = tau[j];
    const double* cj = a + j * m;
    if (tj != 0.0) {
      for (int c = j + warp; c < n; c += nw) {
        double* qc = q + c * m;
        const double top = qc[j];
        double w = 0.0;
        for (int i = j + 1 + lane; i < m; i += 32) w = fma(cj[i], qc[i], w);
        for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
        w = tj * (w + top);
        if (lane == 0) qc[j] -= w;
        for (int i = j + 1 + lane; i < m; i += 32) qc[i] = fma(-w, cj[i], qc[i]);
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < m * n; e += QT) {
    const int j = e / m, i = e % m;
    if (trans) Ab[int64_t(j) * m + i] = q[e];
    else Ab[int64_t(i) * n + j] = q[e];
  }
  double* Rb = Rout + b * sR;
  for (int e = tid; e < n * n; e += QT) {
    const int i = e / n, c = e % n;
    Rb[e] = i <= c ? a[c * m + i] : 0.0;
  }
}

// ---- batched matvec --------------------------------------------------------------------
struct BDims {
  int64_t chi_l, d, chi_r, dl, dr;
  int64_t n() const { return chi_l * d * chi_r; }
  int64_t ne() const { return matvec1_scratch_elems(chi_l, d, chi_r, dl, dr); }
};

// mask (device, B ints, may be null): chains whose entry is 0 are skipped by every launch
// Batched FP64-class products: one tensor-core launch (Ozaki, every chain at its stride, masked
// chains skipped) where scratch `oz` is given and the batch's product is large enough; the
// strided-batched double-FP32 / FP64 GEMM otherwise.
inline bool boz_applies(int64_t m, int64_t n, int64_t k, int B) {
  return k >= 32 && m >= 32 && n >= 32 && double(m) * double(n) * double(k) * B >= double(1 << 26);
}
size_t boz_bytes(int64_t m, int64_t n, int64_t k, int B) {
  return boz_applies(m, n, k, B) ? gemm_oz_ex_workspace_bytes(m, n, k, B, 1) : 0;
}
int bgemm(bool df, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
          int64_t sA, const double* B, int64_t ldb, int64_t sB, double beta, double* C, int64_t ldc, int64_t sC,
          int batch, cudaStream_t st, const int* mask, void* oz, size_t ozb) {
  if (df && oz && boz_applies(m, n, k, batch) && ozb >= gemm_oz_ex_workspace_bytes(m, n, k, batch, 1))
    return gemm_oz_ex(ta, tb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, 1, mask, oz, ozb, st);
  return gemm_fp64_class(df, ta, tb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, st, 0, mask);
}
// Ozaki scratch for the two products of a batched matvec / environment update of these shapes
size_t bmatvec_oz_bytes(const BDims& g, int B) {
  size_t b = boz_bytes(g.dl * g.chi_l, g.d * g.chi_r, g.chi_l, B);
  auto mx = [&](size_t x) { b = x > b ? x : b; };
  mx(boz_bytes(g.chi_l * g.d, g.chi_r, g.chi_r * g.dr, B));  // matvec, second product
  mx(boz_bytes(g.chi_r * g.dr, g.chi_r, g.chi_l * g.d, B));  // rightward environment update
  mx(boz_bytes(g.chi_l * g.d, g.dr * g.chi_r, g.chi_r, B));  // leftward environment update
  mx(boz_bytes(g.chi_l * g.dl, g.chi_l, g.d * g.chi_r, B));
  return b;
}

int bmatvec(const double* L, int64_t sL, const double* W, int64_t sW, const double* R, int64_t sR, const double* x,
            int64_t sx, double* y, int64_t sy, int B, const BDims& g, double* T1, double* T2, bool df,
            cudaStream_t st, const int* mask = nullptr, void* oz = nullptr, size_t ozb = 0) {
  const int64_t ne = g.ne();
  // T1[(w,a'),(s,c)] = sum_a L[a,(w,a')] x[a,(s,c)]
  TNX_TRY(bgemm(df, true, false, g.dl * g.chi_l, g.d * g.chi_r, g.chi_l, 1.0, L, g.dl * g.chi_l, sL, x,
                g.d * g.chi_r, sx, 0.0, T1, g.d * g.chi_r, ne, B, st, mask, oz, ozb));
  const size_t smem = size_t(g.dl * g.dr * g.d * g.d) * sizeof(double);
  bw_left_kernel<<<dim3(bgrid(g.chi_l * g.chi_r, 128, 64), B), 128, smem, st>>>(
      T1, ne, W, sW, T2, ne, g.chi_l, int(g.d), g.chi_r, int(g.dl), int(g.dr), mask);
  TNX_LAUNCH_CHECK();
  // y[(a',s'),c'] = sum_{(c,v)} T2[(a',s'),(c,v)] R[(c,v),c']
  TNX_TRY(bgemm(df, false, false, g.chi_l * g.d, g.chi_r, g.chi_r * g.dr, 1.0, T2, g.chi_r * g.dr, ne, R, g.chi_r,
                sR, 0.0, y, g.chi_r, sy, B, st, mask, oz, ozb));
  return TNX_OK;
}

int check_bdims(const void* a, const void* b, const void* c, const void* x, int B, const BDims& g) {
  TNX_CHECK_ARG(a && b && c && x, "null pointer");
  TNX_CHECK_ARG(B > 0 && B <= 65535, "batch must be in [1, 65535] (got %d)", B);
  TNX_CHECK_ARG(g.chi_l > 0 && g.d > 0 && g.chi_r > 0 && g.dl > 0 && g.dr > 0, "non-positive dimension");
  TNX_CHECK_SHAPE(g.dl * g.d <= BWMAX && g.dr * g.d <= BWMAX, "MPO bond too large (dl*d, dr*d <= %d)", BWMAX);
  TNX_CHECK_SHAPE(g.chi_l <= (1 << 20) && g.chi_r <= (1 << 20) && g.d <= 64, "dimension too large");
  return TNX_OK;
}

struct BDavWs {
  double *V, *AV, *x, *ax, *t, *diag, *Hm, *evals, *evecs, *evecs_prev, *h, *nrm2, *nrm2_0, *rn2, *T1, *T2, *xp,
      *axp;
  int *active, *count;
  void* oz;
  size_t oz_bytes;
};

size_t bdav_layout(const BDims& g, int B, int mb, void* base, BDavWs* w) {
  const int64_t n = g.n(), ne = g.ne();
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align_up(bytes);
    return o;
  };
  const size_t Bz = size_t(B);
  size_t oV = take(Bz * mb * n * 8), oAV = take(Bz * mb * n * 8), ox = take(Bz * n * 8), oax = take(Bz * n * 8),
         ot = take(Bz * n * 8), od = take(Bz * n * 8), oH = take(Bz * mb * mb * 8), oev = take(Bz * 8),
         oevec = take(Bz * mb * 8), oh = take(Bz * mb * 8), on = take(Bz * 8), on0 = take(Bz * 8), orn = take(Bz * 8),
         oT1 = take(Bz * ne * 8), oT2 = take(Bz * ne * 8), oa = take(Bz * 4), oc = take(16),
         oep = take(Bz * mb * 8), oxp = take(Bz * n * 8), oaxp = take(Bz * n * 8);
  const size_t ozb = bmatvec_oz_bytes(g, B), ooz = take(ozb);
  if (w && base) {
    char* p = static_cast<char*>(base);
    w->V = reinterpret_cast<double*>(p + oV);
    w->AV = reinterpret_cast<double*>(p + oAV);
    w->x = reinterpret_cast<double*>(p + ox);
    w->ax = reinterpret_cast<double*>(p + oax);
    w->t = reinterpret_cast<double*>(p + ot);
    w->diag = reinterpret_cast<double*>(p + od);
    w->Hm = reinterpret_cast<double*>(p + oH);
    w->evals = reinterpret_cast<double*>(p + oev);
    w->evecs = reinterpret_cast<double*>(p + oevec);
    w->h = reinterpret_cast<double*>(p + oh);
    w->nrm2 = reinterpret_cast<double*>(p + on);
    w->nrm2_0 = reinterpret_cast<double*>(p + on0);
    w->rn2 = reinterpret_cast<double*>(p + orn);
    w->T1 = reinterpret_cast<double*>(p + oT1);
    w->T2 = reinterpret_cast<double*>(p + oT2);
    w->active = reinterpret_cast<int*>(p + oa);
    w->count = reinterpret_cast<int*>(p + oc);
    w->evecs_prev = reinterpret_cast<double*>(p + oep);
    w->xp = reinterpret_cast<double*>(p + oxp);
    w->axp = reinterpret_cast<double*>(p + oaxp);
    w->oz = ozb ? p + ooz : nullptr;
    w->oz_bytes = ozb;
  }
  return off;
}

}  // namespace
}  // namespace tnx

using namespace tnx;

extern "C" {

size_t tnx_batched_matvec1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                           int batch) {
  const BDims g{chi_l, d, chi_r, dl, dr};
  return 2 * align_up(size_t(batch) * size_t(g.ne()) * 8) + align_up(bmatvec_oz_bytes(g, batch));
}

int tnx_batched_matvec1(const double* L, int64_t sL, const double* W, int64_t sW, const double* R, int64_t sR,
                        const double* x, int64_t sx, double* y, int64_t sy, int batch, int64_t chi_l, int64_t d,
                        int64_t chi_r, int64_t dl, int64_t dr, int precision, void* workspace,
                        size_t workspace_bytes, void* stream) {
  const BDims g{chi_l, d, chi_r, dl, dr};
  TNX_TRY(check_bdims(L, W, R, x, batch, g));
  TNX_CHECK_ARG(y, "null y pointer");
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  const size_t need = tnx_batched_matvec1_workspace_bytes(chi_l, d, chi_r, dl, dr, batch);
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_batched_matvec1: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  double* T1 = static_cast<double*>(workspace);
  double* T2 = reinterpret_cast<double*>(static_cast<char*>(workspace) + align_up(size_t(batch) * g.ne() * 8));
  const size_t ozb = bmatvec_oz_bytes(g, batch);
  void* oz = ozb ? static_cast<char*>(workspace) + 2 * align_up(size_t(batch) * g.ne() * 8) : nullptr;
  return bmatvec(L, sL, W, sW, R, sR, x, sx, y, sy, batch, g, T1, T2, use_df64(precision), as_stream(stream), nullptr,
                 oz, ozb);
}

int tnx_batched_full_matrix1(const double* L, int64_t sL, const double* W, int64_t sW, const double* R, int64_t sR,
                             double* H, int batch, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                             void* stream) {
  const BDims g{chi_l, d, chi_r, dl, dr};
  TNX_TRY(check_bdims(L, W, R, H, batch, g));
  TNX_CHECK_SHAPE(g.n() <= 4096, "dense H_eff only for n <= 4096 (got %lld)", (long long)g.n());
  bfull_kernel<<<dim3(bgrid(g.n() * g.n(), 256, 64), batch), 256, 0, as_stream(stream)>>>(
      L, sL, W, sW, R, sR, H, chi_l, int(d), chi_r, int(dl), int(dr));
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

size_t tnx_batched_env_update_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                              int batch) {
  return tnx_batched_matvec1_workspace_bytes(chi_l, d, chi_r, dl, dr, batch);
}

int tnx_batched_env_update(int direction, const double* E_in, int64_t sE, const double* A, int64_t sA,
                           const double* W, int64_t sW, double* E_out, int64_t sO, int batch, int64_t chi_l, int64_t d,
                           int64_t chi_r, int64_t dl, int64_t dr, int precision, void* workspace,
                           size_t workspace_bytes, void* stream) {
  const BDims g{chi_l, d, chi_r, dl, dr};
  TNX_TRY(check_bdims(E_in, A, W, E_out, batch, g));
  TNX_CHECK_ARG(direction == 1 || direction == -1, "direction must be +1 or -1 (got %d)", direction);
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  const size_t need = tnx_batched_env_update_workspace_bytes(chi_l, d, chi_r, dl, dr, batch);
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_batched_env_update: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  const bool df = use_df64(precision);
  const int64_t ne = g.ne();
  double* T1 = static_cast<double*>(workspace);
  double* T2 = reinterpret_cast<double*>(static_cast<char*>(workspace) + align_up(size_t(batch) * ne * 8));
  const size_t ozb = bmatvec_oz_bytes(g, batch);
  void* oz = ozb ? static_cast<char*>(workspace) + 2 * align_up(size_t(batch) * ne * 8) : nullptr;
  const size_t smem = size_t(dl * dr * d * d) * sizeof(double);
  if (direction == 1) {
    TNX_TRY(bgemm(df, true, false, dl * chi_l, d * chi_r, chi_l, 1.0, E_in, dl * chi_l, sE, A, d * chi_r, sA, 0.0, T1,
                  d * chi_r, ne, batch, st, nullptr, oz, ozb));
    bw_left_kernel<<<dim3(bgrid(chi_l * chi_r, 128, 64), batch), 128, smem, st>>>(T1, ne, W, sW, T2, ne, chi_l,
                                                                                  int(d), chi_r, int(dl), int(dr));
    TNX_LAUNCH_CHECK();
    TNX_TRY(bgemm(df, true, false, chi_r * dr, chi_r, chi_l * d, 1.0, T2, chi_r * dr, ne, A, chi_r, sA, 0.0, E_out,
                  chi_r, sO, batch, st, nullptr, oz, ozb));
  } else {
    TNX_TRY(bgemm(df, false, false, chi_l * d, dr * chi_r, chi_r, 1.0, A, chi_r, sA, E_in, dr * chi_r, sE, 0.0, T1,
                  dr * chi_r, ne, batch, st, nullptr, oz, ozb));
    bw_right_kernel<<<dim3(bgrid(chi_l * chi_r, 128, 64), batch), 128, smem, st>>>(T1, ne, W, sW, T2, ne, chi_l,
                                                                                   int(d), chi_r, int(dl), int(dr));
    TNX_LAUNCH_CHECK();
    TNX_TRY(bgemm(df, false, true, chi_l * dl, chi_l, d * chi_r, 1.0, T2, d * chi_r, ne, A, d * chi_r, sA, 0.0, E_out,
                  chi_l, sO, batch, st, nullptr, oz, ozb));
  }
  return TNX_OK;
}

size_t tnx_batched_davidson1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                             int batch, int max_basis) {
  if (max_basis > BMB) max_basis = BMB;
  return bdav_layout(BDims{chi_l, d, chi_r, dl, dr}, batch, max_basis, nullptr, nullptr);
}

int tnx_batched_davidson1(const double* L, int64_t sL, const double* W, int64_t sW, const double* R, int64_t sR,
                          double* X, int64_t sX, int batch, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                          int64_t dr, double tol, int max_iter, int max_basis, int precision, double* evals_out,
                          double* resid_out, int* iters_out, int* active_out, void* workspace,
                          size_t workspace_bytes, void* stream) {
  const BDims g{chi_l, d, chi_r, dl, dr};
  TNX_TRY(check_bdims(L, W, R, X, batch, g));
  TNX_CHECK_ARG(max_basis >= 2 && max_basis <= BMB, "max_basis must be in [2, %d] (got %d)", BMB, max_basis);
  TNX_CHECK_ARG(max_iter >= 1 && tol >= 0.0, "max_iter must be >= 1 and tol >= 0");
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  TNX_CHECK_ARG(evals_out && resid_out, "null output pointer");
  const int64_t n = g.n();
  int mb = max_basis;
  if (mb > n) mb = int(n < 2 ? 2 : n);
  const size_t need = bdav_layout(g, batch, mb, nullptr, nullptr);
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_batched_davidson1: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  BDavWs w;
  bdav_layout(g, batch, mb, workspace, &w);
  cudaStream_t st = as_stream(stream);
  const bool df = use_df64(precision);
  const int64_t sVB = int64_t(mb) * n;  // chain stride of V / AV
  const int B = batch;
  const unsigned vchunks = bgrid(n, BT, 8);
  bdiag_kernel<<<dim3(bgrid(n, 256, 16), B), 256, 0, st>>>(L, sL, W, sW, R, sR, w.diag, n, chi_l, int(d), chi_r,
                                                           int(dl), int(dr));
  TNX_LAUNCH_CHECK();
  bfill_kernel<<<(B + 255) / 256, 256, 0, st>>>(w.active, B, 1);
  TNX_LAUNCH_CHECK();
  bcopy_kernel<<<dim3(vchunks, B), BT, 0, st>>>(X, sX, w.t, n, n, nullptr);
  TNX_LAUNCH_CHECK();
  int k = 0, iters = 0, host_count = B;
  // Stragglers: once at most B / 64 chains are still active (it_most: the expansion at which
  // that was first seen), the remaining chains get max(it_most, 32) more expansions and then
  // stop with their current Ritz pair (reported as not converged). Every expansion of a
  // lockstep batch costs the launches of the whole batch, so one slow chain at 400 expansions
  // would otherwise cost as much as the rest of the site.
  const int straggler_max = B / 64;
  int it_most = -1;
  for (;;) {
    double* vk = w.V + int64_t(k) * n;
    bcopy_kernel<<<dim3(vchunks, B), BT, 0, st>>>(w.t, n, vk, sVB, n, w.active);
    TNX_LAUNCH_CHECK();
    bupdate_kernel<<<B, BT, 0, st>>>(w.V, sVB, n, 0, w.h, mb, vk, sVB, w.nrm2_0, w.active);
    TNX_LAUNCH_CHECK();
    if (k == 0) {
      TNX_CUDA(cudaMemcpyAsync(w.nrm2, w.nrm2_0, size_t(B) * 8, cudaMemcpyDeviceToDevice, st));
    } else {
      for (int pass = 0; pass < 2; ++pass) {  // classical Gram-Schmidt, twice
        bdots_kernel<<<dim3(k, B), BT, 0, st>>>(w.V, sVB, n, vk, sVB, w.h, mb, 1, nullptr, 0, w.active);
        TNX_LAUNCH_CHECK();
        bupdate_kernel<<<B, BT, 0, st>>>(w.V, sVB, n, k, w.h, mb, vk, sVB, w.nrm2, w.active);
        TNX_LAUNCH_CHECK();
      }
    }
    bscale_kernel<<<dim3(vchunks, B), BT, 0, st>>>(vk, sVB, n, w.nrm2, w.nrm2_0, w.active);
    TNX_LAUNCH_CHECK();
    double* avk = w.AV + int64_t(k) * n;
    // converged chains are masked out of the products too
    TNX_TRY(bmatvec(L, sL, W, sW, R, sR, vk, sVB, avk, sVB, B, g, w.T1, w.T2, df, st, w.active, w.oz, w.oz_bytes));
    // column k of the projected matrix (and its mirror row)
    bdots_kernel<<<dim3(k + 1, B), BT, 0, st>>>(w.V, sVB, n, avk, sVB, w.Hm + k, int64_t(mb) * mb, mb,
                                                w.Hm + int64_t(k) * mb, 1, w.active);
    TNX_LAUNCH_CHECK();
    ++k;
    ++iters;
    // the previous step's Ritz coefficients, for the GD+1 restart
    TNX_CUDA(cudaMemcpyAsync(w.evecs_prev, w.evecs, size_t(B) * mb * 8, cudaMemcpyDeviceToDevice, st));
    TNX_TRY(rr_lowest_f64_batched(w.Hm, k, mb, int64_t(mb) * mb, w.evals, 1, w.evecs, mb, B, w.active, st));
    britz_kernel<<<B, BT, 0, st>>>(w.V, w.AV, sVB, n, k, w.evecs, mb, w.evals, w.diag, n, w.x, w.ax, w.t, n, w.rn2,
                                   w.active);
    TNX_LAUNCH_CHECK();
    bcheck_kernel<<<1, 256, 0, st>>>(w.evals, w.rn2, tol, B, w.active, w.count);
    TNX_LAUNCH_CHECK();
    // the active count is read every 4th expansion (the kernels already skip retired chains, so
    // the expansions in between cost only launches once every chain has converged)
    if (iters % 4 == 0 || iters >= max_iter || k >= n) {
      TNX_CUDA(cudaMemcpyAsync(&host_count, w.count, sizeof(int), cudaMemcpyDeviceToHost, st));
      TNX_CUDA(cudaStreamSynchronize(st));
      if (host_count == 0 || iters >= max_iter || k >= n) break;
      if (it_most < 0 && host_count <= straggler_max) it_most = iters;
      if (it_most >= 0 && iters >= it_most + (it_most > 32 ? it_most : 32)) break;
    }
    if (k == mb) {  // GD+1 restart of every active chain: its Ritz vector and the previous one
      brestart_plus_kernel<<<B, BT, 0, st>>>(w.V, w.AV, sVB, n, k, w.Hm, int64_t(mb) * mb, mb, w.evecs,
                                             w.evecs_prev, mb, w.xp, w.axp, n, w.active);
      TNX_LAUNCH_CHECK();
      bcopy_kernel<<<dim3(vchunks, B), BT, 0, st>>>(w.x, n, w.V, sVB, n, w.active);
      TNX_LAUNCH_CHECK();
      bcopy_kernel<<<dim3(vchunks, B), BT, 0, st>>>(w.ax, n, w.AV, sVB, n, w.active);
      TNX_LAUNCH_CHECK();
      bcopy_kernel<<<dim3(vchunks, B), BT, 0, st>>>(w.xp, n, w.V + n, sVB, n, w.active);
      TNX_LAUNCH_CHECK();
      bcopy_kernel<<<dim3(vchunks, B), BT, 0, st>>>(w.axp, n, w.AV + n, sVB, n, w.active);
      TNX_LAUNCH_CHECK();
      bset_theta_kernel<<<(B + 255) / 256, 256, 0, st>>>(w.Hm, int64_t(mb) * mb, w.evals, B, w.active);
      TNX_LAUNCH_CHECK();
      k = 2;
    }
  }
  // results: the last Ritz pair of every chain (frozen when its chain retired)
  bcopy_kernel<<<dim3(vchunks, B), BT, 0, st>>>(w.x, n, X, sX, n, nullptr);
  TNX_LAUNCH_CHECK();
  TNX_CUDA(cudaMemcpyAsync(evals_out, w.evals, size_t(B) * 8, cudaMemcpyDeviceToDevice, st));
  bsqrt_kernel<<<(B + 255) / 256, 256, 0, st>>>(w.rn2, resid_out, B);
  TNX_LAUNCH_CHECK();
  if (active_out) TNX_CUDA(cudaMemcpyAsync(active_out, w.active, size_t(B) * 4, cudaMemcpyDeviceToDevice, st));
  if (iters_out) *iters_out = iters;
  return host_count == 0 ? TNX_OK : TNX_ERR_NOT_CONVERGED;
}

size_t tnx_batched_gauge_move_workspace_bytes(int direction, int64_t chi_l, int64_t d, int64_t chi_r,
                                              int64_t chi_other, int batch) {
  const int64_t nb = direction == 1 ? chi_r : chi_l;
  const int64_t other = direction == 1 ? chi_r * d * chi_other : chi_other * d * chi_l;
  const size_t ozb = direction == 1 ? boz_bytes(chi_r, d * chi_other, chi_r, batch)
                                    : boz_bytes(chi_other * d, chi_l, chi_l, batch);
  return align_up(size_t(batch) * nb * nb * 8) + align_up(size_t(batch) * other * 8) + align_up(ozb);
}

int tnx_batched_gauge_move(int direction, double* A_site, int64_t sA, double* A_nb, int64_t sN, int batch,
                           int64_t chi_l, int64_t d, int64_t chi_r, int64_t chi_other, int precision, void* workspace,
                           size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(A_site && A_nb, "null pointer");
  TNX_CHECK_ARG(batch > 0 && batch <= 65535, "batch must be in [1, 65535]");
  TNX_CHECK_ARG(direction == 1 || direction == -1, "direction must be +1 or -1 (got %d)", direction);
  TNX_CHECK_ARG(chi_l > 0 && d > 0 && chi_r > 0 && chi_other > 0, "non-positive dimension");
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  const int64_t m = direction == 1 ? chi_l * d : d * chi_r, nn = direction == 1 ? chi_r : chi_l;
  TNX_CHECK_SHAPE(m >= nn, "the split bond (%lld) exceeds the fused dimension (%lld)", (long long)nn, (long long)m);
  TNX_CHECK_SHAPE(nn <= 128 && m * nn * 16 <= 200 * 1024,
                  "batched gauge move holds the site matrix in shared memory: m*n <= 12800, n <= 128 (got %lld x %lld)",
                  (long long)m, (long long)nn);
  const size_t need = tnx_batched_gauge_move_workspace_bytes(direction, chi_l, d, chi_r, chi_other, batch);
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_batched_gauge_move: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  double* Rm = static_cast<double*>(workspace);
  double* tmp = reinterpret_cast<double*>(static_cast<char*>(workspace) + align_up(size_t(batch) * nn * nn * 8));
  const size_t smem = size_t(2 * m * nn) * sizeof(double);
  TNX_CUDA(cudaFuncSetAttribute(bqr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  bqr_kernel<<<batch, QT, smem, st>>>(A_site, sA, int(m), int(nn), direction == 1 ? 0 : 1, Rm, nn * nn);
  TNX_LAUNCH_CHECK();
  const bool df = use_df64(precision);
  const int64_t other = direction == 1 ? chi_r * d * chi_other : chi_other * d * chi_l;
  const size_t ozb = direction == 1 ? boz_bytes(chi_r, d * chi_other, chi_r, batch)
                                    : boz_bytes(chi_other * d, chi_l, chi_l, batch);
  void* oz = ozb ? reinterpret_cast<char*>(tmp) + align_up(size_t(batch) * other * 8) : nullptr;
  if (direction == 1) {
    // A_next (chi_r x (d chi_other)) <- R A_next
    TNX_TRY(bgemm(df, false, false, chi_r, d * chi_other, chi_r, 1.0, Rm, chi_r, chi_r * chi_r, A_nb, d * chi_other,
                  sN, 0.0, tmp, d * chi_other, other, batch, st, nullptr, oz, ozb));
  } else {
    // A_prev ((chi_other d) x chi_l) <- A_prev R^T
    TNX_TRY(bgemm(df, false, true, chi_other * d, chi_l, chi_l, 1.0, A_nb, chi_l, sN, Rm, chi_l, chi_l * chi_l, 0.0,
                  tmp, chi_l, other, batch, st, nullptr, oz, ozb));
  }
  bcopy_kernel<<<dim3(bgrid(other, 256, 16), batch), 256, 0, st>>>(tmp, other, A_nb, sN, other, nullptr);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

}  // extern "C"
