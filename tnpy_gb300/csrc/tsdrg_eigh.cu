// Lowest-k eigenpairs of tSDRG block Hamiltonians H = sum_w A_w (x) B_w without forming H.
//
// Reference: TreeTensorNetworkSDRG.block_eigen_solver (tnpy/tsdrg.py:569-592) diagonalises
// the dense two-block Hamiltonian of block_hamiltonian (:607-631) with np.linalg.eigh and keeps
// the lowest chi pairs. Here A_w = W1[0, w] (m1 x m1) and B_w = W2[w, dr2-1] (m2 x m2), so
// H v = sum_w vec(A_w X B_w^T) for X the m1 x m2 reshaping of v: a matvec costs
// 2 D m1 m2 (m1 + m2) flops instead of 2 (m1 m2)^2 and only the small factors sit in shared
// memory. One CTA per block, batched over blocks and disorder realisations:
//
//   1. Chebyshev-filtered subspace iteration in precision T (float or double) on p = k + guard
//      vectors: Rayleigh-Ritz with a one-warp Jacobi of the p x p projected matrix, a degree-q
//      Chebyshev filter damping [theta_p, upper bound], CGS2 orthonormalisation; stop when the
//      k wanted residuals reach T's rounding level.
//      In FP64 precision the FP32 iteration runs first and the FP64 iteration starts from its
//      k vectors, so the slow FP64 pipe only takes the last digits (a few outer iterations).
//      The filter's upper bound comes from 24 Lanczos steps (largest Ritz value + |beta|).
//   2. FP64 Rayleigh-Ritz refinement of the k kept vectors (kron_refine_kernel): CGS2 in FP64,
//      Z = H V in FP64, G = V^T Z, FP64 Jacobi of G, V <- V Q. Ritz values are second order in
//      the subspace error, so an FP32 subspace (~1e-6) gives FP64-accurate kept spectra.
//
// Work vectors live in global memory (L2-resident): 4 p m values of T per CTA.
#include <cuda_runtime.h>

#include <atomic>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

constexpr int KT = 256;       // threads per CTA
constexpr int KM1 = 32;       // largest node dimension (m1, m2)
constexpr int KP = 48;        // largest subspace block (k <= 32 kept + guard)
constexpr int KD = 6;         // largest MPO bond

template <typename T>
struct KSmem {
  T A[KD][KM1 * KM1];
  T B[KD][KM1 * KM1];
  T Xs[KM1 * KM1];
  T Ts[KM1 * KM1];
  T G[KP][KP + 1];
  T Q[KP][KP + 1];
  T theta[KP];
  T red[KT / 32][KP];
  T scal[KP];
  int order[KP];
  int flag;
};

template <typename T>
__device__ __forceinline__ T wsum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// a . b over m entries, returned to every thread
template <typename T>
__device__ T dot1(KSmem<T>& s, const T* a, const T* b, int m) {
  T part = T(0);
  for (int e = threadIdx.x; e < m; e += KT) part += a[e] * b[e];
  part = wsum(part);
  if ((threadIdx.x & 31) == 0) s.red[threadIdx.x >> 5][0] = part;
  __syncthreads();
  T t = T(0);
  for (int q = 0; q < KT / 32; ++q) t += s.red[q][0];
  __syncthreads();
  return t;
}

// largest eigenvalue of the symmetric tridiagonal (alpha[0..n), beta[1..n)) by Sturm bisection
__device__ double tridiag_max(const double* alpha, const double* beta, int n) {
  double lo = alpha[0], hi = alpha[0];
  for (int i = 0; i < n; ++i) {  // Gershgorin interval
    const double r = (i > 0 ? fabs(beta[i]) : 0.0) + (i + 1 < n ? fabs(beta[i + 1]) : 0.0);
    lo = fmin(lo, alpha[i] - r);
    hi = fmax(hi, alpha[i] + r);
  }
  for (int it = 0; it < 60; ++it) {
    const double x = 0.5 * (lo + hi);
    int below = 0;  // eigenvalues < x
    double q = alpha[0] - x;
    below += q < 0.0;
    for (int i = 1; i < n; ++i) {
      if (q == 0.0) q = 1e-300;
      q = alpha[i] - x - beta[i] * beta[i] / q;
      below += q < 0.0;
    }
    if (below == n) hi = x;  // every eigenvalue below x
    else lo = x;
  }
  return hi;
}

// Y[:, j] = H X[:, j] for j < ncols (vector-major storage [j][m]).
template <typename T>
__device__ void kron_apply(KSmem<T>& s, const T* X, T* Y, int ncols, int m1, int m2, int D) {
  const int m = m1 * m2;
  for (int j = 0; j < ncols; ++j) {
    for (int e = threadIdx.x; e < m; e += KT) s.Xs[e] = X[size_t(j) * m + e];
    T acc[4] = {T(0), T(0), T(0), T(0)};  // m <= 1024 = 4 * KT
    __syncthreads();
    for (int w = 0; w < D; ++w) {
      for (int e = threadIdx.x; e < m; e += KT) {  // Ts = A_w Xs
        const int k1 = e / m2, b2 = e % m2;
        T t = T(0);
        for (int b1 = 0; b1 < m1; ++b1) t += s.A[w][k1 * m1 + b1] * s.Xs[b1 * m2 + b2];
        s.Ts[e] = t;
      }
      __syncthreads();
      int q = 0;
      for (int e = threadIdx.x; e < m; e += KT, ++q) {  // acc += Ts B_w^T
        const int k1 = e / m2, k2 = e % m2;
        T t = T(0);
        for (int b2 = 0; b2 < m2; ++b2) t += s.Ts[k1 * m2 + b2] * s.B[w][k2 * m2 + b2];
        acc[q] += t;
      }
      __syncthreads();
    }
    int q = 0;
    for (int e = threadIdx.x; e < m; e += KT, ++q) Y[size_t(j) * m + e] = acc[q];
  }
  __syncthreads();
}

// out[i] = sum_e (U[i][e] - c[i] V[i][e]) * (W[i][e] - d[i] Z[i][e]) style reductions are
// expressed through this one helper: out[i] = U_i . W_i (pairwise) when pairwise, else
// out[i] = U_i . w for a single vector w. n <= KP.
template <typename T>
__device__ void block_dots(KSmem<T>& s, const T* U, const T* w, int n, int m, T* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T part[KP];
#pragma unroll
  for (int i = 0; i < KP; ++i) part[i] = T(0);
  for (int e = threadIdx.x; e < m; e += KT) {
    const T we = w[e];
#pragma unroll
    for (int i = 0; i < KP; ++i)
      if (i < n) part[i] += U[size_t(i) * m + e] * we;
  }
#pragma unroll
  for (int i = 0; i < KP; ++i)
    if (i < n) {
      const T t = wsum(part[i]);
      if (lane == 0) s.red[warp][i] = t;
    }
  __syncthreads();
  if (threadIdx.x < n) {
    T t = T(0);
    for (int q = 0; q < KT / 32; ++q) t += s.red[q][threadIdx.x];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// CGS2 orthonormalisation of the p columns of X (vector-major, length m)
template <typename T>
__device__ void orthonormalise(KSmem<T>& s, T* X, int p, int m) {
  for (int j = 0; j < p; ++j) {
    T* xj = X + size_t(j) * m;
    for (int pass = 0; pass < 2 && j > 0; ++pass) {
      block_dots(s, X, xj, j, m, s.scal);
      for (int e = threadIdx.x; e < m; e += KT) {
        T t = xj[e];
        for (int i = 0; i < j; ++i) t -= s.scal[i] * X[size_t(i) * m + e];
        xj[e] = t;
      }
      __syncthreads();
    }
    block_dots(s, xj, xj, 1, m, s.scal);
    const T nrm = sqrt(s.scal[0]);
    const T inv = nrm > T(0) ? T(1) / nrm : T(0);
    for (int e = threadIdx.x; e < m; e += KT) xj[e] *= inv;
    __syncthreads();
  }
}

// out[:, r] = sum_i in[:, i] Q[i][r] for r < p (vector-major)
template <typename T>
__device__ void rotate(KSmem<T>& s, const T* in, T* out, int p, int m) {
  for (int e = threadIdx.x; e < m; e += KT) {
    T x[KP];
#pragma unroll
    for (int i = 0; i < KP; ++i) x[i] = i < p ? in[size_t(i) * m + e] : T(0);
    for (int r = 0; r < p; ++r) {
      T t = T(0);
#pragma unroll
      for (int i = 0; i < KP; ++i)
        if (i < p) t += x[i] * s.Q[i][r];
      out[size_t(r) * m + e] = t;
    }
  }
  __syncthreads();
}

// Eigendecomposition of the n x n (n <= KP) symmetric s.G by one warp (parallel cyclic Jacobi,
// one pair per lane per round): eigenvalues ascending in s.theta, vectors in the columns of s.Q.
template <typename T>
__device__ void small_eigh(KSmem<T>& s, int n) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    for (int e = lane; e < n * n; e += 32) s.Q[e / n][e % n] = (e / n == e % n) ? T(1) : T(0);
    T fro = T(0);
    for (int e = lane; e < n * n; e += 32) fro += s.G[e / n][e % n] * s.G[e / n][e % n];
    fro = sqrt(wsum(fro));
    const T eps = sizeof(T) == 4 ? T(1e-7) : T(2e-16);
    const int np = n + (n & 1), npairs = np / 2;
    __syncwarp();
    for (int sweep = 0; sweep < 40 && n > 1; ++sweep) {
      int any = 0;
      for (int r = 0; r < np - 1; ++r) {
        int p = 0, q = 0;
        T c = T(1), sn = T(0);
        const bool mine = lane < npairs;
        if (mine) {
          p = lane == 0 ? 0 : 1 + (lane - 1 + r) % (np - 1);
          q = 1 + (np - 2 - lane + r) % (np - 1);
          if (p > q) { const int t = p; p = q; q = t; }
          if (q < n) {
            const T apq = s.G[p][q], app = s.G[p][p], aqq = s.G[q][q];
            if (abs(apq) > eps * fro && abs(apq) > eps * sqrt(abs(app * aqq))) {
              const T th = (aqq - app) / (T(2) * apq);
              const T t = (th >= T(0) ? T(1) : T(-1)) / (abs(th) + sqrt(T(1) + th * th));
              c = T(1) / sqrt(T(1) + t * t);
              sn = t * c;
              any = 1;
            }
          }
        }
        __syncwarp();
        const bool act = mine && q < n && sn != T(0);
        if (act)
          for (int i = 0; i < n; ++i) {  // columns p, q
            const T a = s.G[i][p], b = s.G[i][q];
            s.G[i][p] = c * a - sn * b;
            s.G[i][q] = sn * a + c * b;
          }
        __syncwarp();
        if (act) {
          for (int j = 0; j < n; ++j) {  // rows p, q; vectors
            const T a = s.G[p][j], b = s.G[q][j];
            s.G[p][j] = c * a - sn * b;
            s.G[q][j] = sn * a + c * b;
            const T va = s.Q[j][p], vb = s.Q[j][q];
            s.Q[j][p] = c * va - sn * vb;
            s.Q[j][q] = sn * va + c * vb;
          }
          s.G[p][q] = T(0);
          s.G[q][p] = T(0);
        }
        __syncwarp();
      }
      if (!__any_sync(0xffffffffu, any)) break;
    }
    for (int i = lane; i < n; i += 32) {
      const T di = s.G[i][i];
      int rank = 0;
      for (int j = 0; j < n; ++j) {
        const T dj = s.G[j][j];
        rank += (dj < di) || (dj == di && j < i);
      }
      s.order[rank] = i;
      s.theta[rank] = di;
    }
  }
  __syncthreads();
  // reorder the eigenvector columns (G is free now)
  for (int e = threadIdx.x; e < n * n; e += KT) {
    const int i = e / n, r = e % n;
    s.G[i][r] = s.Q[i][s.order[r]];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += KT) s.Q[e / n][e % n] = s.G[e / n][e % n];
  __syncthreads();
}

// deterministic pseudo-random start vectors in [-1, 1)
__device__ __forceinline__ float hash_unit(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ (c + 0x165667B1u) * 0xC2B2AE3Du;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return float(h) * (2.0f / 4294967296.0f) - 1.0f;
}

// meta[5b..5b+4] = m1, m2, dr2, k, p
template <typename T>
__global__ void __launch_bounds__(KT) kron_chfsi_kernel(const double* const* __restrict__ w1s,
                                                       const double* const* __restrict__ w2s,
                                                       const int* __restrict__ meta, int D, T* __restrict__ work,
                                                       int64_t work_stride, int max_outer, int degree,
                                                       double* __restrict__ vec_base, int64_t vec_stride,
                                                       int* __restrict__ out_iters, int warm) {
  extern __shared__ __align__(16) unsigned char ksm_raw[];
  KSmem<T>& s = *reinterpret_cast<KSmem<T>*>(ksm_raw);
  const int b = blockIdx.x;
  const int m1 = meta[5 * b], m2 = meta[5 * b + 1], dr2 = meta[5 * b + 2], k = meta[5 * b + 3], p = meta[5 * b + 4];
  const int m = m1 * m2;
  const double* W1 = w1s[b];
  const double* W2 = w2s[b];
  for (int e = threadIdx.x; e < D * m1 * m1; e += KT) s.A[e / (m1 * m1)][e % (m1 * m1)] = T(W1[e]);  // row 0
  for (int e = threadIdx.x; e < D * m2 * m2; e += KT) {
    const int w = e / (m2 * m2), r = e % (m2 * m2);
    s.B[w][r] = T(W2[(size_t(w) * dr2 + dr2 - 1) * m2 * m2 + r]);
  }
  __syncthreads();
  // spectral bound: ||H|| <= sum_w ||A_w||_inf ||B_w||_inf (row-sum norms)
  if (threadIdx.x == 0) {
    T bound = T(0);
    for (int w = 0; w < D; ++w) {
      T na = T(0), nb = T(0);
      for (int i = 0; i < m1; ++i) {
        T r = T(0);
        for (int j = 0; j < m1; ++j) r += abs(s.A[w][i * m1 + j]);
        na = r > na ? r : na;
      }
      for (int i = 0; i < m2; ++i) {
        T r = T(0);
        for (int j = 0; j < m2; ++j) r += abs(s.B[w][i * m2 + j]);
        nb = r > nb ? r : nb;
      }
      bound += na * nb;
    }
    s.scal[KP - 1] = bound;
  }
  __syncthreads();
  T* X = work + size_t(b) * work_stride;
  T* Y = X + size_t(p) * m;
  T* Z = Y + size_t(p) * m;
  T* U = Z + size_t(p) * m;
  // Upper end of the spectrum for the filter: 24 Lanczos steps on one vector give the largest
  // Ritz value theta_max; theta_max + |beta_last| (plus 1% of the Ritz range) bounds lambda_max
  // in practice and is far tighter than the norm bound, which caps it. A tighter damping
  // interval makes every filter application converge faster.
  T ub;
  {
    __shared__ double lal[25], lbe[25];
    const int nl = m < 24 ? m : 24;
    T* v = X;
    T* vp = X + m;
    T* w = Y;
    for (int e = threadIdx.x; e < m; e += KT) {
      v[e] = T(hash_unit(b + 7919u, 0u, uint32_t(e)));
      vp[e] = T(0);
    }
    __syncthreads();
    T nv = sqrt(dot1(s, v, v, m));
    for (int e = threadIdx.x; e < m; e += KT) v[e] /= nv;
    __syncthreads();
    T beta = T(0);
    int steps = 0;
    for (int j = 0; j < nl; ++j) {
      kron_apply(s, v, w, 1, m1, m2, D);
      const T alpha = dot1(s, w, v, m);
      for (int e = threadIdx.x; e < m; e += KT) w[e] -= alpha * v[e] + beta * vp[e];
      __syncthreads();
      const T bnew = sqrt(dot1(s, w, w, m));
      if (threadIdx.x == 0) {
        lal[j] = double(alpha);
        lbe[j + 1] = double(bnew);
      }
      steps = j + 1;
      if (!(bnew > T(1e-12) * (abs(alpha) + T(1e-30)))) break;
      for (int e = threadIdx.x; e < m; e += KT) {
        vp[e] = v[e];
        v[e] = w[e] / bnew;
      }
      beta = bnew;
      __syncthreads();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      lbe[0] = 0.0;
      double tmin = lal[0], tmax = lal[0];
      for (int i = 0; i < steps; ++i) {
        tmin = fmin(tmin, lal[i]);
        tmax = fmax(tmax, lal[i]);
      }
      const double top = tridiag_max(lal, lbe, steps);
      double est = top + fabs(lbe[steps]) + 0.01 * fabs(top - tmin) + 1e-12 * fabs(top);
      const double cap = double(s.scal[KP - 1]) * 1.01;
      s.scal[KP - 2] = T(est < cap ? est : cap);
    }
    __syncthreads();
    ub = s.scal[KP - 2] + T(1e-30);
  }
  // start block: random, or (warm) the k vectors a previous stage left in vec_base plus random
  // guard vectors
  const double* prev = vec_base + size_t(b) * vec_stride;
  for (int e = threadIdx.x; e < p * m; e += KT)
    X[e] = (warm && e < k * m) ? T(prev[e]) : T(hash_unit(b, e / m, e % m));
  __syncthreads();
  orthonormalise(s, X, p, m);
  const T tolr = sizeof(T) == 4 ? T(3e-6) : T(1e-13);
  int it = 0;
  for (; it < max_outer; ++it) {
    // Rayleigh-Ritz: Y = H X, G = X^T Y
    kron_apply(s, X, Y, p, m1, m2, D);
    for (int i = 0; i < p; ++i) {
      block_dots(s, Y, X + size_t(i) * m, p, m, s.scal);
      for (int j = threadIdx.x; j < p; j += KT) s.G[i][j] = s.scal[j];
      __syncthreads();
    }
    for (int e = threadIdx.x; e < p * p; e += KT) {
      const int i = e / p, j = e % p;
      if (i < j) {
        const T a = T(0.5) * (s.G[i][j] + s.G[j][i]);
        s.G[i][j] = a;
        s.G[j][i] = a;
      }
    }
    __syncthreads();
    small_eigh(s, p);
    rotate(s, X, Z, p, m);  // Z = X Q (Ritz vectors)
    rotate(s, Y, U, p, m);  // U = H Z
    { T* t = X; X = Z; Z = t; }
    { T* t = Y; Y = U; U = t; }
    // residuals of the k wanted pairs: ||H x_i - theta_i x_i||
    const T scale = abs(s.theta[0]) > abs(s.theta[p - 1]) ? abs(s.theta[0]) : abs(s.theta[p - 1]);
    if (threadIdx.x == 0) s.flag = 1;
    __syncthreads();
    for (int i = 0; i < k; ++i) {
      T part = T(0);
      const T th = s.theta[i];
      for (int e = threadIdx.x; e < m; e += KT) {
        const T r = Y[size_t(i) * m + e] - th * X[size_t(i) * m + e];
        part += r * r;
      }
      part = wsum(part);
      if ((threadIdx.x & 31) == 0) s.red[threadIdx.x >> 5][0] = part;
      __syncthreads();
      if (threadIdx.x == 0) {
        T t = T(0);
        for (int q = 0; q < KT / 32; ++q) t += s.red[q][0];
        if (sqrt(t) > tolr * (scale + T(1e-30))) s.flag = 0;
      }
      __syncthreads();
    }
    if (s.flag) break;
    // Chebyshev filter of degree `degree` on [a, ub], a = largest Ritz value of the block
    const T a = s.theta[p - 1];
    const T c = T(0.5) * (a + ub), h = T(0.5) * (ub - a) + T(1e-30);
    // Z = (Y - c X) / h   (Y = H X)
    for (int e = threadIdx.x; e < p * m; e += KT) Z[e] = (Y[e] - c * X[e]) / h;
    __syncthreads();
    T* prev = X;  // T_0
    T* cur = Z;   // T_1
    for (int d = 2; d <= degree; ++d) {
      kron_apply(s, cur, Y, p, m1, m2, D);  // Y = H cur
      for (int e = threadIdx.x; e < p * m; e += KT) U[e] = T(2) * (Y[e] - c * cur[e]) / h - prev[e];
      __syncthreads();
      // rotate buffers: prev <- cur, cur <- U, U <- old prev
      T* t = prev;
      prev = cur;
      cur = U;
      U = t;
    }
    // the filtered block becomes X; keep the other three buffers distinct
    T* bufs[4] = {X, Y, Z, U};
    (void)bufs;
    X = cur;
    // pick three remaining distinct buffers for Y, Z, U
    {
      T* cand[4] = {prev, U, Y, Z};
      T* rest[3];
      int nr = 0;
      for (int i = 0; i < 4 && nr < 3; ++i) {
        bool dup = cand[i] == X;
        for (int j = 0; j < nr; ++j) dup = dup || cand[i] == rest[j];
        if (!dup) rest[nr++] = cand[i];
      }
      Y = rest[0];
      Z = rest[1];
      U = rest[2];
    }
    orthonormalise(s, X, p, m);
  }
  // write the k lowest Ritz vectors (FP64, vector-major [i][m])
  double* out = vec_base + size_t(b) * vec_stride;
  for (int e = threadIdx.x; e < k * m; e += KT) out[e] = double(X[e]);
  // iterations used, or -max_outer when the wanted residuals never reached the tolerance
  if (threadIdx.x == 0 && out_iters) out_iters[b] = s.flag ? it + 1 : -max_outer;
}

// FP64 Rayleigh-Ritz of the k vectors in vecs[b] (vector-major [k][m]); writes evals[b][i]
// ascending and evecs[b] as [m][k] (row-major, columns = eigenvectors); scratch: 2 k m doubles.
__global__ void __launch_bounds__(KT) kron_refine_kernel(const double* const* __restrict__ w1s,
                                                        const double* const* __restrict__ w2s,
                                                        const int* __restrict__ meta, int D,
                                                        double* __restrict__ vec_base, int64_t vec_stride,
                                                        double* __restrict__ scratch, int64_t scratch_stride,
                                                        double* __restrict__ evals, int keep, double* __restrict__ evecs,
                                                        int max_m) {
  extern __shared__ __align__(16) unsigned char ksm_raw[];
  KSmem<double>& s = *reinterpret_cast<KSmem<double>*>(ksm_raw);
  const int b = blockIdx.x;
  const int m1 = meta[5 * b], m2 = meta[5 * b + 1], dr2 = meta[5 * b + 2], k = meta[5 * b + 3];
  const int m = m1 * m2;
  const double* W1 = w1s[b];
  const double* W2 = w2s[b];
  for (int e = threadIdx.x; e < D * m1 * m1; e += KT) s.A[e / (m1 * m1)][e % (m1 * m1)] = W1[e];
  for (int e = threadIdx.x; e < D * m2 * m2; e += KT) {
    const int w = e / (m2 * m2), r = e % (m2 * m2);
    s.B[w][r] = W2[(size_t(w) * dr2 + dr2 - 1) * m2 * m2 + r];
  }
  __syncthreads();
  double* V = vec_base + size_t(b) * vec_stride;
  double* Zb = scratch + size_t(b) * scratch_stride;
  double* Ub = Zb + size_t(k) * m;
  orthonormalise(s, V, k, m);
  kron_apply(s, V, Zb, k, m1, m2, D);
  for (int i = 0; i < k; ++i) {
    block_dots(s, Zb, V + size_t(i) * m, k, m, s.scal);
    for (int j = threadIdx.x; j < k; j += KT) s.G[i][j] = s.scal[j];
    __syncthreads();
  }
  for (int e = threadIdx.x; e < k * k; e += KT) {
    const int i = e / k, j = e % k;
    if (i < j) {
      const double a = 0.5 * (s.G[i][j] + s.G[j][i]);
      s.G[i][j] = a;
      s.G[j][i] = a;
    }
  }
  __syncthreads();
  small_eigh(s, k);
  rotate(s, V, Ub, k, m);
  double* ev = evals + size_t(b) * keep;
  for (int i = threadIdx.x; i < k; i += KT) ev[i] = s.theta[i];
  double* out = evecs + size_t(b) * max_m * keep;  // [max_m][keep], like tnx_eigh_batched
  for (int e = threadIdx.x; e < k * m; e += KT) {
    const int i = e / m, row = e % m;
    out[size_t(row) * keep + i] = Ub[e];
  }
}

}  // namespace

size_t kron_smem_bytes(bool fp64) { return fp64 ? sizeof(KSmem<double>) : sizeof(KSmem<float>); }

}  // namespace tnx

using namespace tnx;

extern "C" {

size_t tnx_tsdrg_block_eigh_workspace_bytes(int batch, int max_m, int keep, int precision) {
  const size_t tsize = precision == TNX_FP64 ? 8 : 4;
  const size_t per_work = align_up(4 * size_t(KP) * max_m * tsize);
  const size_t per_vec = align_up(size_t(keep) * max_m * 8);
  const size_t per_scr = align_up(2 * size_t(keep) * max_m * 8);
  return size_t(batch) * (per_work + per_vec + per_scr) + 1024;
}

int tnx_tsdrg_block_eigh(const double* const* w1, const double* const* w2, const int* meta, int D, int batch,
                         int max_m, int keep, int precision, double* evals, double* evecs, int* iters,
                         void* workspace, size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(w1 && w2 && meta && evals && evecs && workspace, "null pointer");
  TNX_CHECK_ARG(batch >= 0 && D > 0 && D <= KD && keep > 0 && keep <= 32, "bad batch / D / keep");
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  TNX_CHECK_SHAPE(max_m > 0 && max_m <= KM1 * KM1, "block dimension %d outside (0, %d]", max_m, KM1 * KM1);
  if (batch == 0) return TNX_OK;
  const size_t need = tnx_tsdrg_block_eigh_workspace_bytes(batch, max_m, keep, precision);
  if (workspace_bytes < need) {
    set_error("tnx_tsdrg_block_eigh: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  const bool fp64 = precision == TNX_FP64;
  const size_t tsize = fp64 ? 8 : 4;
  const size_t per_work = align_up(4 * size_t(KP) * max_m * tsize);
  const size_t per_vec = align_up(size_t(keep) * max_m * 8);
  const size_t per_scr = align_up(2 * size_t(keep) * max_m * 8);
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  char* work = base;
  double* vecs = reinterpret_cast<double*>(work + size_t(batch) * per_work);
  double* scr = reinterpret_cast<double*>(reinterpret_cast<char*>(vecs) + size_t(batch) * per_vec);
  const int max_outer = 60, degree = 10;
  if (fp64) {
    static std::atomic<bool> attr{false};  // idempotent setup; threads may race to it
    if (!attr.load()) {
      TNX_CUDA(cudaFuncSetAttribute(kron_chfsi_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(sizeof(KSmem<double>))));
      attr.store(true);
    }
    static std::atomic<bool> fattr{false};  // idempotent setup; threads may race to it
    if (!fattr.load()) {
      TNX_CUDA(cudaFuncSetAttribute(kron_chfsi_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(sizeof(KSmem<float>))));
      fattr.store(true);
    }
    // FP32 iterations to the FP32 rounding level, then FP64 iterations from that subspace:
    // the FP64 pipe (~2 FMA/clock/SM) only has to take the last digits
    profile_mark(KF_EIGH, st, true);
    kron_chfsi_kernel<float><<<batch, KT, sizeof(KSmem<float>), st>>>(
        w1, w2, meta, D, reinterpret_cast<float*>(work), int64_t(per_work / 4), max_outer, degree, vecs,
        int64_t(per_vec / 8), nullptr, 0);
    TNX_LAUNCH_CHECK();
    kron_chfsi_kernel<double><<<batch, KT, sizeof(KSmem<double>), st>>>(
        w1, w2, meta, D, reinterpret_cast<double*>(work), int64_t(per_work / 8), max_outer, degree, vecs,
        int64_t(per_vec / 8), iters, 1);
    profile_mark(KF_EIGH, st, false);
  } else {
    static std::atomic<bool> attr{false};  // idempotent setup; threads may race to it
    if (!attr.load()) {
      TNX_CUDA(cudaFuncSetAttribute(kron_chfsi_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(sizeof(KSmem<float>))));
      attr.store(true);
    }
    profile_mark(KF_EIGH, st, true);
    kron_chfsi_kernel<float><<<batch, KT, sizeof(KSmem<float>), st>>>(
        w1, w2, meta, D, reinterpret_cast<float*>(work), int64_t(per_work / 4), max_outer, degree, vecs,
        int64_t(per_vec / 8), iters, 0);
    profile_mark(KF_EIGH, st, false);
  }
  TNX_LAUNCH_CHECK();
  static std::atomic<bool> rattr{false};  // idempotent setup; threads may race to it
  if (!rattr.load()) {
    TNX_CUDA(cudaFuncSetAttribute(kron_refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(sizeof(KSmem<double>))));
    rattr.store(true);
  }
  kron_refine_kernel<<<batch, KT, sizeof(KSmem<double>), st>>>(w1, w2, meta, D, vecs, int64_t(per_vec / 8), scr,
                                                               int64_t(per_scr / 8), evals, keep, evecs, max_m);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

}  // extern "C"
