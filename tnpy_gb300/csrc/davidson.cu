// Lowest eigenpair of the one-site effective Hamiltonian: a Davidson eigensolver that
// stays on the device, replacing linalg.eigshmv -> primme.eigsh(k=1, which='SA')
// (tnpy/linalg.py:64-87) called from FiniteDMRG.one_site_solver (tnpy/finite_dmrg.py:97-111).
//
// Basis V (orthonormal; FP64, or FP32 in the mixed form's first phase) and AV = H V live in the
// caller's workspace; each expansion
//   1. orthogonalises the new direction against V (classical Gram-Schmidt, FP64, with a
//      second pass when the first removed more than half of its norm: DGKS),
//   2. applies H (FP64, double-FP32 or split-BF16 tensor-core matvec),
//   3. extends the projected matrix V^T H V (FP64 dots),
//   4. solves it for the lowest pair (Jacobi Rayleigh-Ritz, FP32 + FP64 correction),
//   5. forms the Ritz vector, the residual r = H x - theta x and its norm, and the next
//      direction t = r / (diag(H) - theta) (diagonal preconditioner).
// The host loop reads three scalars per expansion to decide convergence. With the
// split-BF16 matvec a second, anchored phase takes the residual from the split-BF16
// floor to FP64-class accuracy: one FP64-class matvec (tensor-core Ozaki GEMMs where large,
// double-FP32 otherwise) per anchor; a start vector already near that floor goes to the
// anchored phase after one matvec (see davidson1).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

constexpr int DT = 256;     // threads per block of the vector kernels
constexpr int MAXB = 64;    // largest basis

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// part[j*nchunk + chunk] = sum over the chunk of V[j][i] * w[i], j < k. With a gate (|t|^2
// before and after one Gram-Schmidt pass), the pass is skipped (zero partials) when the first
// pass kept at least half of |t|^2: the DGKS criterion for a second classical Gram-Schmidt pass.
__device__ __forceinline__ bool gs_pass_skipped(const double* gate) { return gate && gate[1] >= 0.5 * gate[0]; }

// T = double (FP64 arithmetic) or float (FP32 products and per-thread sums, FP64 block sums)
template <typename T>
__global__ void __launch_bounds__(DT) dots_kernel(const T* __restrict__ V, int64_t ldv,
                                                 const T* __restrict__ w, int64_t n,
                                                 double* __restrict__ part, int nchunk,
                                                 const double* __restrict__ gate) {
  __shared__ double sh[DT / 32];
  const int j = blockIdx.y, chunk = blockIdx.x;
  if (gs_pass_skipped(gate)) {
    if (threadIdx.x == 0) part[j * nchunk + chunk] = 0.0;
    return;
  }
  const T* v = V + int64_t(j) * ldv;
  T acc0 = T(0), acc1 = T(0);
  const int64_t stride = int64_t(nchunk) * DT;
  int64_t i = int64_t(chunk) * DT + threadIdx.x;
  for (; i + stride < n; i += 2 * stride) {
    acc0 = fma(v[i], w[i], acc0);
    acc1 = fma(v[i + stride], w[i + stride], acc1);
  }
  if (i < n) acc0 = fma(v[i], w[i], acc0);
  const double acc = block_sum(double(acc0) + double(acc1), sh);
  if (threadIdx.x == 0) part[j * nchunk + chunk] = acc;
}

// out[j * out_stride] = sum_c part[j*nchunk + c]  (fixed order: deterministic)
// optionally also mirrors into out2[j * out2_stride] (symmetric fill of the projected matrix)
__global__ void __launch_bounds__(DT) reduce_kernel(const double* __restrict__ part, int nchunk,
                                                   double* __restrict__ out, int out_stride,
                                                   double* __restrict__ out2, int out2_stride) {
  __shared__ double sh[DT / 32];
  const int j = blockIdx.x;
  double acc = 0.0;
  for (int c = threadIdx.x; c < nchunk; c += DT) acc += part[j * nchunk + c];
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    out[j * out_stride] = acc;
    if (out2) out2[j * out2_stride] = acc;
  }
}

// w -= sum_{j<k} h[j] V[j]; partial ||w||^2 (a skipped gated pass only recomputes the norm)
template <typename T>
__global__ void __launch_bounds__(DT) update_kernel(const T* __restrict__ V, int64_t ldv, int k,
                                                   const double* __restrict__ h, T* __restrict__ w,
                                                   int64_t n, double* __restrict__ part, int nchunk,
                                                   const double* __restrict__ gate) {
  __shared__ double sh[DT / 32];
  __shared__ T hs[MAXB];
  const bool skip = gs_pass_skipped(gate);
  if (threadIdx.x < k) hs[threadIdx.x] = T(h[threadIdx.x]);
  __syncthreads();
  T nrm = T(0);
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(nchunk) * DT) {
    T acc = w[i];
    if (!skip) {
      int j = 0;
      for (; j + 4 <= k; j += 4) {
        const T v0 = V[int64_t(j) * ldv + i], v1 = V[int64_t(j + 1) * ldv + i];
        const T v2 = V[int64_t(j + 2) * ldv + i], v3 = V[int64_t(j + 3) * ldv + i];
        acc = fma(-hs[j], v0, acc);
        acc = fma(-hs[j + 1], v1, acc);
        acc = fma(-hs[j + 2], v2, acc);
        acc = fma(-hs[j + 3], v3, acc);
      }
      for (; j < k; ++j) acc = fma(-hs[j], V[int64_t(j) * ldv + i], acc);
      w[i] = acc;
    }
    nrm = fma(acc, acc, nrm);
  }
  const double tot = block_sum(double(nrm), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// w *= 1/sqrt(nrm2[0])
template <typename T>
__global__ void scale_kernel(T* __restrict__ w, int64_t n, const double* __restrict__ nrm2) {
  const T s = T(1.0 / sqrt(nrm2[0]));
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    w[i] *= s;
}

// part[block] = max |v| over the block's grid-stride share; then max over the partials (one block)
__global__ void __launch_bounds__(DT) absmax_kernel(const double* __restrict__ v, int64_t n, double* __restrict__ part,
                                                   int nchunk) {
  __shared__ double sh[DT / 32];
  double m = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(nchunk) * DT) m = fmax(m, fabs(v[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 0; w < DT / 32; ++w) m = fmax(m, sh[w]);
    part[blockIdx.x] = m;
  }
}

__global__ void max_reduce_kernel(const double* __restrict__ part, int nchunk, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int c = 0; c < nchunk; ++c) m = fmax(m, part[c]);
    out[0] = m;
  }
}

// out = T(in) (precision change of one vector)
template <typename Tin, typename Tout>
__global__ void convert_kernel(const Tin* __restrict__ in, Tout* __restrict__ out, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = Tout(in[i]);
}

// x = V s, ax = AV s, r = ax - theta x, t = r / (diag - theta) (or r), partial ||r||^2
template <typename T>
__global__ void __launch_bounds__(DT) ritz_kernel(const T* __restrict__ V, const T* __restrict__ AV,
                                                 int64_t ldv, int k, const double* __restrict__ s,
                                                 const double* __restrict__ theta_p,
                                                 const T* __restrict__ diag, int precond,
                                                 T* __restrict__ x, T* __restrict__ ax,
                                                 T* __restrict__ t, int64_t n,
                                                 double* __restrict__ part, int nchunk) {
  __shared__ double sh[DT / 32];
  __shared__ T ss[MAXB];
  if (threadIdx.x < k) ss[threadIdx.x] = T(s[threadIdx.x]);
  __syncthreads();
  const T theta = T(theta_p[0]);
  T nrm = T(0);
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(nchunk) * DT) {
    T xv = T(0), av = T(0), xw = T(0), aw = T(0);
    int j = 0;
    for (; j + 2 <= k; j += 2) {
      const T v0 = V[int64_t(j) * ldv + i], v1 = V[int64_t(j + 1) * ldv + i];
      const T a0 = AV[int64_t(j) * ldv + i], a1 = AV[int64_t(j + 1) * ldv + i];
      xv = fma(ss[j], v0, xv);
      av = fma(ss[j], a0, av);
      xw = fma(ss[j + 1], v1, xw);
      aw = fma(ss[j + 1], a1, aw);
    }
    if (j < k) {
      xv = fma(ss[j], V[int64_t(j) * ldv + i], xv);
      av = fma(ss[j], AV[int64_t(j) * ldv + i], av);
    }
    xv += xw;
    av += aw;
    const T r = av - theta * xv;
    x[i] = xv;
    ax[i] = av;
    T tv = r;
    if (precond) {
      T den = diag[i] - theta;
      const T floor = T(1e-2);
      if (abs(den) < floor) den = den >= T(0) ? floor : -floor;
      tv = r / den;
    }
    t[i] = tv;
    nrm = fma(r, r, nrm);
  }
  const double tot = block_sum(double(nrm), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// generalised form: x = V s, ax = AV s, bx = BV s, r = ax - theta bx,
// t = r / (diagA - theta diagB), partial ||r||^2 (FP64)
__global__ void __launch_bounds__(DT) gritz_kernel(const double* __restrict__ V, const double* __restrict__ AV,
                                                  const double* __restrict__ BV, int64_t ldv, int k,
                                                  const double* __restrict__ s, const double* __restrict__ theta_p,
                                                  const double* __restrict__ da, const double* __restrict__ db,
                                                  double* __restrict__ x, double* __restrict__ ax,
                                                  double* __restrict__ bx, double* __restrict__ t, int64_t n,
                                                  double* __restrict__ part, int nchunk) {
  __shared__ double sh[DT / 32];
  __shared__ double ss[MAXB];
  if (threadIdx.x < k) ss[threadIdx.x] = s[threadIdx.x];
  __syncthreads();
  const double theta = theta_p[0];
  double nrm = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(nchunk) * DT) {
    double xv = 0.0, av = 0.0, bv = 0.0;
    for (int j = 0; j < k; ++j) {
      xv = fma(ss[j], V[int64_t(j) * ldv + i], xv);
      av = fma(ss[j], AV[int64_t(j) * ldv + i], av);
      bv = fma(ss[j], BV[int64_t(j) * ldv + i], bv);
    }
    const double r = av - theta * bv;
    x[i] = xv;
    ax[i] = av;
    bx[i] = bv;
    double den = da[i] - theta * db[i];
    if (fabs(den) < 1e-2) den = den >= 0.0 ? 1e-2 : -1e-2;
    t[i] = r / den;
    nrm = fma(r, r, nrm);
  }
  const double tot = block_sum(nrm, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// w2 -= sum_{j<k} h[j] V2[j] (the B-images follow the same combination as the vectors)
__global__ void __launch_bounds__(DT) axpy_basis_kernel(const double* __restrict__ V2, int64_t ldv, int k,
                                                       const double* __restrict__ h, double* __restrict__ w2,
                                                       int64_t n) {
  __shared__ double hs[MAXB];
  if (threadIdx.x < k) hs[threadIdx.x] = h[threadIdx.x];
  __syncthreads();
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(gridDim.x) * DT) {
    double acc = w2[i];
    for (int j = 0; j < k; ++j) acc = fma(-hs[j], V2[int64_t(j) * ldv + i], acc);
    w2[i] = acc;
  }
}

// w *= 1/sqrt(nrm2[0]) for two vectors at once
__global__ void scale2_kernel(double* __restrict__ w, double* __restrict__ w2, int64_t n,
                              const double* __restrict__ nrm2) {
  const double s = 1.0 / sqrt(nrm2[0]);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    w[i] *= s;
    w2[i] *= s;
  }
}

// after a restart to the single Ritz vector x: H = [[theta]], Ritz coefficients s = [1]
__global__ void restart_kernel(double* Hm, const double* evals, double* evecs) {
  Hm[0] = evals[0];
  evecs[0] = 1.0;
}

// out_v = V s, out_av = AV s over the first k basis vectors (the second vector of a GD+1 restart)
template <typename T>
__global__ void __launch_bounds__(DT) lincomb_kernel(const T* __restrict__ V, const T* __restrict__ AV, int64_t ldv,
                                                    int k, const double* __restrict__ s, T* __restrict__ out_v,
                                                    T* __restrict__ out_av, int64_t n) {
  __shared__ T ss[MAXB];
  if (threadIdx.x < k) ss[threadIdx.x] = T(s[threadIdx.x]);
  __syncthreads();
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(gridDim.x) * DT) {
    T xv = T(0), av = T(0);
    for (int j = 0; j < k; ++j) {
      xv = fma(ss[j], V[int64_t(j) * ldv + i], xv);
      av = fma(ss[j], AV[int64_t(j) * ldv + i], av);
    }
    out_v[i] = xv;
    out_av[i] = av;
  }
}

inline int nchunk_for(int64_t n) {
  int64_t c = (n + DT * 4 - 1) / (DT * 4);
  if (c > 2 * 152) c = 2 * 152;
  return int(c < 1 ? 1 : c);
}

struct DavWs {
  double *V, *AV, *x, *ax, *t, *diag, *Hm, *Hwork, *evals, *evecs, *jwork, *part, *scal;
  double *xp, *axp;  // second vector of a GD+1 restart (previous Ritz vector, orthogonalised)
  void* mv;
  size_t mv_bytes;
  double *T1, *T2;  // FP64-class matvec scratch (also used by the anchored phase)
  float* diag32;     // diag(H) in FP32 for the mixed form's first phase
  void* oz;         // operand slices of the tensor-core FP64-class GEMMs
  size_t oz_bytes;
};

size_t dav_layout(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, int mb, int precision,
                  void* base, size_t size, DavWs* w) {
  const int64_t n = chi_l * d * chi_r;
  const int64_t ne = matvec1_scratch_elems(chi_l, d, chi_r, dl, dr);
  const size_t mv_bytes = (precision == TNX_BF16X3 && mixed_supported(chi_l, d, chi_r, dl, dr))
                              ? matvec1_bf16x3_scratch_bytes(chi_l, d, chi_r, dl, dr)
                              : 0;
  const size_t oz_bytes =
      (precision == TNX_BF16X3 || precision == TNX_DF64) ? matvec1_oz_bytes(chi_l, d, chi_r, dl, dr) : 0;
  const int nch = nchunk_for(n);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align_up(bytes);
    return o;
  };
  size_t oV = take(size_t(mb) * n * 8), oAV = take(size_t(mb) * n * 8), ox = take(n * 8),
         oax = take(n * 8), ot = take(n * 8), odiag = take(n * 8), oH = take(size_t(mb) * mb * 8),
         oHw = take(size_t(mb) * mb * 8), oev = take(size_t(mb) * 8), oevec = take(size_t(mb) * mb * 8),
         ojw = take(2 * size_t(mb) * mb * 8), opart = take(size_t(mb + 1) * nch * 8),
         oscal = take(size_t(4 * MAXB) * 8), oT1 = take(ne * 8), oT2 = take(ne * 8), omv = take(mv_bytes),
         ooz = take(oz_bytes), od32 = take(precision == TNX_BF16X3 ? size_t(n) * 4 : 0), oxp = take(n * 8),
         oaxp = take(n * 8);
  if (w && base && off <= size) {
    char* b = static_cast<char*>(base);
    w->V = reinterpret_cast<double*>(b + oV);
    w->AV = reinterpret_cast<double*>(b + oAV);
    w->x = reinterpret_cast<double*>(b + ox);
    w->ax = reinterpret_cast<double*>(b + oax);
    w->t = reinterpret_cast<double*>(b + ot);
    w->diag = reinterpret_cast<double*>(b + odiag);
    w->Hm = reinterpret_cast<double*>(b + oH);
    w->Hwork = reinterpret_cast<double*>(b + oHw);
    w->evals = reinterpret_cast<double*>(b + oev);
    w->evecs = reinterpret_cast<double*>(b + oevec);
    w->jwork = reinterpret_cast<double*>(b + ojw);
    w->part = reinterpret_cast<double*>(b + opart);
    w->scal = reinterpret_cast<double*>(b + oscal);
    w->T1 = reinterpret_cast<double*>(b + oT1);
    w->T2 = reinterpret_cast<double*>(b + oT2);
    w->mv = mv_bytes ? static_cast<void*>(b + omv) : nullptr;
    w->mv_bytes = mv_bytes;
    w->oz = oz_bytes ? static_cast<void*>(b + ooz) : nullptr;
    w->oz_bytes = oz_bytes;
    w->diag32 = precision == TNX_BF16X3 ? reinterpret_cast<float*>(b + od32) : nullptr;
    w->xp = reinterpret_cast<double*>(b + oxp);
    w->axp = reinterpret_cast<double*>(b + oaxp);
  }
  return off;
}

// h[0..k) = V[0..k) . w
template <typename T>
int dots(const T* V, int64_t ldv, int k, const T* w, int64_t n, double* part, double* out,
         int out_stride, double* out2, int out2_stride, cudaStream_t st, const double* gate = nullptr) {
  const int nch = nchunk_for(n);
  dots_kernel<T><<<dim3(nch, k), DT, 0, st>>>(V, ldv, w, n, part, nch, gate);
  TNX_LAUNCH_CHECK();
  reduce_kernel<<<k, DT, 0, st>>>(part, nch, out, out_stride, out2, out2_stride);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

}  // namespace

// Counters of the calling thread's last davidson1 call (tnx_davidson1_stats)
struct DavStats {
  int phase1 = 0, anchored = 0, anchors = 0, restarts = 0;
};
thread_local DavStats g_dav_stats;

// Davidson driver. All pointers device; eval/resid/iters host.
int davidson1(const double* L, const double* W, const double* R, double* x_io, int64_t chi_l, int64_t d,
              int64_t chi_r, int64_t dl, int64_t dr, double tol, int max_iter, int mb, int precision,
              double* eval_out, double* resid_out, int* iters_out, void* ws, size_t ws_bytes,
              cudaStream_t st, int flags = 0) {
  DavWs w;
  const size_t need = dav_layout(chi_l, d, chi_r, dl, dr, mb, precision, ws, ws_bytes, &w);
  if (ws_bytes < need || !ws) {
    set_error("tnx_davidson1: workspace %zu bytes < required %zu", ws_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  const int64_t n = chi_l * d * chi_r;
  const int nch = nchunk_for(n);
  const unsigned sblocks = (unsigned)((n + DT - 1) / DT < 152 * 8 ? (n + DT - 1) / DT : 152 * 8);
  if (mb > n) mb = int(n);
  if (mb < 2) mb = 2;
  const bool mixed = precision == TNX_BF16X3 && w.mv != nullptr;
  // mixed form, start vector expected at the answer (the site converged in the previous sweep):
  // certify it with the FP64-class anchor at once instead of a first split-BF16 phase that
  // would only hand over after its first product
  const bool start_anchored = mixed && (flags & TNX_DAV_START_ANCHORED);
  int* dflag = nullptr;
  // Vector storage of the current phase. The mixed form's first phase (split-BF16 products,
  // converged only to ~3e-6) keeps its basis, Ritz vector and residual in FP32 views of the
  // same buffers: half the bytes, and FP32 instead of FP64-pipe arithmetic in every vector
  // kernel; the anchored phase restarts from the Ritz vector converted to FP64.
  struct Vecs32 {
    float *V, *AV, *x, *ax, *t, *diag;
  };
  struct Vecs64 {
    double *V, *AV, *x, *ax, *t, *diag;
  };
  const Vecs32 v32{reinterpret_cast<float*>(w.V), reinterpret_cast<float*>(w.AV), reinterpret_cast<float*>(w.x),
                   reinterpret_cast<float*>(w.ax), reinterpret_cast<float*>(w.t), w.diag32};
  const Vecs64 v64{w.V, w.AV, w.x, w.ax, w.t, w.diag};
  const bool f32 = mixed && w.diag32 != nullptr;
  auto matvec = [&](auto* in, auto* out) -> int {
    using T = std::remove_const_t<std::remove_pointer_t<decltype(in)>>;
    if constexpr (std::is_same_v<T, float>) {
      return mixed_apply_f32(W, in, out, chi_l, d, chi_r, dl, dr, w.mv, st);
    } else {
      if (mixed) return mixed_apply(W, in, out, chi_l, d, chi_r, dl, dr, w.mv, st);
      return matvec1_f64(L, W, R, in, out, chi_l, d, chi_r, dl, dr, w.T1, w.T2, st, precision == TNX_DF64, w.oz,
                         w.oz_bytes);
    }
  };
  int hflag = 0;
  double* h = w.scal;               // [MAXB]
  double* nrm2 = w.scal + MAXB;     // [2]: |t|^2 before, after orthogonalisation
  double* rn2 = w.scal + MAXB + 2;  // ||r||^2
  double host[4];

  // Operands of the expansions: the split-BF16 layout of L and R (mixed form), diag(H) for the
  // preconditioner and max |diag H| for the operator scale. A settled site that the first anchor
  // certifies needs none of them, so they are prepared on first use.
  bool prepared = false;
  double hdiag = 0.0;
  auto prepare = [&]() -> int {
    if (prepared) return TNX_OK;
    prepared = true;
    if (mixed) {
      TNX_TRY(mixed_prepare(L, R, chi_l, d, chi_r, dl, dr, w.mv, st));
      mixed_flag(w.mv, chi_l, d, chi_r, dl, dr, &dflag);
    }
    if (int e = tnx_diag1(L, W, R, w.diag, chi_l, d, chi_r, dl, dr, st); e != TNX_OK) return e;
    if (f32) {
      convert_kernel<double, float><<<sblocks, DT, 0, st>>>(w.diag, w.diag32, n);
      TNX_LAUNCH_CHECK();
    }
    // max |diag H|: with 2 |theta| it estimates |H| for the floors and bounds below (the
    // diagonal alone is a lower bound of the spectral radius and catches operators whose lowest
    // eigenvalue is small against their width)
    absmax_kernel<<<nch, DT, 0, st>>>(w.diag, n, w.part, nch);
    TNX_LAUNCH_CHECK();
    max_reduce_kernel<<<1, 32, 0, st>>>(w.part, nch, w.scal + MAXB + 3);
    TNX_LAUNCH_CHECK();
    TNX_CUDA(cudaMemcpyAsync(&hdiag, w.scal + MAXB + 3, 8, cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaStreamSynchronize(st));
    return TNX_OK;
  };
  if (f32) {
    convert_kernel<double, float><<<sblocks, DT, 0, st>>>(x_io, v32.t, n);
    TNX_LAUNCH_CHECK();
  } else {
    TNX_CUDA(cudaMemcpyAsync(w.t, x_io, n * 8, cudaMemcpyDeviceToDevice, st));
  }

  int k = 0, iters = 0, precond = 1;
  double theta = 0.0, rnorm = INFINITY, c0 = 1.0;
  // Ritz coefficients of the last two Rayleigh-Ritz steps (host copies) for the GD+1 restart:
  // s_prev is valid when it was computed on the basis V[0..k-1) that the current one extends.
  std::vector<double> s_cur(MAXB, 0.0), s_prev(MAXB, 0.0), hm_host(size_t(MAXB) * MAXB, 0.0);
  int cur_k = 0, prev_k = 0;

  // Rayleigh-Ritz on V[0..k), Ritz vector x, AV-combination ax, residual norm and the next
  // direction t; reads theta, ||r|| and the Ritz coefficient of V[0] back to the host.
  auto rayleigh_ritz = [&](const auto& vs) -> int {
    TNX_TRY(rr_lowest_f64(w.Hm, k, mb, w.evals, w.evecs, st));
    ritz_kernel<<<nch, DT, 0, st>>>(vs.V, vs.AV, n, k, w.evecs, w.evals, vs.diag, precond, vs.x, vs.ax, vs.t, n,
                                    w.part, nch);
    TNX_LAUNCH_CHECK();
    reduce_kernel<<<1, DT, 0, st>>>(w.part, nch, rn2, 1, nullptr, 0);
    TNX_LAUNCH_CHECK();
    TNX_CUDA(cudaMemcpyAsync(host, w.evals, 8, cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaMemcpyAsync(host + 1, rn2, 8, cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaMemcpyAsync(host + 2, w.evecs, 8, cudaMemcpyDeviceToHost, st));
    std::swap(s_prev, s_cur);
    prev_k = cur_k;
    TNX_CUDA(cudaMemcpyAsync(s_cur.data(), w.evecs, size_t(k) * 8, cudaMemcpyDeviceToHost, st));
    cur_k = k;
    if (dflag) TNX_CUDA(cudaMemcpyAsync(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaStreamSynchronize(st));
    if (hflag) {
      set_error("tnx_davidson1: a bounded wait in the tensor-core matvec expired");
      return TNX_ERR_TIMEOUT;
    }
    theta = host[0];
    rnorm = sqrt(fmax(host[1], 0.0));
    c0 = host[2];
    if (!std::isfinite(theta) || !std::isfinite(rnorm)) {
      set_error("tnx_davidson1: non-finite Ritz value or residual");
      return TNX_ERR_INVALID_ARG;
    }
    return TNX_OK;
  };

  // One expansion: t -> V[k] (classical Gram-Schmidt, second pass by the DGKS criterion),
  // AV[k] = H V[k], column k of V^T H V, Rayleigh-Ritz. With `anchored`, V[0] is a vector whose
  // product AV[0] = H V[0] is FP64-class exact, and row 0 of the projected matrix is taken as
  // AV[0] . V[k] (exact, H being symmetric) instead of V[0] . AV[k]. `*fell_in` reports a
  // direction that vanished against the basis (nothing expanded).
  auto expand = [&](const auto& vs, bool anchored, bool* fell_in) -> int {
    using T = std::remove_pointer_t<decltype(vs.V)>;
    *fell_in = false;
    T* vk = vs.V + int64_t(k) * n;
    TNX_CUDA(cudaMemcpyAsync(vk, vs.t, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    TNX_TRY(dots<T>(vk, n, 1, vk, n, w.part, nrm2, 1, nullptr, 0, st));
    for (int pass = 0; pass < 2 && k > 0; ++pass) {
      const double* gate = pass == 0 ? nullptr : nrm2;
      TNX_TRY(dots<T>(vs.V, n, k, vk, n, w.part, h, 1, nullptr, 0, st, gate));
      update_kernel<T><<<nch, DT, 0, st>>>(vs.V, n, k, h, vk, n, w.part, nch, gate);
      TNX_LAUNCH_CHECK();
      reduce_kernel<<<1, DT, 0, st>>>(w.part, nch, nrm2 + 1, 1, nullptr, 0);
      TNX_LAUNCH_CHECK();
    }
    if (k == 0) TNX_CUDA(cudaMemcpyAsync(nrm2 + 1, nrm2, 8, cudaMemcpyDeviceToDevice, st));
    TNX_CUDA(cudaMemcpyAsync(host, nrm2, 16, cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaStreamSynchronize(st));
    if (!(host[1] > 1e-26 * host[0]) || !(host[1] > 0.0) || !std::isfinite(host[1])) {
      if (k == 0) {
        set_error("tnx_davidson1: zero or non-finite start vector");
        return TNX_ERR_INVALID_ARG;
      }
      *fell_in = true;
      return TNX_OK;
    }
    scale_kernel<T><<<sblocks, DT, 0, st>>>(vk, n, nrm2 + 1);
    TNX_LAUNCH_CHECK();
    T* avk = vs.AV + int64_t(k) * n;
    TNX_TRY(matvec(vk, avk));
    ++iters;
    TNX_TRY(dots<T>(vs.V, n, k + 1, avk, n, w.part, w.Hm + k, mb, w.Hm + int64_t(k) * mb, 1, st));
    if (anchored && k > 0)
      TNX_TRY(dots<T>(vs.AV, n, 1, vk, n, w.part, w.Hm + k, mb, w.Hm + int64_t(k) * mb, 1, st));
    ++k;
    return rayleigh_ritz(vs);
  };

  // thick restart with the current Ritz vector
  auto restart = [&](const auto& vs) -> int {
    using T = std::remove_pointer_t<decltype(vs.V)>;
    TNX_CUDA(cudaMemcpyAsync(vs.V, vs.x, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    TNX_CUDA(cudaMemcpyAsync(vs.AV, vs.ax, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    restart_kernel<<<1, 1, 0, st>>>(w.Hm, w.evals, w.evecs);
    TNX_LAUNCH_CHECK();
    k = 1;
    cur_k = prev_k = 0;
    return TNX_OK;
  };

  // GD+1 restart (the "+k" of primme's GD+k, k = 1): keep the Ritz vector x = V s and the
  // previous step's Ritz vector V s_prev orthogonalised against it, s' = s_prev - (s.s_prev) s
  // (V is orthonormal, so this is done on the coefficients). The 2 x 2 projected matrix is
  // [s s']^T H_k [s s'] from the current projected matrix H_k. Far from convergence this keeps
  // the search direction a one-vector restart throws away; it falls back to that restart when
  // the previous vector is not available or lies along x.
  auto restart_plus = [&](const auto& vs) -> int {
    using T = std::remove_pointer_t<decltype(vs.V)>;
    if (prev_k != k - 1 || cur_k != k || k < 2) return restart(vs);
    double dot = 0.0;
    for (int j = 0; j < k - 1; ++j) dot += s_cur[j] * s_prev[j];
    double sp[MAXB], nrm = 0.0;
    for (int j = 0; j < k; ++j) {
      sp[j] = (j < k - 1 ? s_prev[j] : 0.0) - dot * s_cur[j];
      nrm += sp[j] * sp[j];
    }
    nrm = sqrt(nrm);
    if (!(nrm > 1e-6)) return restart(vs);
    for (int j = 0; j < k; ++j) sp[j] /= nrm;
    TNX_CUDA(cudaMemcpy2DAsync(hm_host.data(), size_t(k) * 8, w.Hm, size_t(mb) * 8, size_t(k) * 8, size_t(k),
                               cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaStreamSynchronize(st));
    double h01 = 0.0, h11 = 0.0;
    for (int i = 0; i < k; ++i) {
      double hs = 0.0;
      for (int j = 0; j < k; ++j) hs += hm_host[size_t(i) * k + j] * sp[j];
      h01 += s_cur[i] * hs;
      h11 += sp[i] * hs;
    }
    double* dsp = w.scal + 2 * MAXB;  // free part of the scalar block
    TNX_CUDA(cudaMemcpyAsync(dsp, sp, size_t(k) * 8, cudaMemcpyHostToDevice, st));
    T* xp = reinterpret_cast<T*>(w.xp);
    T* axp = reinterpret_cast<T*>(w.axp);
    lincomb_kernel<T><<<sblocks, DT, 0, st>>>(vs.V, vs.AV, n, k, dsp, xp, axp, n);
    TNX_LAUNCH_CHECK();
    TNX_CUDA(cudaMemcpyAsync(vs.V, vs.x, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    TNX_CUDA(cudaMemcpyAsync(vs.AV, vs.ax, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    TNX_CUDA(cudaMemcpyAsync(vs.V + n, xp, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    TNX_CUDA(cudaMemcpyAsync(vs.AV + n, axp, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    const double h2[4] = {theta, h01, h01, h11};
    TNX_CUDA(cudaMemcpy2DAsync(w.Hm, size_t(mb) * 8, h2, 16, 16, 2, cudaMemcpyHostToDevice, st));
    TNX_CUDA(cudaStreamSynchronize(st));  // h2 / sp are host stack memory
    k = 2;
    cur_k = prev_k = 0;
    return TNX_OK;
  };

  if (!start_anchored) TNX_TRY(prepare());
  auto hscale = [&]() { return fmax(fmax(2.0 * fabs(theta), hdiag), 1.0); };

  bool converged = false;
  int restarts = 0, anchors = 0, phase1 = 0;
  // Stagnation: the split-BF16 operand is not exactly symmetric, so the residual of the
  // mixed operator stops falling at ~1e-5 |H| (its rounding floor). The first phase treats
  // "no 10% gain within `patience` matvecs" as that floor only when the residual is already
  // within ~10x of it (below 1e-4 |H|); further out a Davidson residual can plateau for tens of
  // matvecs while theta still falls (hard starts of a first sweep, small local gaps), and the
  // phase keeps expanding, with GD+1 restarts, until max_iter. The FP64 forms treat
  // stagnation as their floor below 1e-11 |H| (tol = 0 asks for machine accuracy, as primme's
  // default does).
  double best = INFINITY;
  int best_it = 0;
  const int patience = mixed ? 8 : 40;
  const double mixed_floor_band = 1e-4, fp64_floor_band = 1e-11;
  // The mixed form hands over to the anchored phase once the split-BF16 residual is below
  // 3e-6 |theta| or has stagnated at its ~1e-5 |H| floor (an earlier hand-over can leave the
  // solve on an excited state), and then converges the FP64-class residual to
  // max(tol, 2e-7) |theta|: the energy error is quadratic in the residual,
  // ~ (2e-7 |theta|)^2 / gap, i.e. below 1e-12 |E| for local gaps above 1e-2.
  const double mixed_handover = 3e-6, mixed_near_floor = 1e-4, mixed_rtol = tol > 2e-7 ? tol : 2e-7;
  if (start_anchored) TNX_CUDA(cudaMemcpyAsync(w.x, x_io, n * 8, cudaMemcpyDeviceToDevice, st));
  for (; !start_anchored;) {
    bool fell_in = false;
    TNX_TRY(f32 ? expand(v32, false, &fell_in) : expand(v64, false, &fell_in));
    if (fell_in) {
      if (precond) {  // preconditioned direction fell inside the basis: retry with r
        precond = 0;
        if (f32)
          ritz_kernel<<<nch, DT, 0, st>>>(v32.V, v32.AV, n, k, w.evecs, w.evals, v32.diag, 0, v32.x, v32.ax, v32.t,
                                          n, w.part, nch);
        else
          ritz_kernel<<<nch, DT, 0, st>>>(w.V, w.AV, n, k, w.evecs, w.evals, w.diag, 0, w.x, w.ax, w.t, n, w.part,
                                          nch);
        TNX_LAUNCH_CHECK();
        continue;
      }
      converged = mixed;  // the mixed form still refines below
      break;
    }
    // primme's convention (linalg.py:86): residual relative to the operator scale, here |theta|
    if (rnorm <= tol * fmax(1.0, fabs(theta)) || k >= n) {
      converged = true;
      break;
    }
    if (mixed && rnorm <= mixed_handover * fmax(1.0, fabs(theta))) {
      converged = true;
      break;
    }
    // A start vector already within ~10x of the split-BF16 residual floor (the usual case
    // once the sweeps have converged) gains nothing from the first phase, which would only
    // stagnate there: hand over at once.
    if (mixed && k == 1 && rnorm <= mixed_near_floor * fmax(1.0, fabs(theta))) {
      converged = true;
      break;
    }
    if (rnorm < 0.9 * best) {
      best = rnorm;
      best_it = iters;
    } else if (iters - best_it >= patience) {
      if (rnorm <= (mixed ? mixed_floor_band : fp64_floor_band) * hscale()) {
        converged = true;  // at the rounding floor (mixed: the anchored phase takes over)
        break;
      }
      best = rnorm;  // far above the floor: a plateau, not the floor; keep expanding
      best_it = iters;
    }
    if (iters >= max_iter) break;
    precond = 1;
    if (k == mb) {
      TNX_TRY(f32 ? restart_plus(v32) : restart_plus(v64));
      ++restarts;
    }
  }
  phase1 = iters;
  if (mixed) {
    // Anchored phase. One double-FP32 matvec gives AV[0] = H x exactly for the current Ritz
    // vector x = V[0]; the Davidson then continues with split-BF16 products for the new
    // directions. Row 0 of the projected matrix (x^T H v = (H x)^T v) is exact, and the
    // split-BF16 error E ~ 3e-5 |H| enters the Ritz value only through c^T E c and the
    // residual through E c, where c (|c| = sqrt(1 - c0^2)) is the small part of the Ritz
    // vector outside x. The residual of the anchored Ritz pair is therefore FP64-class
    // while 3e-5 |H| |c| stays below half the target; otherwise (or on stagnation) the phase
    // re-anchors at the current Ritz vector with another FP64-class matvec.
    // anchors are FP64-class products (several split-BF16 matvecs each); they are bounded by
    // max_iter / 8 (at least 6), the split-BF16 products by max_iter
    const int max_anchor = std::max(6, max_iter / 8);
    const double eps_h = 3e-5;  // bound on the split-BF16 matvec error relative to |H|
    converged = false;
    for (int anchor = 0;; ++anchor) {
      if (anchor == 0 && f32 && !start_anchored) {
        convert_kernel<float, double><<<sblocks, DT, 0, st>>>(v32.x, w.V, n);
        TNX_LAUNCH_CHECK();
      } else {
        TNX_CUDA(cudaMemcpyAsync(w.V, w.x, n * 8, cudaMemcpyDeviceToDevice, st));
      }
      // unit norm in FP64: the Rayleigh-Ritz below treats the basis as orthonormal, and a
      // Ritz vector formed in FP32 is normalised only to ~1e-8 (an offset of theta that size)
      TNX_TRY(dots(w.V, n, 1, w.V, n, w.part, nrm2, 1, nullptr, 0, st));
      scale_kernel<double><<<sblocks, DT, 0, st>>>(w.V, n, nrm2);
      TNX_LAUNCH_CHECK();
      TNX_TRY(matvec1_f64(L, W, R, w.V, w.AV, chi_l, d, chi_r, dl, dr, w.T1, w.T2, st, /*df=*/true, w.oz,
                          w.oz_bytes));
      ++anchors;
      TNX_TRY(dots(w.V, n, 1, w.AV, n, w.part, w.Hm, 1, nullptr, 0, st));
      k = 1;
      precond = 1;
      TNX_TRY(rayleigh_ritz(v64));
      double drift = 0.0;  // sum of |c| over restarts inside this anchor
      auto bound_ok = [&]() {
        const double c = sqrt(fmax(1.0 - c0 * c0, 0.0));
        return eps_h * hscale() * (drift + c) <= 0.5 * mixed_rtol * fmax(1.0, fabs(theta));
      };
      if (rnorm <= mixed_rtol * fmax(1.0, fabs(theta))) {
        converged = true;
        break;
      }
      if (anchor >= max_anchor || iters >= max_iter) break;
      if (!prepared) {  // anchored start that needs expansions: operands, then the correction again
        TNX_TRY(prepare());
        TNX_TRY(rayleigh_ritz(v64));
      }
      best = rnorm;
      best_it = iters;
      // The bound decides whether a converged residual is accepted and, within 100x of the
      // target, when to refresh the anchor (also once the Ritz vector has moved far from the
      // anchor there); while the residual is still large the phase keeps expanding (a Davidson
      // whose row 0 is exact) and re-anchors only on stagnation.
      for (;;) {
        bool fell_in = false;
        TNX_TRY(expand(v64, true, &fell_in));
        if (fell_in) break;
        if (rnorm <= mixed_rtol * fmax(1.0, fabs(theta))) {
          if (bound_ok()) converged = true;
          break;
        }
        const bool near = rnorm < 100.0 * mixed_rtol * fmax(1.0, fabs(theta));
        // close to the target but the anchor no longer vouches for the residual: refresh it
        if (near && !bound_ok()) break;
        if (near && drift + sqrt(fmax(1.0 - c0 * c0, 0.0)) > 0.3) break;
        if (rnorm < 0.9 * best) {
          best = rnorm;
          best_it = iters;
        } else if (iters - best_it >= patience) {
          if (near || rnorm <= mixed_floor_band * hscale()) break;  // at the floor: a fresh anchor
          best = rnorm;  // a plateau far above the floor: keep the subspace and expand
          best_it = iters;
        }
        if (iters >= max_iter) break;
        if (k == mb) {
          drift += sqrt(fmax(1.0 - c0 * c0, 0.0));
          TNX_TRY(restart(v64));
          ++restarts;
        }
      }
      if (converged || iters >= max_iter) break;
    }
  }
  // the Ritz vector of the last Rayleigh-Ritz step, unit norm
  TNX_CUDA(cudaMemcpyAsync(x_io, w.x, n * 8, cudaMemcpyDeviceToDevice, st));
  if (eval_out) *eval_out = theta;
  if (resid_out) *resid_out = rnorm;
  if (iters_out) *iters_out = iters;
  g_dav_stats = {phase1, iters - phase1, anchors, restarts};
  if (!converged) {
    set_error("tnx_davidson1: %d matvecs, residual %.3e > tol %.3e", iters, rnorm,
              mixed ? mixed_rtol * fmax(1.0, fabs(theta)) : tol);
    return TNX_ERR_NOT_CONVERGED;
  }
  return TNX_OK;
}

// ---- generalised problem A x = lambda B x (B symmetric positive definite) ------------------
// Davidson with a B-orthonormal basis: V^T B V = I, so the projected problem V^T A V s = theta s
// is standard. Each expansion B-orthogonalises the correction t against V (two classical
// passes; the B-images BV follow the same combinations, so one B product per expansion), applies
// A once, and forms x = V s, the residual A x - theta B x and the correction
// (diag A - theta diag B)^-1 r. Converged when ||A x - theta B x|| <= tol max(1, |theta|), or
// when the residual has stagnated (no 10 % gain in 40 expansions) below 1e-6 max(1, |theta|):
// shift-invert pencils converge slowly near their floor, and there the Ritz value is already
// accurate to ~|r|^2 / gap.
struct GDavWs {
  double *V, *AV, *BV, *x, *ax, *bx, *t, *da, *db, *Hm, *evals, *evecs, *part, *scal, *T1, *T2;
};

size_t gdav_layout(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, int64_t dl2, int64_t dr2, int mb,
                   void* base, GDavWs* w) {
  const int64_t n = chi_l * d * chi_r;
  const int64_t ne1 = matvec1_scratch_elems(chi_l, d, chi_r, dl, dr);
  const int64_t ne2 = matvec1_scratch_elems(chi_l, d, chi_r, dl2, dr2);
  const int64_t ne = ne1 > ne2 ? ne1 : ne2;
  const int nch = nchunk_for(n);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align_up(bytes);
    return o;
  };
  size_t oV = take(size_t(mb) * n * 8), oAV = take(size_t(mb) * n * 8), oBV = take(size_t(mb) * n * 8),
         ox = take(n * 8), oax = take(n * 8), obx = take(n * 8), ot = take(n * 8), oda = take(n * 8),
         odb = take(n * 8), oH = take(size_t(mb) * mb * 8), oev = take(size_t(mb) * 8),
         oevec = take(size_t(mb) * mb * 8), opart = take(size_t(mb + 1) * nch * 8), oscal = take(size_t(4 * MAXB) * 8),
         oT1 = take(ne * 8), oT2 = take(ne * 8);
  if (w && base) {
    char* b = static_cast<char*>(base);
    w->V = reinterpret_cast<double*>(b + oV);
    w->AV = reinterpret_cast<double*>(b + oAV);
    w->BV = reinterpret_cast<double*>(b + oBV);
    w->x = reinterpret_cast<double*>(b + ox);
    w->ax = reinterpret_cast<double*>(b + oax);
    w->bx = reinterpret_cast<double*>(b + obx);
    w->t = reinterpret_cast<double*>(b + ot);
    w->da = reinterpret_cast<double*>(b + oda);
    w->db = reinterpret_cast<double*>(b + odb);
    w->Hm = reinterpret_cast<double*>(b + oH);
    w->evals = reinterpret_cast<double*>(b + oev);
    w->evecs = reinterpret_cast<double*>(b + oevec);
    w->part = reinterpret_cast<double*>(b + opart);
    w->scal = reinterpret_cast<double*>(b + oscal);
    w->T1 = reinterpret_cast<double*>(b + oT1);
    w->T2 = reinterpret_cast<double*>(b + oT2);
  }
  return off;
}

int gdavidson1(const double* L, const double* W, const double* R, const double* L2, const double* W2,
               const double* R2, double* x_io, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
               int64_t dl2, int64_t dr2, double tol, int max_iter, int mb, int precision, double* eval_out,
               double* resid_out, int* iters_out, void* ws, size_t ws_bytes, cudaStream_t st) {
  GDavWs w;
  const size_t need = gdav_layout(chi_l, d, chi_r, dl, dr, dl2, dr2, mb, ws, &w);
  if (ws_bytes < need || !ws) {
    set_error("tnx_gdavidson1: workspace %zu bytes < required %zu", ws_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  const int64_t n = chi_l * d * chi_r;
  if (mb > n) mb = int(n < 2 ? 2 : n);
  const int nch = nchunk_for(n);
  const unsigned sblocks = (unsigned)((n + DT - 1) / DT < 152 * 8 ? (n + DT - 1) / DT : 152 * 8);
  const bool df = precision != TNX_FP64;
  auto amul = [&](const double* in, double* out) {
    return matvec1_f64(L, W, R, in, out, chi_l, d, chi_r, dl, dr, w.T1, w.T2, st, df);
  };
  auto bmul = [&](const double* in, double* out) {
    return matvec1_f64(L2, W2, R2, in, out, chi_l, d, chi_r, dl2, dr2, w.T1, w.T2, st, df);
  };
  double* h = w.scal;
  double* nrm2 = w.scal + MAXB;
  double* rn2 = w.scal + MAXB + 2;
  double host[2];
  TNX_TRY(tnx_diag1(L, W, R, w.da, chi_l, d, chi_r, dl, dr, st));
  TNX_TRY(tnx_diag1(L2, W2, R2, w.db, chi_l, d, chi_r, dl2, dr2, st));
  TNX_CUDA(cudaMemcpyAsync(w.t, x_io, n * 8, cudaMemcpyDeviceToDevice, st));
  int k = 0, iters = 0, best_it = 0;
  double theta = 0.0, rnorm = INFINITY, best = INFINITY;
  bool converged = false;
  for (;;) {
    double* vk = w.V + int64_t(k) * n;
    double* bvk = w.BV + int64_t(k) * n;
    TNX_CUDA(cudaMemcpyAsync(vk, w.t, n * 8, cudaMemcpyDeviceToDevice, st));
    // pass 1: against V in the B inner product, h_j = (B V_j) . t
    if (k > 0) {
      TNX_TRY(dots<double>(w.BV, n, k, vk, n, w.part, h, 1, nullptr, 0, st));
      update_kernel<double><<<nch, DT, 0, st>>>(w.V, n, k, h, vk, n, w.part, nch, nullptr);
      TNX_LAUNCH_CHECK();
    }
    TNX_TRY(bmul(vk, bvk));
    ++iters;
    // pass 2: h_j = V_j . (B t), applied to t and (linearly) to B t
    if (k > 0) {
      TNX_TRY(dots<double>(w.V, n, k, bvk, n, w.part, h, 1, nullptr, 0, st));
      update_kernel<double><<<nch, DT, 0, st>>>(w.V, n, k, h, vk, n, w.part, nch, nullptr);
      TNX_LAUNCH_CHECK();
      axpy_basis_kernel<<<sblocks, DT, 0, st>>>(w.BV, n, k, h, bvk, n);
      TNX_LAUNCH_CHECK();
    }
    TNX_TRY(dots<double>(vk, n, 1, bvk, n, w.part, nrm2, 1, nullptr, 0, st));
    TNX_CUDA(cudaMemcpyAsync(host, nrm2, 8, cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaStreamSynchronize(st));
    if (!(host[0] > 0.0) || !std::isfinite(host[0])) {
      if (k == 0) {
        set_error("tnx_gdavidson1: start vector has zero or non-finite B-norm");
        return TNX_ERR_INVALID_ARG;
      }
      break;  // the correction fell into the basis
    }
    scale2_kernel<<<sblocks, DT, 0, st>>>(vk, bvk, n, nrm2);
    TNX_LAUNCH_CHECK();
    double* avk = w.AV + int64_t(k) * n;
    TNX_TRY(amul(vk, avk));
    TNX_TRY(dots<double>(w.V, n, k + 1, avk, n, w.part, w.Hm + k, mb, w.Hm + int64_t(k) * mb, 1, st));
    ++k;
    TNX_TRY(rr_lowest_f64(w.Hm, k, mb, w.evals, w.evecs, st));
    gritz_kernel<<<nch, DT, 0, st>>>(w.V, w.AV, w.BV, n, k, w.evecs, w.evals, w.da, w.db, w.x, w.ax, w.bx, w.t, n,
                                     w.part, nch);
    TNX_LAUNCH_CHECK();
    reduce_kernel<<<1, DT, 0, st>>>(w.part, nch, rn2, 1, nullptr, 0);
    TNX_LAUNCH_CHECK();
    TNX_CUDA(cudaMemcpyAsync(host, w.evals, 8, cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaMemcpyAsync(host + 1, rn2, 8, cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaStreamSynchronize(st));
    theta = host[0];
    rnorm = sqrt(fmax(host[1], 0.0));
    if (!std::isfinite(theta) || !std::isfinite(rnorm)) {
      set_error("tnx_gdavidson1: non-finite Ritz value or residual");
      return TNX_ERR_INVALID_ARG;
    }
    const double scale = fmax(1.0, fabs(theta));
    if (rnorm <= tol * scale || k >= n) {
      converged = true;
      break;
    }
    if (rnorm < 0.9 * best) {
      best = rnorm;
      best_it = iters;
    } else if (iters - best_it >= 40 && rnorm <= 1e-6 * scale) {
      converged = true;  // stagnated near the floor
      break;
    }
    if (iters >= max_iter) break;
    if (k == mb) {  // restart to the Ritz vector (B-unit by construction)
      TNX_CUDA(cudaMemcpyAsync(w.V, w.x, n * 8, cudaMemcpyDeviceToDevice, st));
      TNX_CUDA(cudaMemcpyAsync(w.AV, w.ax, n * 8, cudaMemcpyDeviceToDevice, st));
      TNX_CUDA(cudaMemcpyAsync(w.BV, w.bx, n * 8, cudaMemcpyDeviceToDevice, st));
      restart_kernel<<<1, 1, 0, st>>>(w.Hm, w.evals, w.evecs);
      TNX_LAUNCH_CHECK();
      k = 1;
    }
  }
  TNX_CUDA(cudaMemcpyAsync(x_io, w.x, n * 8, cudaMemcpyDeviceToDevice, st));
  if (eval_out) *eval_out = theta;
  if (resid_out) *resid_out = rnorm;
  if (iters_out) *iters_out = iters;
  if (!converged) {
    set_error("tnx_gdavidson1: %d products, residual %.3e > tol %.3e", iters, rnorm, tol);
    return TNX_ERR_NOT_CONVERGED;
  }
  return TNX_OK;
}

}  // namespace tnx

using namespace tnx;

extern "C" {

size_t tnx_davidson1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                     int max_basis, int precision) {
  if (max_basis > MAXB) max_basis = MAXB;
  return dav_layout(chi_l, d, chi_r, dl, dr, max_basis, precision, nullptr, 0, nullptr);
}

int tnx_davidson1_stats(int* out) {
  TNX_CHECK_ARG(out, "null pointer");
  out[0] = g_dav_stats.phase1;
  out[1] = g_dav_stats.anchored;
  out[2] = g_dav_stats.anchors;
  out[3] = g_dav_stats.restarts;
  return TNX_OK;
}

size_t tnx_gdavidson1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                      int64_t dl2, int64_t dr2, int max_basis) {
  if (max_basis > MAXB) max_basis = MAXB;
  return gdav_layout(chi_l, d, chi_r, dl, dr, dl2, dr2, max_basis, nullptr, nullptr);
}

int tnx_gdavidson1(const double* L, const double* W, const double* R, const double* L2, const double* W2,
                   const double* R2, double* x, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                   int64_t dl2, int64_t dr2, double tol, int max_iter, int max_basis, int precision,
                   double* eval_out, double* resid_out, int* iters_out, void* workspace, size_t workspace_bytes,
                   void* stream) {
  TNX_CHECK_ARG(L && W && R && L2 && W2 && R2 && x, "null pointer");
  TNX_CHECK_ARG(chi_l > 0 && d > 0 && chi_r > 0 && dl > 0 && dr > 0 && dl2 > 0 && dr2 > 0, "non-positive dimension");
  TNX_CHECK_ARG(max_basis >= 2 && max_basis <= MAXB, "max_basis must be in [2, %d] (got %d)", MAXB, max_basis);
  TNX_CHECK_ARG(max_iter >= 1 && tol >= 0.0, "max_iter must be >= 1 and tol >= 0");
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  TNX_CHECK_SHAPE(dl * d <= 64 && dr * d <= 64 && dl2 * d <= 64 && dr2 * d <= 64, "MPO bond too large");
  return gdavidson1(L, W, R, L2, W2, R2, x, chi_l, d, chi_r, dl, dr, dl2, dr2, tol, max_iter, max_basis, precision,
                    eval_out, resid_out, iters_out, workspace, workspace_bytes, as_stream(stream));
}

int tnx_davidson1(const double* L, const double* W, const double* R, double* x, int64_t chi_l, int64_t d,
                  int64_t chi_r, int64_t dl, int64_t dr, double tol, int max_iter, int max_basis,
                  int precision, double* eval_out, double* resid_out, int* iters_out, void* workspace,
                  size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(L && W && R && x, "null pointer");
  TNX_CHECK_ARG(chi_l > 0 && d > 0 && chi_r > 0 && dl > 0 && dr > 0, "non-positive dimension");
  TNX_CHECK_ARG(max_basis >= 2 && max_basis <= MAXB, "max_basis must be in [2, %d] (got %d)", MAXB,
                max_basis);
  TNX_CHECK_ARG(max_iter >= 1, "max_iter must be >= 1");
  TNX_CHECK_ARG(tol >= 0.0, "tol must be >= 0");
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  TNX_CHECK_SHAPE(dl * d <= 64 && dr * d <= 64, "MPO bond too large");
  return davidson1(L, W, R, x, chi_l, d, chi_r, dl, dr, tol, max_iter, max_basis, precision, eval_out,
                   resid_out, iters_out, workspace, workspace_bytes, as_stream(stream));
}

int tnx_davidson1_ex(const double* L, const double* W, const double* R, double* x, int64_t chi_l, int64_t d,
                     int64_t chi_r, int64_t dl, int64_t dr, double tol, int max_iter, int max_basis, int precision,
                     int flags, double* eval_out, double* resid_out, int* iters_out, void* workspace,
                     size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(L && W && R && x, "null pointer");
  TNX_CHECK_ARG(chi_l > 0 && d > 0 && chi_r > 0 && dl > 0 && dr > 0, "non-positive dimension");
  TNX_CHECK_ARG(max_basis >= 2 && max_basis <= MAXB, "max_basis must be in [2, %d] (got %d)", MAXB,
                max_basis);
  TNX_CHECK_ARG(max_iter >= 1, "max_iter must be >= 1");
  TNX_CHECK_ARG(tol >= 0.0, "tol must be >= 0");
  TNX_CHECK_ARG(precision >= TNX_FP64 && precision <= TNX_DF64, "unknown precision %d", precision);
  TNX_CHECK_ARG((flags & ~TNX_DAV_START_ANCHORED) == 0, "unknown flags 0x%x", flags);
  TNX_CHECK_SHAPE(dl * d <= 64 && dr * d <= 64, "MPO bond too large");
  return davidson1(L, W, R, x, chi_l, d, chi_r, dl, dr, tol, max_iter, max_basis, precision, eval_out,
                   resid_out, iters_out, workspace, workspace_bytes, as_stream(stream), flags);
}

}  // extern "C"
