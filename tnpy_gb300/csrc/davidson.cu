// Lowest eigenpair of the one-site effective Hamiltonian: a Davidson eigensolver that
// stays on the device, replacing linalg.eigshmv -> primme.eigsh(k=1, which='SA')
// (tnpy/linalg.py:64-87) called from FiniteDMRG.one_site_solver (tnpy/finite_dmrg.py:97-111).
//
// Basis V (orthonormal, FP64) and AV = H V live in the caller's workspace; each expansion
//   1. orthogonalises the new direction against V twice (classical Gram-Schmidt, FP64),
//   2. applies H (FP64 or split-BF16 tensor-core matvec),
//   3. extends the projected matrix V^T H V (FP64 dots),
//   4. solves it with the one-CTA Jacobi eigensolver (FP64 Rayleigh-Ritz),
//   5. forms the Ritz vector, the residual r = H x - theta x and its norm, and the next
//      direction t = r / (diag(H) - theta) (diagonal preconditioner).
// The host loop reads two scalars per expansion to decide convergence. With the
// split-BF16 matvec the final energy and residual are recomputed with one FP64 matvec
// (defect correction), so the reported Rayleigh quotient is an FP64 one.
#include <cuda_runtime.h>

#include <cmath>

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

// part[j*nchunk + chunk] = sum over the chunk of V[j][i] * w[i], j < k
__global__ void __launch_bounds__(DT) dots_kernel(const double* __restrict__ V, int64_t ldv,
                                                 const double* __restrict__ w, int64_t n,
                                                 double* __restrict__ part, int nchunk) {
  __shared__ double sh[DT / 32];
  const int j = blockIdx.y, chunk = blockIdx.x;
  const double* v = V + int64_t(j) * ldv;
  double acc = 0.0;
  for (int64_t i = int64_t(chunk) * DT + threadIdx.x; i < n; i += int64_t(nchunk) * DT)
    acc = fma(v[i], w[i], acc);
  acc = block_sum(acc, sh);
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

// w -= sum_{j<k} h[j] V[j]; partial ||w||^2
__global__ void __launch_bounds__(DT) update_kernel(const double* __restrict__ V, int64_t ldv, int k,
                                                   const double* __restrict__ h, double* __restrict__ w,
                                                   int64_t n, double* __restrict__ part, int nchunk) {
  __shared__ double sh[DT / 32];
  __shared__ double hs[MAXB];
  if (threadIdx.x < k) hs[threadIdx.x] = h[threadIdx.x];
  __syncthreads();
  double nrm = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(nchunk) * DT) {
    double acc = w[i];
    for (int j = 0; j < k; ++j) acc = fma(-hs[j], V[int64_t(j) * ldv + i], acc);
    w[i] = acc;
    nrm = fma(acc, acc, nrm);
  }
  nrm = block_sum(nrm, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = nrm;
}

// w *= 1/sqrt(nrm2[0])
__global__ void scale_kernel(double* __restrict__ w, int64_t n, const double* __restrict__ nrm2) {
  const double s = 1.0 / sqrt(nrm2[0]);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    w[i] *= s;
}

// x = V s, ax = AV s, r = ax - theta x, t = r / (diag - theta) (or r), partial ||r||^2
__global__ void __launch_bounds__(DT) ritz_kernel(const double* __restrict__ V, const double* __restrict__ AV,
                                                 int64_t ldv, int k, const double* __restrict__ s,
                                                 const double* __restrict__ theta_p,
                                                 const double* __restrict__ diag, int precond,
                                                 double* __restrict__ x, double* __restrict__ ax,
                                                 double* __restrict__ t, int64_t n,
                                                 double* __restrict__ part, int nchunk) {
  __shared__ double sh[DT / 32];
  __shared__ double ss[MAXB];
  if (threadIdx.x < k) ss[threadIdx.x] = s[threadIdx.x];
  __syncthreads();
  const double theta = theta_p[0];
  double nrm = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(nchunk) * DT) {
    double xv = 0.0, av = 0.0;
    for (int j = 0; j < k; ++j) {
      xv = fma(ss[j], V[int64_t(j) * ldv + i], xv);
      av = fma(ss[j], AV[int64_t(j) * ldv + i], av);
    }
    const double r = av - theta * xv;
    x[i] = xv;
    ax[i] = av;
    double tv = r;
    if (precond) {
      double den = diag[i] - theta;
      const double floor = 1e-2;
      if (fabs(den) < floor) den = den >= 0.0 ? floor : -floor;
      tv = r / den;
    }
    t[i] = tv;
    nrm = fma(r, r, nrm);
  }
  nrm = block_sum(nrm, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = nrm;
}

// r = ax - theta x with theta = (x . ax) given in th[0]; partial ||r||^2
__global__ void __launch_bounds__(DT) resid_kernel(const double* __restrict__ x, const double* __restrict__ ax,
                                                  const double* __restrict__ th, int64_t n,
                                                  double* __restrict__ part, int nchunk) {
  __shared__ double sh[DT / 32];
  const double theta = th[0];
  double nrm = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(nchunk) * DT) {
    const double r = ax[i] - theta * x[i];
    nrm = fma(r, r, nrm);
  }
  nrm = block_sum(nrm, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = nrm;
}

// t = ax - theta x (theta = th[0]); partial ||t||^2
__global__ void __launch_bounds__(DT) resid_write_kernel(const double* __restrict__ x, const double* __restrict__ ax,
                                                        const double* __restrict__ th, double* __restrict__ t,
                                                        int64_t n, double* __restrict__ part, int nchunk) {
  __shared__ double sh[DT / 32];
  const double theta = th[0];
  double nrm = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * DT + threadIdx.x; i < n; i += int64_t(nchunk) * DT) {
    const double r = ax[i] - theta * x[i];
    t[i] = r;
    nrm = fma(r, r, nrm);
  }
  nrm = block_sum(nrm, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = nrm;
}

// out = in / (diag - theta), the diagonal preconditioner with its denominator kept >= 1e-2
__global__ void precond_kernel(const double* __restrict__ in, const double* __restrict__ diag, double theta,
                               double* __restrict__ out, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    double den = diag[i] - theta;
    if (fabs(den) < 1e-2) den = den >= 0.0 ? 1e-2 : -1e-2;
    out[i] = in[i] / den;
  }
}

// y = a * x + b * y with host scalars
__global__ void axpby_kernel(double a, const double* __restrict__ x, double b, double* __restrict__ y, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    y[i] = fma(a, x[i], b * y[i]);
}

// out = sum_{j<k} c[j] V[j]  (host coefficients passed by value in a small struct)
struct Coef64 {
  double c[64];
};
__global__ void combine_kernel(const double* __restrict__ V, int64_t ldv, int k, Coef64 c, double* __restrict__ out,
                               int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < k; ++j) acc = fma(c.c[j], V[int64_t(j) * ldv + i], acc);
    out[i] = acc;
  }
}

// after a restart to the single Ritz vector x: H = [[theta]], Ritz coefficients s = [1]
__global__ void restart_kernel(double* Hm, const double* evals, double* evecs) {
  Hm[0] = evals[0];
  evecs[0] = 1.0;
}

inline int nchunk_for(int64_t n) {
  int64_t c = (n + DT * 4 - 1) / (DT * 4);
  if (c > 2 * 152) c = 2 * 152;
  return int(c < 1 ? 1 : c);
}

struct DavWs {
  double *V, *AV, *x, *ax, *t, *diag, *Hm, *Hwork, *evals, *evecs, *jwork, *part, *scal;
  void* mv;
  size_t mv_bytes;
  double *T1, *T2;  // FP64 matvec scratch (also used by the defect correction)
};

size_t dav_layout(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, int mb, int precision,
                  void* base, size_t size, DavWs* w) {
  const int64_t n = chi_l * d * chi_r;
  const int64_t ne = matvec1_scratch_elems(chi_l, d, chi_r, dl, dr);
  const size_t mv_bytes = (precision == TNX_BF16X3 && mixed_supported(chi_l, d, chi_r, dl, dr))
                              ? matvec1_bf16x3_scratch_bytes(chi_l, d, chi_r, dl, dr)
                              : 0;
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
         oscal = take(size_t(4 * MAXB) * 8), oT1 = take(ne * 8), oT2 = take(ne * 8), omv = take(mv_bytes);
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
  }
  return off;
}

// h[0..k) = V[0..k) . w
int dots(const double* V, int64_t ldv, int k, const double* w, int64_t n, double* part, double* out,
         int out_stride, double* out2, int out2_stride, cudaStream_t st) {
  const int nch = nchunk_for(n);
  dots_kernel<<<dim3(nch, k), DT, 0, st>>>(V, ldv, w, n, part, nch);
  TNX_LAUNCH_CHECK();
  reduce_kernel<<<k, DT, 0, st>>>(part, nch, out, out_stride, out2, out2_stride);
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

}  // namespace

// Davidson driver. All pointers device; eval/resid/iters host.
int davidson1(const double* L, const double* W, const double* R, double* x_io, int64_t chi_l, int64_t d,
              int64_t chi_r, int64_t dl, int64_t dr, double tol, int max_iter, int mb, int precision,
              double* eval_out, double* resid_out, int* iters_out, void* ws, size_t ws_bytes,
              cudaStream_t st) {
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
  int* dflag = nullptr;
  if (mixed) {
    TNX_TRY(mixed_prepare(L, R, chi_l, d, chi_r, dl, dr, w.mv, st));
    mixed_flag(w.mv, chi_l, d, chi_r, dl, dr, &dflag);
  }
  auto matvec = [&](const double* in, double* out) -> int {
    if (mixed) return mixed_apply(W, in, out, chi_l, d, chi_r, dl, dr, w.mv, st);
    return matvec1_f64(L, W, R, in, out, chi_l, d, chi_r, dl, dr, w.T1, w.T2, st, precision == TNX_DF64);
  };
  int hflag = 0;
  double* h = w.scal;               // [MAXB]
  double* nrm2 = w.scal + MAXB;     // [2]: |t|^2 before, after orthogonalisation
  double* rn2 = w.scal + MAXB + 2;  // ||r||^2
  double host[4];

  TNX_CUDA(cudaMemcpyAsync(w.t, x_io, n * 8, cudaMemcpyDeviceToDevice, st));
  if (int e = tnx_diag1(L, W, R, w.diag, chi_l, d, chi_r, dl, dr, st); e != TNX_OK) return e;

  int k = 0, iters = 0, precond = 1;
  double theta = 0.0, rnorm = INFINITY;
  bool converged = false;
  // Stagnation: the split-BF16 operand is not exactly symmetric, so the residual of the
  // mixed operator stops falling at ~1e-5 |H| (its rounding floor); the solve ends when the
  // residual has not improved by 10% within `patience` matvecs (the FP64 defect correction
  // below then gives the energy). The FP64 form uses a longer patience as a safeguard.
  double best = INFINITY;
  int best_it = 0;
  const int patience = mixed ? 8 : 40;
  const int max_refine = 6;  // defect-correction steps of the mixed form
  // The mixed form hands over to the FP64-class defect correction once the split-BF16 residual
  // is below 3e-6 |theta| or has stagnated at its ~1e-5 |H| floor (an earlier hand-over can leave
  // the Davidson on an excited state that the correction then converges to), and refines the
  // FP64-class residual
  // to max(tol, 2e-7) |theta|: the energy error is quadratic in the residual,
  // ~ (2e-7 |theta|)^2 / gap, i.e. below 1e-12 |E| for local gaps above 1e-2.
  const double mixed_handover = 3e-6, mixed_rtol = tol > 2e-7 ? tol : 2e-7;
  for (;;) {
    // -- new direction t -> V[k], orthogonalised against V[0..k) twice --
    double* vk = w.V + int64_t(k) * n;
    TNX_CUDA(cudaMemcpyAsync(vk, w.t, n * 8, cudaMemcpyDeviceToDevice, st));
    TNX_TRY(dots(vk, n, 1, vk, n, w.part, nrm2, 1, nullptr, 0, st));
    for (int pass = 0; pass < 2 && k > 0; ++pass) {
      TNX_TRY(dots(w.V, n, k, vk, n, w.part, h, 1, nullptr, 0, st));
      update_kernel<<<nch, DT, 0, st>>>(w.V, n, k, h, vk, n, w.part, nch);
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
      if (precond) {  // preconditioned direction fell inside the basis: retry with r
        precond = 0;
        // recompute t = r from the current Ritz pair
        ritz_kernel<<<nch, DT, 0, st>>>(w.V, w.AV, n, k, w.evecs, w.evals, w.diag, 0, w.x, w.ax, w.t, n,
                                        w.part, nch);
        TNX_LAUNCH_CHECK();
        continue;
      }
      break;  // stagnation: keep the current Ritz pair
    }
    scale_kernel<<<sblocks, DT, 0, st>>>(vk, n, nrm2 + 1);
    TNX_LAUNCH_CHECK();
    // -- AV[k] = H V[k]; projected matrix column k --
    double* avk = w.AV + int64_t(k) * n;
    TNX_TRY(matvec(vk, avk));
    ++iters;
    TNX_TRY(dots(w.V, n, k + 1, avk, n, w.part, w.Hm + k, mb, w.Hm + int64_t(k) * mb, 1, st));
    ++k;
    // -- Rayleigh-Ritz (FP64 Jacobi on the k x k projected matrix, leading dim mb) --
    TNX_TRY(rr_lowest_f64(w.Hm, k, mb, w.evals, w.evecs, st));
    ritz_kernel<<<nch, DT, 0, st>>>(w.V, w.AV, n, k, w.evecs, w.evals, w.diag, precond, w.x, w.ax, w.t, n,
                                    w.part, nch);
    TNX_LAUNCH_CHECK();
    reduce_kernel<<<1, DT, 0, st>>>(w.part, nch, rn2, 1, nullptr, 0);
    TNX_LAUNCH_CHECK();
    TNX_CUDA(cudaMemcpyAsync(host, w.evals, 8, cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaMemcpyAsync(host + 1, rn2, 8, cudaMemcpyDeviceToHost, st));
    if (dflag) TNX_CUDA(cudaMemcpyAsync(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost, st));
    TNX_CUDA(cudaStreamSynchronize(st));
    if (hflag) {
      set_error("tnx_davidson1: a bounded wait in the tensor-core matvec expired");
      return TNX_ERR_TIMEOUT;
    }
    theta = host[0];
    rnorm = sqrt(fmax(host[1], 0.0));
    if (!std::isfinite(theta) || !std::isfinite(rnorm)) {
      set_error("tnx_davidson1: non-finite Ritz value or residual");
      return TNX_ERR_INVALID_ARG;
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
    if (rnorm < 0.9 * best) {
      best = rnorm;
      best_it = iters;
    } else if (iters - best_it >= patience) {
      converged = mixed;  // at the mixed rounding floor: done; FP64: report non-convergence
      break;
    }
    if (iters >= max_iter) break;
    precond = 1;
    if (k == mb) {  // thick restart with the current Ritz vector
      TNX_CUDA(cudaMemcpyAsync(w.V, w.x, n * 8, cudaMemcpyDeviceToDevice, st));
      TNX_CUDA(cudaMemcpyAsync(w.AV, w.ax, n * 8, cudaMemcpyDeviceToDevice, st));
      restart_kernel<<<1, 1, 0, st>>>(w.Hm, w.evals, w.evecs);
      TNX_LAUNCH_CHECK();
      k = 1;
    }
  }
  // -- output: unit Ritz vector; FP64-class Rayleigh quotient and residual for the mixed form --
  if (mixed) {
    // Defect correction. The split-BF16 operand H~ only converges the Davidson to its own
    // eigenvector; the FP64-class residual r = H x - theta x (double-FP32 matvec) then drives
    // Jacobi-Davidson correction steps: solve (I - x x^T)(H~ - theta)(I - x x^T) delta = -r
    // approximately with GMRES on the tensor-core matvec, x <- (x + delta) / ||x + delta||.
    // Each step contracts the error by about (error of H~) * ||H|| / gap.
    double* V = w.V;    // GMRES basis (the Davidson basis is no longer needed)
    double* Wv = w.AV;  // operator output scratch
    const int mg = mb - 1;
    for (int ref = 0;; ++ref) {
      TNX_TRY(matvec1_f64(L, W, R, w.x, w.ax, chi_l, d, chi_r, dl, dr, w.T1, w.T2, st, /*df=*/true));
      TNX_TRY(dots(w.x, n, 1, w.ax, n, w.part, h, 1, nullptr, 0, st));
      resid_write_kernel<<<nch, DT, 0, st>>>(w.x, w.ax, h, w.t, n, w.part, nch);
      TNX_LAUNCH_CHECK();
      reduce_kernel<<<1, DT, 0, st>>>(w.part, nch, rn2, 1, nullptr, 0);
      TNX_LAUNCH_CHECK();
      TNX_CUDA(cudaMemcpyAsync(host, h, 8, cudaMemcpyDeviceToHost, st));
      TNX_CUDA(cudaMemcpyAsync(host + 1, rn2, 8, cudaMemcpyDeviceToHost, st));
      TNX_CUDA(cudaStreamSynchronize(st));
      theta = host[0];
      rnorm = sqrt(fmax(host[1], 0.0));
      if (rnorm <= mixed_rtol * fmax(1.0, fabs(theta)) || ref >= max_refine || iters >= max_iter) break;
      // right-preconditioned GMRES(mg) on P (H~ - theta) P M^-1, M = diag(H) - theta, x0 = 0,
      // b = -r; the correction is delta = P M^-1 V y
      const double beta = rnorm;
      axpby_kernel<<<sblocks, DT, 0, st>>>(-1.0 / beta, w.t, 0.0, V, n);
      TNX_LAUNCH_CHECK();
      double Hh[65][64] = {};
      double cs[64], sn[64], g[65] = {};
      g[0] = beta;
      int j = 0;
      for (; j < mg && iters < max_iter; ++j) {
        double* vj = V + int64_t(j) * n;
        double* wj = Wv + int64_t(j) * n;
        // t = P M^-1 v_j
        precond_kernel<<<sblocks, DT, 0, st>>>(vj, w.diag, theta, w.t, n);
        TNX_LAUNCH_CHECK();
        TNX_TRY(dots(w.x, n, 1, w.t, n, w.part, h, 1, nullptr, 0, st));
        update_kernel<<<nch, DT, 0, st>>>(w.x, n, 1, h, w.t, n, w.part, nch);
        TNX_LAUNCH_CHECK();
        TNX_TRY(mixed_apply(W, w.t, wj, chi_l, d, chi_r, dl, dr, w.mv, st));
        ++iters;
        axpby_kernel<<<sblocks, DT, 0, st>>>(-theta, w.t, 1.0, wj, n);
        TNX_LAUNCH_CHECK();
        // project out x
        TNX_TRY(dots(w.x, n, 1, wj, n, w.part, h, 1, nullptr, 0, st));
        update_kernel<<<nch, DT, 0, st>>>(w.x, n, 1, h, wj, n, w.part, nch);
        TNX_LAUNCH_CHECK();
        // Arnoldi: two classical Gram-Schmidt passes against V[0..j]
        double hcol[65] = {};
        for (int pass = 0; pass < 2; ++pass) {
          TNX_TRY(dots(V, n, j + 1, wj, n, w.part, h, 1, nullptr, 0, st));
          update_kernel<<<nch, DT, 0, st>>>(V, n, j + 1, h, wj, n, w.part, nch);
          TNX_LAUNCH_CHECK();
          reduce_kernel<<<1, DT, 0, st>>>(w.part, nch, nrm2, 1, nullptr, 0);
          TNX_LAUNCH_CHECK();
          double hh[64];
          TNX_CUDA(cudaMemcpyAsync(hh, h, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, st));
          TNX_CUDA(cudaMemcpyAsync(host, nrm2, 8, cudaMemcpyDeviceToHost, st));
          TNX_CUDA(cudaStreamSynchronize(st));
          for (int i = 0; i <= j; ++i) hcol[i] += hh[i];
        }
        const double hn = sqrt(fmax(host[0], 0.0));
        hcol[j + 1] = hn;
        if (hn > 0.0) {
          double* vn = V + int64_t(j + 1) * n;
          axpby_kernel<<<sblocks, DT, 0, st>>>(1.0 / hn, wj, 0.0, vn, n);
          TNX_LAUNCH_CHECK();
        }
        // apply previous Givens rotations, then a new one zeroing hcol[j+1]
        for (int i = 0; i < j; ++i) {
          const double a = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
          hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
          hcol[i] = a;
        }
        const double den = sqrt(hcol[j] * hcol[j] + hcol[j + 1] * hcol[j + 1]);
        cs[j] = den > 0.0 ? hcol[j] / den : 1.0;
        sn[j] = den > 0.0 ? hcol[j + 1] / den : 0.0;
        hcol[j] = den;
        hcol[j + 1] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        for (int i = 0; i <= j; ++i) Hh[i][j] = hcol[i];
        if (fabs(g[j + 1]) <= 1e-2 * beta || hn == 0.0) {
          ++j;
          break;
        }
      }
      // y = R^-1 g (upper triangular), delta = V y, x <- (x + delta) / ||x + delta||
      Coef64 y = {};
      for (int i = j - 1; i >= 0; --i) {
        double t = g[i];
        for (int q = i + 1; q < j; ++q) t -= Hh[i][q] * y.c[q];
        y.c[i] = Hh[i][i] != 0.0 ? t / Hh[i][i] : 0.0;
      }
      combine_kernel<<<sblocks, DT, 0, st>>>(V, n, j, y, w.ax, n);
      TNX_LAUNCH_CHECK();
      precond_kernel<<<sblocks, DT, 0, st>>>(w.ax, w.diag, theta, w.t, n);
      TNX_LAUNCH_CHECK();
      TNX_TRY(dots(w.x, n, 1, w.t, n, w.part, h, 1, nullptr, 0, st));
      update_kernel<<<nch, DT, 0, st>>>(w.x, n, 1, h, w.t, n, w.part, nch);
      TNX_LAUNCH_CHECK();
      axpby_kernel<<<sblocks, DT, 0, st>>>(1.0, w.t, 1.0, w.x, n);
      TNX_LAUNCH_CHECK();
      TNX_TRY(dots(w.x, n, 1, w.x, n, w.part, nrm2, 1, nullptr, 0, st));
      scale_kernel<<<sblocks, DT, 0, st>>>(w.x, n, nrm2);
      TNX_LAUNCH_CHECK();
    }
    converged = rnorm <= mixed_rtol * fmax(1.0, fabs(theta));
  }
  TNX_CUDA(cudaMemcpyAsync(x_io, w.x, n * 8, cudaMemcpyDeviceToDevice, st));
  if (eval_out) *eval_out = theta;
  if (resid_out) *resid_out = rnorm;
  if (iters_out) *iters_out = iters;
  if (!converged) {
    set_error("tnx_davidson1: %d matvecs, residual %.3e > tol %.3e", iters, rnorm, tol);
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

}  // extern "C"
