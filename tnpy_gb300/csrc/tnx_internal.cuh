// Internal helpers shared by the tnx translation units.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <functional>

#include "../../include/tnx.h"

namespace tnx {

// Thread-local error message of the last failing entry point.
void set_error(const char* fmt, ...);

#define TNX_CHECK_ARG(cond, ...)          \
  do {                                    \
    if (!(cond)) {                        \
      ::tnx::set_error(__VA_ARGS__);      \
      return TNX_ERR_INVALID_ARG;         \
    }                                     \
  } while (0)

#define TNX_CHECK_SHAPE(cond, ...)        \
  do {                                    \
    if (!(cond)) {                        \
      ::tnx::set_error(__VA_ARGS__);      \
      return TNX_ERR_SHAPE;               \
    }                                     \
  } while (0)

#define TNX_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t err__ = (call);                                                          \
    if (err__ != cudaSuccess) {                                                          \
      ::tnx::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(err__)); \
      return TNX_ERR_CUDA;                                                               \
    }                                                                                    \
  } while (0)

// every kernel launch of the library goes through TNX_LAUNCH_CHECK, which also counts it
void count_launch();
#define TNX_LAUNCH_CHECK()       \
  do {                           \
    ::tnx::count_launch();       \
    TNX_CUDA(cudaGetLastError()); \
  } while (0)

// Optional CUDA-event timing of one kernel family (enabled by tnx_profile_begin).
enum KernelFamily { KF_TC_GEMM = 0, KF_F64_GEMM = 1, KF_VECTOR = 2, KF_QR_PANEL = 3, KF_EIGH = 4, KF_OTHER = 5,
                    KF_OZ_GEMM = 6, KF_OZ_NARROW = 7, KF_COUNT = 8 };
bool profiling(int family);
void profile_mark(int family, cudaStream_t st, bool start);
// algorithmic work (flops, bytes) of the launch just marked, summed while profiling
void profile_work(int family, double flops, double bytes);

// ---- autotuner (autotune.cu) -------------------------------------------------------------
// Key: {kind, shape...}; kind 1 double-FP32 GEMM tile, 2 FP64-class GEMM engine, 3 split-BF16
// tcgen05 GEMM tile. autotune_choose returns (in *choice) the cached variant for key, or times
// run(0..nv-1) once each on st, caches the fastest and leaves its output in place (*ran = true);
// `fallback` when tuning is off, the stream is capturing, or no candidate ran (*ran = false:
// the caller launches *choice itself). run(v) must overwrite the same outputs for every v.
using TuneKey = std::array<int64_t, 6>;
constexpr int kTuneMaxVariants = 4;
bool autotune_enabled();
int autotune_choose(const TuneKey& key, int nv, int fallback, cudaStream_t st, const std::function<int(int)>& run,
                    int* choice, bool* ran);
// tuned launch: the chosen variant's output is in place on return
inline int autotuned(const TuneKey& key, int nv, int fallback, bool tunable, cudaStream_t st,
                     const std::function<int(int)>& run) {
  int choice = fallback;
  bool ran = false;
  if (tunable) {
    const int rc = autotune_choose(key, nv, fallback, st, run, &choice, &ran);
    if (rc != TNX_OK) return rc;
  }
  return ran ? TNX_OK : run(choice);
}

#define TNX_TRY(call)                     \
  do {                                    \
    int st__ = (call);                    \
    if (st__ != TNX_OK) return st__;      \
  } while (0)

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Bump allocator over a caller-provided workspace.
struct Arena {
  char* base;
  size_t size;
  size_t used = 0;
  Arena(void* b, size_t s) : base(static_cast<char*>(b)), size(s) {}
  template <class T>
  T* take(size_t count) {
    size_t bytes = align_up(count * sizeof(T));
    if (used + bytes > size) return nullptr;
    T* p = reinterpret_cast<T*>(base + used);
    used += bytes;
    return p;
  }
};

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// ---- double-FP32 ("df64") arithmetic helpers ----------------------------------------
// x = hi + lo with |x - hi - lo| < 2^-47 |x| for 2^-100 < |x| < FLT_MAX: hi is x truncated to
// 24 significant bits, lo the remaining 29 mantissa bits truncated to 24 (a float denormal
// when it falls below 2^-126). Integer operations only: the split takes no FP64-pipe issue
// slots (float(x - double(float(x))) costs a DADD and two conversions on that pipe). Zero and
// |x| < 2^-126 give (+-0, +-0); |x| > FLT_MAX gives (+-inf, 0), NaN gives (NaN, 0).
__device__ __forceinline__ void split_df(double x, float& hi, float& lo) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned hw = unsigned(u >> 32), lw = unsigned(u);
  const unsigned sign = hw & 0x80000000u;
  const int e = int((hw >> 20) & 0x7ffu);
  const int fe = e - 896;  // float exponent field: e - 1023 + 127
  const unsigned m23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
  const unsigned r29 = lw & 0x1fffffffu;
  if (fe <= 0) {
    hi = __uint_as_float(sign);
    lo = hi;
    return;
  }
  if (fe >= 255) {
    hi = __uint_as_float(sign | 0x7f800000u | ((e == 2047 && (m23 | r29)) ? 0x400000u : 0u));
    lo = 0.f;
    return;
  }
  hi = __uint_as_float(sign | (unsigned(fe) << 23) | m23);
  unsigned lb = sign;
  if (r29 != 0u) {
    const int p = 31 - __clz(r29);  // leading one of the remainder
    const unsigned full = p >= 23 ? (r29 >> (p - 23)) : (r29 << (23 - p));
    const int le = e - 948 + p;  // float exponent field of lo: (e - 1075 + p) + 127
    if (le > 0) lb |= (unsigned(le) << 23) | (full & 0x7fffffu);
    else if (1 - le < 24) lb |= full >> (1 - le);
  }
  lo = __uint_as_float(lb);
}

// (h, l) -> the nearest double of h + l (two conversions and one FP64 add)
__device__ __forceinline__ double join_df(float h, float l) { return double(h) + double(l); }

// s + e = a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// ---- FP64 GEMM (row-major, optional transposes, strided batch) --------------------
// k_total > 0 selects split-K: batch z multiplies the K slice [z*k, min((z+1)*k, k_total));
// bmask (device, batch ints, may be null) skips the batch entries whose mask is 0
int gemm_f64(bool trans_a, bool trans_b, int64_t m, int64_t n, int64_t k, double alpha,
             const double* A, int64_t lda, int64_t sa, const double* B, int64_t ldb, int64_t sb,
             double beta, double* C, int64_t ldc, int64_t sc, int64_t batch, cudaStream_t st,
             int64_t k_total = 0, const int* bmask = nullptr);
// C = alpha * op(A) op(B) + beta * C with K split over nsplit CTAs layers; part holds
// nsplit * m * n doubles of partial products
int gemm_f64_splitk(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
                    const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int nsplit, double* part,
                    cudaStream_t st, bool df = false);
// double-FP32 emulated GEMM (same contract as gemm_f64)
int gemm_df64(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
              int64_t sa, const double* B, int64_t ldb, int64_t sb, double beta, double* C, int64_t ldc, int64_t sc,
              int64_t batch, cudaStream_t st, int64_t k_total = 0, const int* bmask = nullptr);
// FP64-class GEMM on the tensor cores (Ozaki slicing, gemm_oz.cu); workspace sized by
// gemm_oz_workspace_bytes(m, n, k)
size_t gemm_oz_workspace_bytes(int64_t m, int64_t n, int64_t k);
// Batched (grid z over `batch` operand sets at element strides sA, sB, sC; chains with
// mask[b] == 0 skipped) and split-K (`nsplit` K ranges, partials summed in order) form
size_t gemm_oz_ex_workspace_bytes(int64_t m, int64_t n, int64_t k, int batch, int nsplit);
int gemm_oz_ex(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
               int64_t sA, const double* B, int64_t ldb, int64_t sB, double beta, double* C, int64_t ldc, int64_t sC,
               int batch, int nsplit, const int* mask, void* ws, size_t ws_bytes, cudaStream_t st);
int gemm_oz(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
            const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* ws, size_t ws_bytes,
            cudaStream_t st);
// df = true: double-FP32 emulation; false: native FP64
int gemm_fp64_class(bool df, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                    int64_t lda, int64_t sa, const double* B, int64_t ldb, int64_t sb, double beta, double* C,
                    int64_t ldc, int64_t sc, int64_t batch, cudaStream_t st, int64_t k_total = 0,
                    const int* bmask = nullptr);

// ---- MPO contraction steps ---------------------------------------------------------
// T2[(a',s'),(c,v)] = sum_{w,s} T1[(w,a'),(s,c)] W[w,v,s,s']   (left / matvec form)
int wcontract_left(const double* T1, const double* W, double* T2, int64_t chi_l, int64_t d,
                   int64_t chi_r, int64_t dl, int64_t dr, cudaStream_t st);
// T2[(a,w),(s',c')] = sum_{v,s} T1[(a,s),(v,c')] W[w,v,s,s']   (right form)
int wcontract_right(const double* T1, const double* W, double* T2, int64_t chi_l, int64_t d,
                    int64_t chi_r, int64_t dl, int64_t dr, cudaStream_t st);

// One FP64 one-site matvec with explicit scratch (T1, T2 of matvec1_scratch_elems each).
int64_t matvec1_scratch_elems(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr);
// df: FP64-class (double-FP32, or the tensor-core Ozaki GEMM for large products when oz_ws
// holds matvec1_oz_bytes); otherwise native FP64
int matvec1_f64(const double* L, const double* W, const double* R, const double* x, double* y,
                int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, double* T1,
                double* T2, cudaStream_t st, bool df = false, void* oz_ws = nullptr, size_t oz_bytes = 0);
size_t matvec1_oz_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr);
bool use_oz(int64_t m, int64_t n, int64_t k);
// gemm_fp64_class with the tensor-core FP64-class GEMM for large df products (needs oz_ws)
int gemm_fp64_class_oz(bool df, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                       int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* oz_ws,
                       size_t oz_bytes, cudaStream_t st);
// FP64-class contraction selected by a precision code: TNX_FP64 -> native FP64,
// TNX_BF16X3 / TNX_DF64 -> double-FP32 emulation
inline bool use_df64(int precision) { return precision == TNX_BF16X3 || precision == TNX_DF64; }

// Mixed-precision (split-BF16, tcgen05) matvec; returns TNX_ERR_UNSUPPORTED when the shape
// is outside what the tensor-core kernel handles.
size_t matvec1_bf16x3_scratch_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                                    int64_t dr);
int matvec1_bf16x3(const double* L, const double* W, const double* R, const double* x, double* y,
                   int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, void* scratch,
                   size_t scratch_bytes, cudaStream_t st);

bool mixed_supported(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr);
int mixed_prepare(const double* L, const double* R, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                  void* scratch, cudaStream_t st);
int mixed_apply(const double* W, const double* x, double* y, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                int64_t dr, void* scratch, cudaStream_t st);
// the same product with FP32 input / output vectors
int mixed_apply_f32(const double* W, const float* x, float* y, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                    int64_t dr, void* scratch, cudaStream_t st);
int mixed_flag(void* scratch, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, int** flag);

// ---- dense symmetric eigensolver ------------------------------------------------------
int eigh_small_f64_ld(const double* A, const int64_t* offsets, const int* sizes, const int* lds,
                      int batch, int max_size, int keep, double* evals, double* evecs, double* work,
                      cudaStream_t st);
// single n x n matrix with leading dimension ld; evecs as [n][keep], work 2*n*n doubles
int eigh_small_f64_uniform(const double* A, int n, int ld, int keep, double* evals, double* evecs,
                           double* work, cudaStream_t st);
// lowest eigenpair of one n x n (n <= 64) matrix, one warp: FP32 Jacobi + FP64 refinement
int rr_lowest_f64(const double* A, int n, int ld, double* eval, double* evec, cudaStream_t st);
// the same for `batch` matrices at A + b sA (results at eval + b sE, evec + b sV); blocks whose
// active[b] is 0 return at once (active may be null)
int rr_lowest_f64_batched(const double* A, int n, int ld, int64_t sA, double* eval, int64_t sE, double* evec,
                          int64_t sV, int batch, const int* active, cudaStream_t st);
int eigh_small_f64(double* A, const int64_t* offsets, const int* sizes, int batch, int max_size,
                   int keep, double* evals, double* evecs, double* work, cudaStream_t st);

}  // namespace tnx
