// Internal helpers shared by the tnx translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>

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
                    KF_COUNT = 6 };
bool profiling(int family);
void profile_mark(int family, cudaStream_t st, bool start);
// algorithmic work (flops, bytes) of the launch just marked, summed while profiling
void profile_work(int family, double flops, double bytes);

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

// ---- FP64 GEMM (row-major, optional transposes, strided batch) --------------------
// k_total > 0 selects split-K: batch z multiplies the K slice [z*k, min((z+1)*k, k_total))
int gemm_f64(bool trans_a, bool trans_b, int64_t m, int64_t n, int64_t k, double alpha,
             const double* A, int64_t lda, int64_t sa, const double* B, int64_t ldb, int64_t sb,
             double beta, double* C, int64_t ldc, int64_t sc, int64_t batch, cudaStream_t st,
             int64_t k_total = 0);
// C = alpha * op(A) op(B) + beta * C with K split over nsplit CTAs layers; part holds
// nsplit * m * n doubles of partial products
int gemm_f64_splitk(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
                    const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int nsplit, double* part,
                    cudaStream_t st, bool df = false);
// double-FP32 emulated GEMM (same contract as gemm_f64)
int gemm_df64(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
              int64_t sa, const double* B, int64_t ldb, int64_t sb, double beta, double* C, int64_t ldc, int64_t sc,
              int64_t batch, cudaStream_t st, int64_t k_total = 0);
// df = true: double-FP32 emulation; false: native FP64
int gemm_fp64_class(bool df, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                    int64_t lda, int64_t sa, const double* B, int64_t ldb, int64_t sb, double beta, double* C,
                    int64_t ldc, int64_t sc, int64_t batch, cudaStream_t st, int64_t k_total = 0);

// ---- MPO contraction steps ---------------------------------------------------------
// T2[(a',s'),(c,v)] = sum_{w,s} T1[(w,a'),(s,c)] W[w,v,s,s']   (left / matvec form)
int wcontract_left(const double* T1, const double* W, double* T2, int64_t chi_l, int64_t d,
                   int64_t chi_r, int64_t dl, int64_t dr, cudaStream_t st);
// T2[(a,w),(s',c')] = sum_{v,s} T1[(a,s),(v,c')] W[w,v,s,s']   (right form)
int wcontract_right(const double* T1, const double* W, double* T2, int64_t chi_l, int64_t d,
                    int64_t chi_r, int64_t dl, int64_t dr, cudaStream_t st);

// One FP64 one-site matvec with explicit scratch (T1, T2 of matvec1_scratch_elems each).
int64_t matvec1_scratch_elems(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr);
int matvec1_f64(const double* L, const double* W, const double* R, const double* x, double* y,
                int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, double* T1,
                double* T2, cudaStream_t st, bool df = false);
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
int eigh_small_f64(double* A, const int64_t* offsets, const int* sizes, int batch, int max_size,
                   int keep, double* evals, double* evecs, double* work, cudaStream_t st);

}  // namespace tnx
