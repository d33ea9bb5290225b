// One-site FP64 matvec that allocates nothing: its two intermediates live in a file-scope
// device array instead of a caller-provided workspace.
//
// Some callers cannot call cudaMalloc at the point where they need H_eff x: code running
// inside a stream capture that must not allocate, allocator-less embeddings (a solver loop
// driven from a host language binding that owns no device allocator), or a process whose
// device memory is fully reserved by another framework's pool. They pass only the inputs
// and the output; the scratch is the static array below.
//
// The array holds 2 x TNX_NOALLOC_MAX_ELEMS doubles (32 MiB) on every device that loads
// the library, for the life of the process. Every call shares it and the array keeps the
// last call's contents; both intermediates are fully overwritten by each call before they
// are read, so nothing needs clearing. Calls that overlap on the GPU (different streams,
// or several host threads) race on the array; serialise them.
#include <cuda_runtime.h>

#include <mutex>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

constexpr int64_t kNoallocElems = TNX_NOALLOC_MAX_ELEMS;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[2 * kNoallocElems];

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the array on the current device. In host code the array's name is only
// a host-side stand-in, so the address is looked up once per device with that device
// current (the first call on a device does this; it should come before any stream capture).
int noalloc_scratch(double** out) {
  int dev = 0;
  TNX_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("tnx_matvec1_noalloc: device ordinal %d out of range", dev);
    return TNX_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    TNX_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return TNX_OK;
}

}  // namespace
}  // namespace tnx

using namespace tnx;

extern "C" int tnx_matvec1_noalloc(const double* L, const double* W, const double* R, const double* x, double* y,
                                   int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, void* stream) {
  TNX_CHECK_ARG(L && W && R && x && y, "null pointer");
  TNX_CHECK_ARG(chi_l > 0 && d > 0 && chi_r > 0 && dl > 0 && dr > 0, "non-positive dimension");
  TNX_CHECK_SHAPE(d <= 64 && dl <= 64 && dr <= 64 && dl * d <= 64 && dr * d <= 64,
                  "MPO bond too large: dl*d=%lld dr*d=%lld (max 64)", (long long)(dl * d), (long long)(dr * d));
  // each bond alone must fit before the product is formed: with chi_l, chi_r <= 2^21 and
  // d, dl, dr <= 64 the product below stays under 2^60 and cannot wrap
  TNX_CHECK_SHAPE(chi_l <= kNoallocElems && chi_r <= kNoallocElems,
                  "tnx_matvec1_noalloc: bond %lld x %lld exceeds the static scratch of %lld elements",
                  (long long)chi_l, (long long)chi_r, (long long)kNoallocElems);
  const int64_t need = matvec1_scratch_elems(chi_l, d, chi_r, dl, dr);
  TNX_CHECK_SHAPE(need <= kNoallocElems,
                  "tnx_matvec1_noalloc: chi_l*d*chi_r*max(dl,dr) = %lld exceeds the static scratch of %lld "
                  "elements; use tnx_matvec1 with a workspace",
                  (long long)need, (long long)kNoallocElems);
  double* scratch = nullptr;
  TNX_TRY(noalloc_scratch(&scratch));
  return matvec1_f64(L, W, R, x, y, chi_l, d, chi_r, dl, dr, scratch, scratch + kNoallocElems, as_stream(stream));
}
