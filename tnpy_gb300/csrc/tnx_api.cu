// Status strings, thread-local error text and the device check of the tnx C ABI.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>

#include "tnx_internal.cuh"

namespace tnx {
static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
}  // namespace tnx

extern "C" {

const char* tnx_status_string(int status) {
  switch (status) {
    case TNX_OK: return "ok";
    case TNX_ERR_INVALID_ARG: return "invalid argument";
    case TNX_ERR_SHAPE: return "bad shape";
    case TNX_ERR_WORKSPACE: return "workspace too small";
    case TNX_ERR_NOT_CONVERGED: return "not converged";
    case TNX_ERR_CUDA: return "CUDA error";
    case TNX_ERR_TIMEOUT: return "device wait timed out";
    case TNX_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char* tnx_last_error(void) { return tnx::g_err; }

int tnx_version(void) { return 100; }

int tnx_device_ok(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return 0;
  return (p.major == 10 && p.minor == 3) ? 1 : 0;
}

}  // extern "C"
