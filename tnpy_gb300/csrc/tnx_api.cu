// Status strings, thread-local error text and the device check of the tnx C ABI.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>

#include "tnx_internal.cuh"

#include <atomic>
#include <mutex>
#include <vector>

namespace tnx {
static thread_local char g_err[1024] = "";
static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// ---- event timing of one kernel family ------------------------------------------------
namespace {
struct Profiler {
  std::mutex mu;
  int family = -1;
  std::vector<cudaEvent_t> ev;  // start, stop pairs
  size_t used = 0;
  bool open = false;
  double flops = 0.0, bytes = 0.0;
};
Profiler g_prof;
constexpr size_t kMaxPairs = 1 << 15;
}  // namespace

bool profiling(int family) { return g_prof.family == family; }

void profile_mark(int family, cudaStream_t st, bool start) {
  if (g_prof.family != family) return;
  std::lock_guard<std::mutex> lk(g_prof.mu);
  if (start) {
    if (g_prof.used >= kMaxPairs) return;
    if (g_prof.ev.size() < 2 * (g_prof.used + 1)) {
      cudaEvent_t a, b;
      if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return;
      g_prof.ev.push_back(a);
      g_prof.ev.push_back(b);
    }
    cudaEventRecord(g_prof.ev[2 * g_prof.used], st);
    g_prof.open = true;
  } else if (g_prof.open) {
    cudaEventRecord(g_prof.ev[2 * g_prof.used + 1], st);
    ++g_prof.used;
    g_prof.open = false;
  }
}

void profile_work(int family, double flops, double bytes) {
  if (g_prof.family != family) return;
  std::lock_guard<std::mutex> lk(g_prof.mu);
  g_prof.flops += flops;
  g_prof.bytes += bytes;
}

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

long long tnx_launch_count(void) { return tnx::g_launches.load(); }

int tnx_profile_begin(int family) {
  std::lock_guard<std::mutex> lk(tnx::g_prof.mu);
  if (family < 0 || family >= tnx::KF_COUNT) return TNX_ERR_INVALID_ARG;
  tnx::g_prof.family = family;
  tnx::g_prof.used = 0;
  tnx::g_prof.open = false;
  tnx::g_prof.flops = tnx::g_prof.bytes = 0.0;
  return TNX_OK;
}

int tnx_profile_end(int* launches, double* total_ms, double* flops, double* bytes) {
  std::lock_guard<std::mutex> lk(tnx::g_prof.mu);
  double tot = 0.0;
  for (size_t i = 0; i < tnx::g_prof.used; ++i) {
    float ms = 0.f;
    if (cudaEventSynchronize(tnx::g_prof.ev[2 * i + 1]) != cudaSuccess ||
        cudaEventElapsedTime(&ms, tnx::g_prof.ev[2 * i], tnx::g_prof.ev[2 * i + 1]) != cudaSuccess) {
      tnx::set_error("tnx_profile_end: event query failed");
      return TNX_ERR_CUDA;
    }
    tot += ms;
  }
  if (launches) *launches = int(tnx::g_prof.used);
  if (total_ms) *total_ms = tot;
  if (flops) *flops = tnx::g_prof.flops;
  if (bytes) *bytes = tnx::g_prof.bytes;
  tnx::g_prof.family = -1;
  tnx::g_prof.used = 0;
  return TNX_OK;
}

int tnx_device_ok(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return 0;
  return (p.major == 10 && p.minor == 3) ? 1 : 0;
}

}  // extern "C"
