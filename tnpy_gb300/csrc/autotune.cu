// Autotuner: the kernel variant of a call site is picked per shape by timing every candidate
// once on the caller's stream and caching the fastest for the rest of the process.
//
// Tuned decisions (kind: key -> candidates):
//   1 double-FP32 GEMM tile        (trans, m, n, k, batch) -> 64 x 128 tiles / 256 threads, 32 x 32 / 64
//   2 FP64-class GEMM engine        (trans, m, n, k)        -> tcgen05 Ozaki GEMM, double-FP32 SIMT GEMM
//   3 split-BF16 tcgen05 GEMM tile  (m, n, k)               -> 128 x 256 tiles, 128 x 128 tiles
// Only calls whose output is overwritten (beta = 0) are tuned, so that running every candidate
// leaves the same result in place; a call inside a stream capture, or with tuning switched off
// (tnx_autotune_set(0) or TNX_AUTOTUNE=0), takes the cached choice or the fixed size rule.
// Each candidate runs once untimed (first-launch set-up, nested tuning of its own sub-calls)
// and once between two CUDA events; the lowest time wins. Tuning holds one process-wide
// (recursive) lock, so concurrent first calls of different streams do not time each other.
#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "tnx_internal.cuh"

namespace tnx {
namespace {

struct Entry {
  int choice = 0;
  int nv = 0;
  float ms[kTuneMaxVariants] = {};
};

std::recursive_mutex g_tune_mu;  // held while candidates run (nested tuning re-enters)
std::mutex g_map_mu;              // guards the cache map only (short lookups)
std::map<TuneKey, Entry> g_tune;

bool lookup(const TuneKey& key, int* choice) {
  std::lock_guard<std::mutex> lk(g_map_mu);
  auto it = g_tune.find(key);
  if (it == g_tune.end()) return false;
  *choice = it->second.choice;
  return true;
}
std::atomic<int> g_tune_on{-1};

}  // namespace

bool autotune_enabled() {
  int e = g_tune_on.load();
  if (e < 0) {
    const char* s = getenv("TNX_AUTOTUNE");
    e = (s && s[0] == '0') ? 0 : 1;
    g_tune_on.store(e);
  }
  return e == 1;
}

int autotune_choose(const TuneKey& key, int nv, int fallback, cudaStream_t st,
                    const std::function<int(int)>& run, int* choice, bool* ran) {
  *choice = fallback;
  *ran = false;
  if (lookup(key, choice)) return TNX_OK;
  std::lock_guard<std::recursive_mutex> lk(g_tune_mu);
  if (lookup(key, choice)) return TNX_OK;  // tuned by another thread meanwhile
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (!autotune_enabled() || nv < 2 || nv > kTuneMaxVariants ||
      cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return TNX_OK;
  cudaEvent_t e0, e1;
  TNX_CUDA(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    set_error("autotune: cudaEventCreate failed");
    return TNX_ERR_CUDA;
  }
  Entry ent;
  ent.nv = nv;
  int best = -1, rc = TNX_OK;
  for (int v = 0; v < nv && rc == TNX_OK; ++v) {
    ent.ms[v] = -1.f;
    if (run(v) != TNX_OK) continue;  // a candidate that does not apply to this shape
    if (cudaEventRecord(e0, st) != cudaSuccess) { rc = TNX_ERR_CUDA; break; }
    const int r = run(v);
    if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) { rc = TNX_ERR_CUDA; break; }
    if (r != TNX_OK) continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) { rc = TNX_ERR_CUDA; break; }
    ent.ms[v] = ms;
    if (best < 0 || ms < ent.ms[best]) best = v;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != TNX_OK) {
    set_error("autotune: event timing failed");
    return rc;
  }
  if (best < 0) return TNX_OK;  // no candidate ran: keep the size rule, tune again next time
  // the winner's output must be the one left in place: rerun it when it was not the last
  if (best != nv - 1 || ent.ms[nv - 1] < 0.f) TNX_TRY(run(best));
  ent.choice = best;
  {
    std::lock_guard<std::mutex> mk(g_map_mu);
    g_tune[key] = ent;
  }
  *choice = best;
  *ran = true;
  return TNX_OK;
}

}  // namespace tnx

using namespace tnx;

extern "C" {

int tnx_autotune_set(int enable) {
  g_tune_on.store(enable ? 1 : 0);
  return TNX_OK;
}

int tnx_autotune_clear(void) {
  std::lock_guard<std::mutex> lk(g_map_mu);
  g_tune.clear();
  return TNX_OK;
}

int tnx_autotune_count(void) {
  std::lock_guard<std::mutex> lk(g_map_mu);
  return int(g_tune.size());
}

size_t tnx_autotune_report(char* buf, size_t len) {
  std::lock_guard<std::mutex> lk(g_map_mu);
  std::string out;
  char line[256];
  for (const auto& [k, e] : g_tune) {
    int o = snprintf(line, sizeof(line), "%lld %lld %lld %lld %lld %lld -> %d", (long long)k[0], (long long)k[1],
                     (long long)k[2], (long long)k[3], (long long)k[4], (long long)k[5], e.choice);
    for (int v = 0; v < e.nv && o > 0 && size_t(o) < sizeof(line); ++v)
      o += snprintf(line + o, sizeof(line) - size_t(o), " %.4f", double(e.ms[v]));
    out += line;
    out += '\n';
  }
  if (buf && len) {
    const size_t n = out.size() < len - 1 ? out.size() : len - 1;
    memcpy(buf, out.data(), n);
    buf[n] = '\0';
  }
  return out.size() + 1;
}

}  // extern "C"
