// Split-BF16 (three-term) tensor-core one-site matvec. Placeholder until the tcgen05
// kernel lands: reports TNX_ERR_UNSUPPORTED so that callers fail loudly.
#include "tnx_internal.cuh"

namespace tnx {

size_t matvec1_bf16x3_scratch_bytes(int64_t, int64_t, int64_t, int64_t, int64_t) { return 256; }

int matvec1_bf16x3(const double*, const double*, const double*, const double*, double*, int64_t, int64_t,
                   int64_t, int64_t, int64_t, void*, size_t, cudaStream_t) {
  set_error("split-BF16 matvec not built");
  return TNX_ERR_UNSUPPORTED;
}

}  // namespace tnx
