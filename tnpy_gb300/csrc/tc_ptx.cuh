// tcgen05 / TMA / mbarrier helpers shared by the tensor-core kernels (inline PTX, sm_103a).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace tnx {
namespace tc {

constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz: bound of every mbarrier wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: true when the phase completed, false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > WAIT_CYCLES) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  // K-major operand, 128-byte swizzle: 8-row groups 1024 bytes apart (SBO), LBO unused,
  // descriptor version 1 (bits 46-47), layout type 2 = SWIZZLE_128B (bits 61-63)
  uint64_t d = 0;
  d |= uint64_t((addr >> 4) & 0x3FFF);
  d |= uint64_t(1) << 16;                // LBO (ignored for swizzled K-major)
  d |= uint64_t(1024 >> 4) << 32;        // SBO
  d |= uint64_t(1) << 46;                // version
  d |= uint64_t(2) << 61;                // SWIZZLE_128B
  return d;
}

__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t addr) {
  // K-major operand, 64-byte swizzle: 64-byte rows, 8-row groups 512 bytes apart (SBO), LBO
  // unused, descriptor version 1, layout type 4 = SWIZZLE_64B (bits 61-63)
  uint64_t d = 0;
  d |= uint64_t((addr >> 4) & 0x3FFF);
  d |= uint64_t(1) << 16;
  d |= uint64_t(512 >> 4) << 32;
  d |= uint64_t(1) << 46;
  d |= uint64_t(4) << 61;
  return d;
}

__host__ __device__ constexpr uint32_t instr_desc_bf16(int m, int n) {
  // D = F32 (bits 4-5 = 1), A = BF16 (bits 7-9 = 1), B = BF16 (bits 10-12 = 1), both K-major,
  // N >> 3 at bits 17-22, M >> 4 at bits 24-28
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 lanes x 32 columns of FP32 from tensor memory into r; the registers are valid only after
// tmem_ld_wait() (several loads may be in flight before one wait)
__device__ __forceinline__ void tmem_ld32_async(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  tmem_ld32_async(taddr, r);
  tmem_ld_wait();
}

}  // namespace tc

// 2-D TMA map over a K-major bf16 matrix rows x ldp (K innermost), box {box_k, box_rows},
// 128-byte swizzle for box_k = 64, 64-byte swizzle for box_k = 32. Rows beyond `rows` read as
// zero.
int make_tma_map_bf16(CUtensorMap* map, const void* ptr, int64_t rows, int64_t ldp, int box_k, int box_rows);

}  // namespace tnx
