// FP64-class GEMM on the tcgen05 tensor cores by exact integer slicing (Ozaki scheme).
//
//   C = alpha op(A) op(B) + beta C,   FP64 in and out.
//
// Row i of op(A) is scaled by 2^-ea_i so that its entries are below 1/2 in magnitude and cut, by
// integer extraction from the 53-bit mantissa in signed fixed point, into S = 8 balanced base-128
// digits (each rounded to nearest, so the remainder after digit s is at most half a unit of it):
//   op(A)_ik 2^-ea_i = sum_{s<S} qa_s,ik 2^-7(s+1) + r_ik,   |r_ik| <= 2^-57,   |qa_s,ik| <= 64,
// integers that BF16 holds exactly. Column j of op(B) likewise with eb_j. Then
//   C_ij = 2^(ea_i + eb_j) sum_{g<S} 2^-7(g+2) P_g,ij + O(2^-53) per product,
//   P_g,ij = sum_{s+t=g} sum_k qa_s,ik qb_t,kj                          (36 slice pairs),
// and every P_g is a sum of integer products of magnitude at most 2^12. Over KC = 480 values of
// k the partial sum of a group (at most 8 pairs) stays below 8 * 480 * 2^12 < 2^24, so the FP32
// accumulation of the tensor cores in tensor memory is exact; every KC the eight group
// accumulators are drained into a double-FP32 running sum per output (epilogue warps), scaled
// by 2^-7(g+2). (Unbalanced 7-bit digits up to 127 would allow only KC = 128: the drains, which
// stall the MMAs, are 3.75x rarer with balanced ones.)
// Error: ~2^-52 per product relative to 2^ea_i 2^eb_j (the row / column maxima), plus the
// double-FP32 summation (~2^-46 of the running sum): FP64-class where rows and columns do not
// span many decades; at the tensor cores' rate divided by 36.
//
// Kernel: one 128 x 64 output tile per CTA, 10 warps: warp 0 TMA producer (all 2 S slice tiles of
// a 32-deep K block per stage, 2 stages of 96 KB, 64-byte swizzle), warp 1 TMEM allocation (512
// columns: eight 64-column group accumulators) and single-thread tcgen05.mma issue of the 36
// slice products per K block as 12 MMAs per 16-deep step (slice q of A against the B slices
// 0..7-q at once, N up to 256), warps 2-9 epilogue (two per TMEM lane quarter, 32 columns
// each). All
// mbarrier waits are bounded (~2 s); on expiry the kernel raises the error flag and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include "tc_ptx.cuh"
#include "tnx_internal.cuh"

namespace tnx {
namespace {

using namespace tc;

constexpr int OZ_S = 8;                         // slices per operand
constexpr int OZ_BM = 128, OZ_BN = 64, OZ_BK = 32;  // BK = 32 bf16 = one 64-byte swizzle row
constexpr int OZ_KC = 480;                      // K values per exact accumulation chunk
constexpr int OZ_STAGES = 2;                    // a stage holds all 2 S slice tiles of one K block
constexpr int OZ_EPI_WARPS = 8;                 // two per TMEM lane quarter, 32 columns each
constexpr int OZ_THREADS = 64 + 32 * OZ_EPI_WARPS;
constexpr uint32_t OZ_TMEM_COLS = 512;

// ---------------------------------------------------------------- operand slicing
// Logical operand X(r, k) = src[r * rs + k * ks], rows x K (FP64). bmax[r] (zeroed before) =
// largest biased FP64 exponent in row r, by atomicMax over CTAs of 32 rows x OZ_SCAN_K values of
// k (the scan runs over the whole grid, not one CTA per row block). The row's scale exponent is
// E = bmax - 1021 (|X(r, k)| < 2^(E-1)), 0 for an all-zero row: row_scale_exp. bmax = 2047 marks
// a row with Inf or NaN, whose outputs the GEMM epilogue sets to NaN.
constexpr int OZ_SCAN_K = 256;
__global__ void oz_rowmax_kernel(const double* __restrict__ src, int64_t rows, int64_t K, int64_t rs, int64_t ks,
                                 int* __restrict__ bmax, int64_t s_src, int64_t s_bmax, const int* __restrict__ mask) {
  __shared__ int tile[32][33];
  if (mask && !mask[blockIdx.z]) return;  // a chain the caller masked out
  src += int64_t(blockIdx.z) * s_src;
  bmax += int64_t(blockIdx.z) * s_bmax;
  const int64_t r0 = int64_t(blockIdx.y) * 32, kb = int64_t(blockIdx.x) * OZ_SCAN_K;
  const int tx = threadIdx.x, ty = threadIdx.y;
  int best = 0;  // biased exponent, 0 = zero / denormal
  for (int64_t k0 = kb; k0 < K && k0 < kb + OZ_SCAN_K; k0 += 32) {
    for (int i = ty; i < 32; i += 8) {
      // unit stride along k: tx runs over k; along r: tx runs over r
      const int64_t r = ks == 1 ? r0 + i : r0 + tx, k = ks == 1 ? k0 + tx : k0 + i;
      int e = 0;
      if (r < rows && k < K) e = int((unsigned(__double_as_longlong(src[r * rs + k * ks]) >> 52)) & 0x7ffu);
      if (ks == 1) tile[i][tx] = e;
      else tile[tx][i] = e;
    }
    __syncthreads();
    if (ty == 0)
      for (int j = 0; j < 32; ++j) best = max(best, tile[tx][j]);
    __syncthreads();
  }
  if (ty == 0 && best > 0 && r0 + tx < rows) atomicMax(&bmax[r0 + tx], best);
}

__device__ __forceinline__ int row_scale_exp(int bmax) { return bmax > 0 ? bmax - 1021 : 0; }

// x 2^e: one multiplication by the power of two where that is a normal double (exact, or rounded
// once where the result is subnormal, as ldexp rounds it), ldexp outside that range
__device__ __forceinline__ double scale_pow2(double x, int e) {
  if (e >= -1022 && e <= 1023) return x * __longlong_as_double(static_cast<long long>(e + 1023) << 52);
  return ldexp(x, e);
}

// bf16 bit pattern of an integer 0 <= q <= 255 (exact)
__device__ __forceinline__ uint16_t bf16_of_small_int(unsigned q, unsigned sign) {
  if (q == 0u) return 0;
  const int e = 31 - __clz(q);
  const unsigned mant = (q << (7 - e)) & 0x7fu;
  return uint16_t((sign << 15) | (unsigned(127 + e) << 7) | mant);
}

// planes[s][r][k] (row pitch Kp, rows_pad rows per plane) = slice s of X(r, k) 2^-E[r];
// zero for r >= rows or k >= K.
__global__ void oz_slice_kernel(const double* __restrict__ src, int64_t rows, int64_t K, int64_t rs, int64_t ks,
                                const int* __restrict__ exps, uint16_t* __restrict__ planes, int64_t rows_pad,
                                int64_t Kp, int64_t s_src, const int* __restrict__ mask) {
  __shared__ double tile[32][33];
  if (mask && !mask[blockIdx.z]) return;
  src += int64_t(blockIdx.z) * s_src;
  exps += int64_t(blockIdx.z) * rows_pad;
  planes += int64_t(blockIdx.z) * OZ_S * rows_pad * Kp;
  const int64_t r0 = int64_t(blockIdx.y) * 32, k0 = int64_t(blockIdx.x) * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int i = ty; i < 32; i += 8) {
    const int64_t r = ks == 1 ? r0 + i : r0 + tx, k = ks == 1 ? k0 + tx : k0 + i;
    const double v = (r < rows && k < K) ? src[r * rs + k * ks] : 0.0;
    if (ks == 1) tile[i][tx] = v;
    else tile[tx][i] = v;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int64_t r = r0 + i, k = k0 + tx;
    if (r >= rows_pad || k >= Kp) continue;
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(tile[i][tx]));
    const int eb = int((u >> 52) & 0x7ffu);
    long long X = 0;  // x 2^-E in signed fixed point with 63 fraction bits, |X| < 2^62
    if (eb != 0 && r < rows) {
      const unsigned long long m53 = (u & ((1ull << 52) - 1)) | (1ull << 52);
      const int shift = eb - 1012 - row_scale_exp(exps[r]);  // <= 9 since |x| < 2^(E-1)
      const unsigned long long F = shift >= 0 ? (m53 << shift) : (-shift < 64 ? (m53 >> -shift) : 0ull);
      X = (u >> 63) ? -static_cast<long long>(F) : static_cast<long long>(F);
    }
    // balanced digits: q_s = X / 2^(56 - 7s) rounded to nearest, X -= q_s 2^(56 - 7s); the
    // remainder before digit s is at most 2^(62 - 7s) in magnitude, so |q_s| <= 64
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) {
      const int sh = 56 - 7 * s;
      const long long q = (X + (1LL << (sh - 1))) >> sh;
      X -= q * (1LL << sh);
      planes[(size_t(s) * rows_pad + r) * Kp + k] = bf16_of_small_int(unsigned(q < 0 ? -q : q), q < 0 ? 1u : 0u);
    }
  }
}

// ---------------------------------------------------------------- GEMM kernel
// Stage layout (one K block of 32): A slices 0..S-1 (128 x 32 bf16, 8 KB each), then B slices
// 0..S-1 (64 x 32 bf16, 4 KB each), 64-byte swizzle; every slice tile is loaded once per K
// block and feeds all S(S+1)/2 slice products that use it. The B slice tiles lie back to back
// with the same 8-row swizzle groups, so B slices t0..t0+w-1 read as one (64 w) x 32 operand; the
// group accumulators lie back to back in TMEM (group g at column 64 g), so the products of A
// slice q with B slices t0..t0+w-1 land in groups q+t0..q+t0+w-1 by one MMA of N = 64 w. Per
// 16-deep step: A slice q against B slices 0..7-q in MMAs of N <= 256 (2, 2, 2, 2, 1, 1, 1, 1 for
// q = 0..7), 12 MMAs instead of 36, each A slice read from shared memory once or twice instead of
// 8 - q times.
// Batch and split-K: blockIdx.z = bz * nsplit + sz. Chain bz reads its slice planes at plane rows
// (bz * S + q) * Mp (A) / (bz * S + q) * Np (B) and its exponents at ea + bz Mp / eb + bz Np;
// split sz covers K blocks [sz kbs, (sz + 1) kbs). With nsplit == 1 the CTA writes
// C + bz sC = alpha P + beta C; otherwise the unscaled partial P to part[(sz * batch + bz) M N]
// (row-major, ld N), which oz_split_reduce_kernel sums in split order.
__global__ void __launch_bounds__(OZ_THREADS, 1)
    oz_gemm_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int M, int N,
                   int Kp, int Mp, int Np, const int* __restrict__ ea, const int* __restrict__ eb, double alpha,
                   double beta, double* __restrict__ C, int64_t ldc, int* __restrict__ err_flag, int batch,
                   int nsplit, int kbs, int64_t sC, double* __restrict__ part, const int* __restrict__ mask) {
  constexpr uint32_t A_TILE = OZ_BM * OZ_BK * 2, B_TILE = OZ_BN * OZ_BK * 2;
  constexpr uint32_t STAGE_BYTES = OZ_S * (A_TILE + B_TILE);
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[OZ_STAGES], empty_bar[OZ_STAGES], chunk_full, chunk_empty;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh, epi_fail_sh;
  const int bz = int(blockIdx.z) / nsplit, sz = int(blockIdx.z) % nsplit;
  if (mask && !mask[bz]) return;  // uniform over the CTA, before any barrier or TMEM allocation
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int m0 = blockIdx.y * OZ_BM, n0 = blockIdx.x * OZ_BN;
  const int kb_all = Kp / OZ_BK;
  const int kb0 = sz * kbs, kb1 = min(kb_all, kb0 + kbs);
  const int kblocks = kb1 > kb0 ? kb1 - kb0 : 0;
  const int kb_per_chunk = OZ_KC / OZ_BK;
  const int nchunks = (kblocks + kb_per_chunk - 1) / kb_per_chunk;
  const int a_row0 = bz * OZ_S * Mp, b_row0 = bz * OZ_S * Np;
  ea += int64_t(bz) * Mp;
  eb += int64_t(bz) * Np;

  if (threadIdx.x == 0) {
    for (int st = 0; st < OZ_STAGES; ++st) {
      mbar_init(smem_u32(&full_bar[st]), 1);
      mbar_init(smem_u32(&empty_bar[st]), 1);
    }
    mbar_init(smem_u32(&chunk_full), 1);
    mbar_init(smem_u32(&chunk_empty), OZ_EPI_WARPS);
    abort_sh = 0;
    epi_fail_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"(OZ_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base_sh;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer: one K block per stage
    if (lane == 0) {
      int issued = 0;
      for (int kb = 0; kb < kblocks; ++kb) {
        const int st = kb % OZ_STAGES;
        const uint32_t ph = (kb / OZ_STAGES) & 1;
        if (kb >= OZ_STAGES && !mbar_wait(smem_u32(&empty_bar[st]), ph ^ 1)) {
          atomicExch(err_flag, 1);
          abort_sh = 1;
          break;
        }
        if (*((volatile int*)&abort_sh)) break;
        const uint32_t sa = base + st * STAGE_BYTES, sb = sa + OZ_S * A_TILE;
        const uint32_t fb = smem_u32(&full_bar[st]);
        mbar_expect_tx(fb, STAGE_BYTES);
        for (int q = 0; q < OZ_S; ++q) {
          tma_load_2d(sa + q * A_TILE, &ta, fb, (kb0 + kb) * OZ_BK, a_row0 + q * Mp + m0);
          tma_load_2d(sb + q * B_TILE, &tb, fb, (kb0 + kb) * OZ_BK, b_row0 + q * Np + n0);
        }
        ++issued;
      }
      for (int kb = issued - OZ_STAGES < 0 ? 0 : issued - OZ_STAGES; kb < issued; ++kb)
        mbar_wait(smem_u32(&full_bar[kb % OZ_STAGES]), (kb / OZ_STAGES) & 1);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      bool ok = true;
      for (int c = 0; c < nchunks && ok; ++c) {
        // the epilogue must have read the previous chunk's accumulators
        if (c > 0 && !mbar_wait(smem_u32(&chunk_empty), (c - 1) & 1)) {
          atomicExch(err_flag, 1);
          abort_sh = 1;
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const int kb_end = min(kblocks, (c + 1) * kb_per_chunk);
        for (int kb = c * kb_per_chunk; kb < kb_end; ++kb) {
          const int st = kb % OZ_STAGES;
          const uint32_t ph = (kb / OZ_STAGES) & 1;
          if (!mbar_wait(smem_u32(&full_bar[st]), ph) || *((volatile int*)&abort_sh)) {
            atomicExch(err_flag, 1);
            abort_sh = 1;
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t sa = base + st * STAGE_BYTES, sb = sa + OZ_S * A_TILE;
          const bool chunk_start = kb == c * kb_per_chunk;
#pragma unroll
          for (int kk = 0; kk < OZ_BK / 16; ++kk) {
#pragma unroll
            for (int q = 0; q < OZ_S; ++q) {
              const uint64_t ad = smem_desc_sw64(sa + q * A_TILE + kk * 32);
#pragma unroll
              for (int t0 = 0; t0 < OZ_S - q; t0 += 4) {
                // slice pairs (q, t0) .. (q, t0 + w - 1) into groups q + t0 .. q + t0 + w - 1; the two
                // MMAs of (q = 0, kk = 0) cover all eight groups and start a chunk's sums
                const int w = OZ_S - q - t0 < 4 ? OZ_S - q - t0 : 4;
                const uint64_t bd = smem_desc_sw64(sb + t0 * B_TILE + kk * 32);
                mma_bf16(tmem + uint32_t((q + t0) * OZ_BN), ad, bd, instr_desc_bf16(OZ_BM, OZ_BN * w),
                         (chunk_start && kk == 0 && q == 0) ? 0u : 1u);
              }
            }
          }
          mma_commit(smem_u32(&empty_bar[st]));
        }
        if (ok) mma_commit(smem_u32(&chunk_full));
      }
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2..9): tile row = lane of
    // the warp's TMEM lane quarter (warp mod 4), columns cb..cb+31 of every group (two warps a
    // quarter)
    const int quad = warp & 3;
    const int cb = (warp - 2) / 4 * 32;
    float hi[32], lo[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) hi[j] = lo[j] = 0.f;
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
      if (!mbar_wait(smem_u32(&chunk_full), c & 1)) {
        if (lane == 0) atomicExch(err_flag, 1);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
      for (int g = 0; g < OZ_S; g += 2) {  // two groups' loads in flight per wait
        uint32_t r[2][32];
        tmem_ld32_async(tmem + (uint32_t(quad * 32) << 16) + uint32_t(g * OZ_BN + cb), r[0]);
        tmem_ld32_async(tmem + (uint32_t(quad * 32) << 16) + uint32_t((g + 1) * OZ_BN + cb), r[1]);
        tmem_ld_wait();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float scale = __uint_as_float(uint32_t(127 - 7 * (g + h + 2)) << 23);  // 2^-7(g+h+2)
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const float v = __uint_as_float(r[h][j]) * scale;  // exact: power-of-two scaling
            float sum, err;
            two_sum_f(hi[j], v, sum, err);
            hi[j] = sum;
            lo[j] += err;
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&chunk_empty)) : "memory");
    }
    // the finished tile goes through shared memory (the stage buffers are free once the last
    // chunk's MMAs are done), so that the global stores are whole row segments: a thread owns one
    // row of 32 columns in TMEM, and storing from there would write 32 rows per warp instruction
    if (!ok) epi_fail_sh = 1;
    double* Cs = reinterpret_cast<double*>(smem_raw + (base - smem_u32(smem_raw)));  // [BM][BN + 1]
    if (ok) {
      const int lr = quad * 32 + lane;
      const int er = row_scale_exp(ea[m0 + lr]);  // ea and eb are padded to Mp and Np entries
      const bool row_nonfinite = ea[m0 + lr] == 2047;  // the row holds Inf / NaN: its slices are not the value
      const int* ebc = eb + n0 + cb;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        double v = scale_pow2(join_df(hi[j], lo[j]), er + row_scale_exp(ebc[j]));
        if (row_nonfinite || ebc[j] == 2047) v = __longlong_as_double(0x7ff8000000000000LL);
        Cs[lr * (OZ_BN + 1) + cb + j] = v;
      }
    }
    asm volatile("bar.sync 1, %0;" ::"n"(32 * OZ_EPI_WARPS) : "memory");  // the epilogue warps only
    if (!epi_fail_sh) {
      const int et = threadIdx.x - 64;
      double* out = nsplit == 1 ? C + int64_t(bz) * sC : part + (int64_t(sz) * batch + bz) * M * N;
      const int64_t ldo = nsplit == 1 ? ldc : N;
      for (int idx = et; idx < OZ_BM * OZ_BN; idx += 32 * OZ_EPI_WARPS) {
        const int r = idx / OZ_BN, c = idx % OZ_BN;
        if (m0 + r < M && n0 + c < N) {
          double v = Cs[r * (OZ_BN + 1) + c];
          double* o = out + int64_t(m0 + r) * ldo + n0 + c;
          if (nsplit == 1) {
            v *= alpha;
            if (beta != 0.0) v = fma(beta, *o, v);
          }
          *o = v;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(OZ_TMEM_COLS));
  }
}

// C[bz] = alpha sum_s part[s][bz] + beta C[bz] (split order fixed: deterministic)
__global__ void oz_split_reduce_kernel(const double* __restrict__ part, int nsplit, int batch, int M, int N,
                                       double alpha, double beta, double* __restrict__ C, int64_t ldc, int64_t sC,
                                       const int* __restrict__ mask) {
  const int bz = blockIdx.y;
  if (mask && !mask[bz]) return;
  const int64_t MN = int64_t(M) * N;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < MN; e += int64_t(gridDim.x) * blockDim.x) {
    double v = 0.0;
    for (int s = 0; s < nsplit; ++s) v += part[(int64_t(s) * batch + bz) * MN + e];
    double* o = C + int64_t(bz) * sC + (e / N) * ldc + (e % N);
    v *= alpha;
    if (beta != 0.0) v = fma(beta, *o, v);
    *o = v;
  }
}

struct OzLayout {
  int64_t Mp, Np, Kp;
  uint16_t *sa, *sb;
  int *ea, *eb, *flag;
  double* part;
};

size_t oz_layout(int64_t m, int64_t n, int64_t k, int64_t batch, int nsplit, void* base, OzLayout* L) {
  OzLayout o;
  o.Mp = (m + OZ_BM - 1) / OZ_BM * OZ_BM;
  o.Np = (n + OZ_BN - 1) / OZ_BN * OZ_BN;
  o.Kp = (k + OZ_BK - 1) / OZ_BK * OZ_BK;
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t r = off; off += align_up(bytes); return r; };
  const size_t osa = take(size_t(batch) * OZ_S * o.Mp * o.Kp * 2), osb = take(size_t(batch) * OZ_S * o.Np * o.Kp * 2),
               oea = take(size_t(batch) * o.Mp * 4), oeb = take(size_t(batch) * o.Np * 4), ofl = take(4),
               opt = take(nsplit > 1 ? size_t(nsplit) * batch * m * n * 8 : 0);
  if (base && L) {
    char* b = static_cast<char*>(base);
    o.sa = reinterpret_cast<uint16_t*>(b + osa);
    o.sb = reinterpret_cast<uint16_t*>(b + osb);
    o.ea = reinterpret_cast<int*>(b + oea);
    o.eb = reinterpret_cast<int*>(b + oeb);
    o.flag = reinterpret_cast<int*>(b + ofl);
    o.part = reinterpret_cast<double*>(b + opt);
    *L = o;
  }
  return off;
}

size_t oz_smem_bytes() { return size_t(OZ_STAGES) * OZ_S * (OZ_BM * OZ_BK * 2 + OZ_BN * OZ_BK * 2) + 1024; }

}  // namespace

size_t gemm_oz_workspace_bytes(int64_t m, int64_t n, int64_t k) { return oz_layout(m, n, k, 1, 1, nullptr, nullptr); }
size_t gemm_oz_ex_workspace_bytes(int64_t m, int64_t n, int64_t k, int batch, int nsplit) {
  return oz_layout(m, n, k, batch, nsplit, nullptr, nullptr);
}

int gemm_oz_ex(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
               int64_t sA, const double* B, int64_t ldb, int64_t sB, double beta, double* C, int64_t ldc, int64_t sC,
               int batch, int nsplit, const int* mask, void* ws, size_t ws_bytes, cudaStream_t st) {
  if (m <= 0 || n <= 0 || batch <= 0) return TNX_OK;
  TNX_CHECK_ARG(nsplit >= 1 && batch <= 65535 && int64_t(batch) * nsplit <= 65535, "gemm_oz: batch %d x split %d",
                batch, nsplit);
  if (k <= 0) {
    if (batch == 1 && !mask) return gemm_f64(ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1, st);
    return gemm_f64(ta, tb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, st, 0, mask);
  }
  TNX_CHECK_SHAPE(int64_t(batch) * OZ_S * ((m + OZ_BM - 1) / OZ_BM * OZ_BM) < (int64_t(1) << 31) &&
                      int64_t(batch) * OZ_S * ((n + OZ_BN - 1) / OZ_BN * OZ_BN) < (int64_t(1) << 31),
                  "gemm_oz: operand too large");
  OzLayout L;
  const size_t need = oz_layout(m, n, k, batch, nsplit, ws, &L);
  if (!ws || ws_bytes < need) {
    set_error("gemm_oz: workspace %zu bytes < required %zu", ws_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  // op(A)(i, kk): ta ? A[kk lda + i] : A[i lda + kk];  op(B) column j: tb ? B[j ldb + kk] : B[kk ldb + j]
  const int64_t a_rs = ta ? 1 : lda, a_ks = ta ? lda : 1;
  const int64_t b_rs = tb ? ldb : 1, b_ks = tb ? 1 : ldb;
  dim3 tb2(32, 8);
  // row maxima (atomicMax into zeroed arrays) and the error flag: ea, eb and flag are consecutive
  TNX_CUDA(cudaMemsetAsync(L.ea, 0, reinterpret_cast<char*>(L.flag + 1) - reinterpret_cast<char*>(L.ea), st));
  const unsigned kscan = unsigned((k + OZ_SCAN_K - 1) / OZ_SCAN_K), bzs = unsigned(batch);
  oz_rowmax_kernel<<<dim3(kscan, unsigned(L.Mp / 32), bzs), tb2, 0, st>>>(A, m, k, a_rs, a_ks, L.ea, sA, L.Mp, mask);
  TNX_LAUNCH_CHECK();
  oz_rowmax_kernel<<<dim3(kscan, unsigned(L.Np / 32), bzs), tb2, 0, st>>>(B, n, k, b_rs, b_ks, L.eb, sB, L.Np, mask);
  TNX_LAUNCH_CHECK();
  oz_slice_kernel<<<dim3(unsigned(L.Kp / 32), unsigned(L.Mp / 32), bzs), tb2, 0, st>>>(A, m, k, a_rs, a_ks, L.ea,
                                                                                        L.sa, L.Mp, L.Kp, sA, mask);
  TNX_LAUNCH_CHECK();
  oz_slice_kernel<<<dim3(unsigned(L.Kp / 32), unsigned(L.Np / 32), bzs), tb2, 0, st>>>(B, n, k, b_rs, b_ks, L.eb,
                                                                                        L.sb, L.Np, L.Kp, sB, mask);
  TNX_LAUNCH_CHECK();
  CUtensorMap ma, mb;
  TNX_TRY(make_tma_map_bf16(&ma, L.sa, int64_t(batch) * OZ_S * L.Mp, L.Kp, OZ_BK, OZ_BM));
  TNX_TRY(make_tma_map_bf16(&mb, L.sb, int64_t(batch) * OZ_S * L.Np, L.Kp, OZ_BK, OZ_BN));
  const size_t smem = oz_smem_bytes();
  static std::atomic<bool> attr{false};  // idempotent setup; threads may race to it
  if (!attr.load()) {
    TNX_CUDA(cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    attr.store(true);
  }
  const int kb_all = int(L.Kp / OZ_BK);
  const int kbs = (kb_all + nsplit - 1) / nsplit;
  nsplit = (kb_all + kbs - 1) / kbs;  // no empty splits
  dim3 grid(unsigned(L.Np / OZ_BN), unsigned(L.Mp / OZ_BM), unsigned(batch * nsplit));
  // profiler family: the large products (environment updates, anchor matvecs, the gauge move's
  // X, Q and R A) apart from the narrow ones (a side of 128 or less, split K, batches)
  const int fam = (nsplit > 1 || batch > 1 || m <= 128 || n <= 128 || k <= 128) ? KF_OZ_NARROW : KF_OZ_GEMM;
  profile_mark(fam, st, true);
  oz_gemm_kernel<<<grid, OZ_THREADS, smem, st>>>(ma, mb, int(m), int(n), int(L.Kp), int(L.Mp), int(L.Np), L.ea, L.eb,
                                                 alpha, beta, C, ldc, L.flag, batch, nsplit, kbs, sC, L.part, mask);
  TNX_LAUNCH_CHECK();
  if (nsplit > 1) {
    const int64_t mn = m * n;
    const unsigned gx = unsigned(std::min<int64_t>((mn + 255) / 256, 64));
    oz_split_reduce_kernel<<<dim3(gx, unsigned(batch)), 256, 0, st>>>(L.part, nsplit, batch, int(m), int(n), alpha,
                                                                      beta, C, ldc, sC, mask);
    TNX_LAUNCH_CHECK();
  }
  profile_mark(fam, st, false);
  profile_work(fam, 2.0 * double(m) * n * k * batch, 8.0 * batch * (double(m) * k + double(k) * n + double(m) * n));
  return TNX_OK;
}

int gemm_oz(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
            const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* ws, size_t ws_bytes,
            cudaStream_t st) {
  return gemm_oz_ex(ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1, 1, nullptr, ws, ws_bytes, st);
}

int gemm_oz_flag(void* ws, int64_t m, int64_t n, int64_t k, int** flag) {
  OzLayout L;
  oz_layout(m, n, k, 1, 1, ws, &L);
  *flag = L.flag;
  return TNX_OK;
}

}  // namespace tnx

using namespace tnx;

extern "C" {

size_t tnx_gemm_oz_workspace_bytes(int64_t m, int64_t n, int64_t k) { return gemm_oz_workspace_bytes(m, n, k); }

int tnx_gemm_oz(int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
                const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* workspace,
                size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(A && B && C, "null pointer");
  TNX_CHECK_ARG(m >= 0 && n >= 0 && k >= 0, "negative size");
  cudaStream_t st = as_stream(stream);
  TNX_TRY(gemm_oz(trans_a != 0, trans_b != 0, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, workspace,
                  workspace_bytes, st));
  // a bounded wait that expired inside the kernel is reported here (one 4-byte read)
  int* flag = nullptr;
  gemm_oz_flag(workspace, m, n, k, &flag);
  int h = 0;
  TNX_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  TNX_CUDA(cudaStreamSynchronize(st));
  if (h) {
    set_error("tnx_gemm_oz: a bounded wait in the tensor-core kernel expired");
    return TNX_ERR_TIMEOUT;
  }
  return TNX_OK;
}

size_t tnx_gemm_oz_batched_workspace_bytes(int64_t m, int64_t n, int64_t k, int batch, int nsplit) {
  return gemm_oz_ex_workspace_bytes(m, n, k, batch < 1 ? 1 : batch, nsplit < 1 ? 1 : nsplit);
}

int tnx_gemm_oz_batched(int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                        int64_t lda, int64_t sA, const double* B, int64_t ldb, int64_t sB, double beta, double* C,
                        int64_t ldc, int64_t sC, int batch, int nsplit, const int* mask, void* workspace,
                        size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(A && B && C, "null pointer");
  TNX_CHECK_ARG(m >= 0 && n >= 0 && k >= 0 && batch >= 1 && nsplit >= 1, "negative size, batch or split");
  cudaStream_t st = as_stream(stream);
  TNX_TRY(gemm_oz_ex(trans_a != 0, trans_b != 0, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch,
                     nsplit, mask, workspace, workspace_bytes, st));
  int* flag = nullptr;
  OzLayout L;
  oz_layout(m, n, k, batch, nsplit, workspace, &L);
  flag = L.flag;
  int h = 0;
  TNX_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  TNX_CUDA(cudaStreamSynchronize(st));
  if (h) {
    set_error("tnx_gemm_oz_batched: a bounded wait in the tensor-core kernel expired");
    return TNX_ERR_TIMEOUT;
  }
  return TNX_OK;
}

}  // extern "C"
