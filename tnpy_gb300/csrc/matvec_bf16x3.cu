// Split-BF16 ("bf16x3") one-site matvec on the tcgen05 tensor cores.
//
// Each FP64 operand X is split into X_hi = bf16(X) and X_lo = bf16(X - X_hi); a product is
// taken as A_hi B_hi + A_hi B_lo + A_lo B_hi with FP32 accumulation in tensor memory, i.e.
// one BF16 GEMM over a K dimension three times as long. Relative error ~2^-16 per product.
//
// The matvec y = H_eff x of Environment.one_site_matvec (tnpy/matrix_product_state.py:411-440)
// is three steps:
//   1. T1[(w,a'),(s,c)] = sum_a L[a,(w,a')] x[a,(s,c)]        tensor cores, K = chi_l
//   2. T2[(a',s'),(c,v)] = sum_{w,s} T1 W[w,v,s,s']            CUDA cores, K = D*d, writes the
//                                                              split BF16 operand of step 3
//   3. y[(a',s'),c'] = sum_{(c,v)} T2 R[(c,v),c']             tensor cores, K = chi_r*D
// L and R are re-laid out once per site as K-major split operands (Davidson reuses them for
// every matvec of the site); x is re-laid out per matvec.
//
// GEMM kernel: one 128 x BN output tile per CTA, 6 warps:
//   warp 0  TMA producer (cp.async.bulk.tensor, 128B swizzle, 64-wide K slabs, 4-stage ring)
//   warp 1  TMEM allocation + single-thread tcgen05.mma issue (kind::f16, BF16 in, FP32 acc)
//   warps 2-5 epilogue: tcgen05.ld of the FP32 accumulator, staged through shared memory in
//             64-column chunks, stored as FP32 or FP64 row segments
// Every mbarrier wait is bounded (~2 s of clock); on expiry the kernel raises a flag in
// global memory, stops issuing work, waits (bounded) for its own TMA copies and frees TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstring>

#include <atomic>

#include "tc_ptx.cuh"
#include "tnx_internal.cuh"

namespace tnx {
namespace {

using namespace tc;

constexpr int BM = 128;
constexpr int BK = 64;  // 64 bf16 = 128 bytes = one swizzle atom row
constexpr int STAGES = 4;
constexpr int GEMM_THREADS = 192;

// ---------------------------------------------------------------- GEMM kernel
// C[M, N] = sum_k A[m, k] B[n, k] over the three split products; A*, B* are K-major BF16
// with row pitch Kp (a multiple of 64). out: FP32 or FP64, row-major with leading dim ldc.
template <int BN>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    bf16x3_gemm_kernel(const __grid_constant__ CUtensorMap ta_hi, const __grid_constant__ CUtensorMap ta_lo,
                       const __grid_constant__ CUtensorMap tb_hi, const __grid_constant__ CUtensorMap tb_lo,
                       int M, int N, int Kp, void* __restrict__ out, int64_t ldc, int out_fp64,
                       int* __restrict__ err_flag) {
  constexpr uint32_t A_BYTES = BM * BK * 2;
  constexpr uint32_t B_BYTES = BN * BK * 2;
  constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
  constexpr uint32_t TMEM_COLS = BN < 32 ? 32 : BN;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[STAGES], empty_bar[STAGES], accum_bar;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh, epi_fail_sh;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int kblocks = Kp / BK;
  const int total = 3 * kblocks;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&accum_bar), 1);
    abort_sh = 0;
    epi_fail_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base_sh;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      int issued = 0;
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (it >= STAGES && !mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1)) {
          atomicExch(err_flag, 1);
          abort_sh = 1;
          break;
        }
        if (*((volatile int*)&abort_sh)) break;
        const int seg = it / kblocks, kb = it % kblocks;
        const CUtensorMap* ma = seg == 2 ? &ta_lo : &ta_hi;
        const CUtensorMap* mb = seg == 1 ? &tb_lo : &tb_hi;
        const uint32_t sa = base + s * STAGE_BYTES, sb = sa + A_BYTES;
        const uint32_t fb = smem_u32(&full_bar[s]);
        mbar_expect_tx(fb, STAGE_BYTES);
        tma_load_2d(sa, ma, fb, kb * BK, m0);
        tma_load_2d(sb, mb, fb, kb * BK, n0);
        ++issued;
      }
      // drain: wait (bounded) until every issued copy has landed before the CTA can exit
      for (int it = issued - STAGES < 0 ? 0 : issued - STAGES; it < issued; ++it)
        mbar_wait(smem_u32(&full_bar[it % STAGES]), (it / STAGES) & 1);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = instr_desc_bf16(BM, BN);
      bool ok = true;
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!mbar_wait(smem_u32(&full_bar[s]), ph) || *((volatile int*)&abort_sh)) {
          atomicExch(err_flag, 1);
          abort_sh = 1;
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t sa = base + s * STAGE_BYTES, sb = sa + A_BYTES;
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
          const uint64_t ad = smem_desc_sw128(sa + kk * 32);
          const uint64_t bd = smem_desc_sw128(sb + kk * 32);
          mma_bf16(tmem, ad, bd, idesc, (it > 0 || kk > 0) ? 1u : 0u);
        }
        mma_commit(smem_u32(&empty_bar[s]));
      }
      if (ok) mma_commit(smem_u32(&accum_bar));
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2..5)
    // The accumulator goes out in 64-column chunks through shared memory (the stage ring is free
    // once the accumulator is complete): a thread holds one row of the tile in TMEM, and storing
    // from there would write 32 rows per warp instruction; from shared memory every warp store
    // covers 32 consecutive columns of one row.
    const int quad = warp & 3;  // TMEM lanes 32*quad .. 32*quad+31
    const int lr = quad * 32 + lane, et = threadIdx.x - 64;
    const bool ok = mbar_wait(smem_u32(&accum_bar), 0);
    if (!ok) {
      if (lane == 0) atomicExch(err_flag, 1);
      epi_fail_sh = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    constexpr int CW = 64;  // columns per chunk; the FP64 chunk [BM][CW + 1] is 66.5 KB
    uint8_t* stg = smem_raw + (base - smem_u32(smem_raw));
    float* sf = reinterpret_cast<float*>(stg);
    double* sd = reinterpret_cast<double*>(stg);
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += CW) {
      if (ok) {
        uint32_t r[2][32];
        tmem_ld32_async(tmem + (uint32_t(quad * 32) << 16) + uint32_t(c0), r[0]);
        tmem_ld32_async(tmem + (uint32_t(quad * 32) << 16) + uint32_t(c0 + 32), r[1]);
        tmem_ld_wait();
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            if (out_fp64) sd[lr * (CW + 1) + h * 32 + j] = double(__uint_as_float(r[h][j]));
            else sf[lr * (CW + 1) + h * 32 + j] = __uint_as_float(r[h][j]);
          }
      }
      asm volatile("bar.sync 1, 128;" ::: "memory");  // the four epilogue warps
      if (!epi_fail_sh) {
        for (int idx = et; idx < BM * CW; idx += 128) {
          const int rr = idx / CW, cc = idx % CW;
          if (m0 + rr < M && n0 + c0 + cc < N) {
            const int64_t o = int64_t(m0 + rr) * ldc + n0 + c0 + cc;
            if (out_fp64) static_cast<double*>(out)[o] = sd[rr * (CW + 1) + cc];
            else static_cast<float*>(out)[o] = sf[rr * (CW + 1) + cc];
          }
        }
      }
      asm volatile("bar.sync 1, 128;" ::: "memory");  // the chunk is out before the next one is staged
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// ---------------------------------------------------------------- operand preparation
// dst_hi/lo[c][r] (row pitch ldp) = split(src[r][c]) for r < rows; zeros for rows <= r < ldp.
// src is row-major rows x cols (FP64).
template <typename T>
__global__ void split_transpose_kernel(const T* __restrict__ src, int64_t rows, int64_t cols,
                                       __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                       int64_t ldp) {
  __shared__ double tile[32][33];
  const int64_t r0 = int64_t(blockIdx.y) * 32, c0 = int64_t(blockIdx.x) * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = r0 + k, c = c0 + threadIdx.x;
    tile[k][threadIdx.x] = (r < rows && c < cols) ? double(src[r * cols + c]) : 0.0;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t c = c0 + k, r = r0 + threadIdx.x;
    if (c < cols && r < ldp) {
      const double v = tile[threadIdx.x][k];
      const __nv_bfloat16 h = __double2bfloat16(v);
      hi[c * ldp + r] = h;
      lo[c * ldp + r] = __double2bfloat16(v - double(__bfloat162float(h)));
    }
  }
}

// T2 split operand: A3[(a',s')][(c,v)] (row pitch ldp) from T1 (FP32, [(w,a')][(s,c)]).
__global__ void wcontract_split_kernel(const float* __restrict__ T1, const double* __restrict__ W,
                                       __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                       int64_t chi_l, int d, int64_t chi_r, int dl, int dr, int64_t ldp) {
  extern __shared__ float wsf[];
  const int wn = dl * dr * d * d;
  for (int i = threadIdx.x; i < wn; i += blockDim.x) wsf[i] = float(W[i]);
  __syncthreads();
  const int64_t total = chi_l * chi_r;
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t ap = idx / chi_r, c = idx % chi_r;
    float in[64];
    for (int w = 0; w < dl; ++w)
      for (int s = 0; s < d; ++s) in[w * d + s] = T1[((w * chi_l + ap) * d + s) * chi_r + c];
    for (int sp = 0; sp < d; ++sp) {
      const int64_t o = (ap * d + sp) * ldp + c * dr;
      for (int v = 0; v < dr; ++v) {
        float acc = 0.f;
        for (int w = 0; w < dl; ++w)
          for (int s = 0; s < d; ++s) acc = fmaf(in[w * d + s], wsf[((w * dr + v) * d + s) * d + sp], acc);
        const __nv_bfloat16 h = __float2bfloat16_rn(acc);
        hi[o + v] = h;
        lo[o + v] = __float2bfloat16_rn(acc - __bfloat162float(h));
      }
    }
  }
}

// dst_hi/lo[r][c] (row pitch ldp) = split(src[r][c]), zeros for cols <= c < ldp
__global__ void split_pad_kernel(const double* __restrict__ src, int64_t rows, int64_t cols,
                                 __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, int64_t ldp) {
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < rows * ldp;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = e / ldp, c = e % ldp;
    const double v = c < cols ? src[r * cols + c] : 0.0;
    const __nv_bfloat16 h = __double2bfloat16(v);
    hi[e] = h;
    lo[e] = __double2bfloat16(v - double(__bfloat162float(h)));
  }
}

// zero the padding columns [k0, ldp) of a rows x ldp bf16 pair
__global__ void zero_pad_kernel(__nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, int64_t rows,
                                int64_t k0, int64_t ldp) {
  const int64_t w = ldp - k0;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < rows * w;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = e / w, c = k0 + e % w;
    hi[r * ldp + c] = __float2bfloat16_rn(0.f);
    lo[r * ldp + c] = __float2bfloat16_rn(0.f);
  }
}

// ---------------------------------------------------------------- host side
// 2-D map over a K-major bf16 matrix rows x ldp (K innermost), box {64, box_rows}, 128B swizzle
int make_map(CUtensorMap* map, const void* ptr, int64_t rows, int64_t ldp, int box_rows) {
  return make_tma_map_bf16(map, ptr, rows, ldp, BK, box_rows);
}

template <int BN>
size_t gemm_smem_bytes() {
  return size_t(STAGES) * (BM * BK * 2 + BN * BK * 2) + 1024;
}

template <int BN>
int launch_gemm(const __nv_bfloat16* a_hi, const __nv_bfloat16* a_lo, const __nv_bfloat16* b_hi,
                const __nv_bfloat16* b_lo, int M, int N, int Kp, void* out, int64_t ldc, bool out_fp64,
                int* err_flag, cudaStream_t st, int64_t k_real = -1) {
  CUtensorMap mah, mal, mbh, mbl;
  TNX_TRY(make_map(&mah, a_hi, M, Kp, BM));
  TNX_TRY(make_map(&mal, a_lo, M, Kp, BM));
  TNX_TRY(make_map(&mbh, b_hi, N, Kp, BN));
  TNX_TRY(make_map(&mbl, b_lo, N, Kp, BN));
  const size_t smem = gemm_smem_bytes<BN>();
  static std::atomic<bool> attr_set{false};  // idempotent setup; threads may race to it
  if (!attr_set.load()) {
    TNX_CUDA(cudaFuncSetAttribute(bf16x3_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    attr_set.store(true);
  }
  dim3 grid(unsigned((N + BN - 1) / BN), unsigned((M + BM - 1) / BM));
  profile_mark(KF_TC_GEMM, st, true);
  bf16x3_gemm_kernel<BN><<<grid, GEMM_THREADS, smem, st>>>(mah, mal, mbh, mbl, M, N, Kp, out, ldc,
                                                           out_fp64 ? 1 : 0, err_flag);
  profile_mark(KF_TC_GEMM, st, false);
  // algorithmic work: one product of the unsplit operands (2 M N K flops)
  profile_work(KF_TC_GEMM, 2.0 * M * N * double(k_real < 0 ? Kp : k_real),
               2.0 * 2.0 * (double(M) + N) * Kp * 3 + double(M) * N * (out_fp64 ? 8 : 4));
  TNX_LAUNCH_CHECK();
  return TNX_OK;
}

inline int64_t pad64(int64_t k) { return (k + 63) / 64 * 64; }

struct MixedLayout {
  int64_t K1p, K3p, M1, N1, M3, N3;
  __nv_bfloat16 *a1h, *a1l, *b1h, *b1l, *a3h, *a3l, *b3h, *b3l;
  float* T1;
  int* flag;
};

size_t mixed_layout(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, void* base, MixedLayout* L) {
  MixedLayout m;
  m.K1p = pad64(chi_l);
  m.K3p = pad64(chi_r * dr);
  m.M1 = dl * chi_l;
  m.N1 = d * chi_r;
  m.M3 = chi_l * d;
  m.N3 = chi_r;
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += align_up(bytes, 1024); return o; };
  size_t o1 = take(m.M1 * m.K1p * 2), o2 = take(m.M1 * m.K1p * 2), o3 = take(m.N1 * m.K1p * 2),
         o4 = take(m.N1 * m.K1p * 2), o5 = take(m.M3 * m.K3p * 2), o6 = take(m.M3 * m.K3p * 2),
         o7 = take(m.N3 * m.K3p * 2), o8 = take(m.N3 * m.K3p * 2), o9 = take(m.M1 * m.N1 * 4), o10 = take(256);
  if (base && L) {
    char* b = static_cast<char*>(base);
    m.a1h = reinterpret_cast<__nv_bfloat16*>(b + o1);
    m.a1l = reinterpret_cast<__nv_bfloat16*>(b + o2);
    m.b1h = reinterpret_cast<__nv_bfloat16*>(b + o3);
    m.b1l = reinterpret_cast<__nv_bfloat16*>(b + o4);
    m.a3h = reinterpret_cast<__nv_bfloat16*>(b + o5);
    m.a3l = reinterpret_cast<__nv_bfloat16*>(b + o6);
    m.b3h = reinterpret_cast<__nv_bfloat16*>(b + o7);
    m.b3l = reinterpret_cast<__nv_bfloat16*>(b + o8);
    m.T1 = reinterpret_cast<float*>(b + o9);
    m.flag = reinterpret_cast<int*>(b + o10);
    *L = m;
  }
  return off + 1024;  // slack for aligning the base
}

void* align1024(void* p) {
  return reinterpret_cast<void*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

dim3 tgrid(int64_t rows, int64_t cols) {
  return dim3(unsigned((cols + 31) / 32), unsigned((rows + 31) / 32));
}

}  // namespace

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeFn get_encode() {
  static EncodeFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<EncodeFn>(p);
    return static_cast<EncodeFn>(nullptr);
  }();
  return fn;
}

int make_tma_map_bf16(CUtensorMap* map, const void* ptr, int64_t rows, int64_t ldp, int box_k, int box_rows) {
  EncodeFn enc = get_encode();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled unavailable");
    return TNX_ERR_CUDA;
  }
  if ((reinterpret_cast<uintptr_t>(ptr) & 15) != 0 || (ldp * 2) % 16 != 0 || (box_k != 64 && box_k != 32)) {
    set_error("TMA operand misaligned");
    return TNX_ERR_INVALID_ARG;
  }
  cuuint64_t dims[2] = {cuuint64_t(ldp), cuuint64_t(rows)};
  cuuint64_t strides[1] = {cuuint64_t(ldp * 2)};
  cuuint32_t box[2] = {cuuint32_t(box_k), cuuint32_t(box_rows)};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, box_k == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", int(r));
    return TNX_ERR_CUDA;
  }
  return TNX_OK;
}

bool mixed_supported(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr) {
  return chi_l >= 16 && chi_r >= 16 && dl * d <= 64 && dr * d <= 64 && dl * chi_l < (1 << 30);
}

size_t matvec1_bf16x3_scratch_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr) {
  return mixed_layout(chi_l, d, chi_r, dl, dr, nullptr, nullptr);
}

// Per-site preparation: split + transpose L and R, zero the padding of the T2 operand.
int mixed_prepare(const double* L, const double* R, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                  void* scratch, cudaStream_t st) {
  MixedLayout m;
  mixed_layout(chi_l, d, chi_r, dl, dr, align1024(scratch), &m);
  dim3 tb(32, 8);
  // A1[(w a')][a] = L[a][(w a')]: src rows = chi_l, cols = dl*chi_l, pitch K1p
  split_transpose_kernel<double><<<tgrid(m.K1p, m.M1), tb, 0, st>>>(L, chi_l, m.M1, m.a1h, m.a1l, m.K1p);
  TNX_LAUNCH_CHECK();
  // B3[c'][(c v)] = R[(c v)][c']: src rows = chi_r*dr, cols = chi_r, pitch K3p
  split_transpose_kernel<double><<<tgrid(m.K3p, m.N3), tb, 0, st>>>(R, chi_r * dr, chi_r, m.b3h, m.b3l, m.K3p);
  TNX_LAUNCH_CHECK();
  if (m.K3p > chi_r * dr) {
    zero_pad_kernel<<<152, 256, 0, st>>>(m.a3h, m.a3l, m.M3, chi_r * dr, m.K3p);
    TNX_LAUNCH_CHECK();
  }
  TNX_CUDA(cudaMemsetAsync(m.flag, 0, sizeof(int), st));
  return TNX_OK;
}

// One matvec with prepared L / R operands; x and y FP64 or FP32 (T).
template <typename T>
int mixed_apply_t(const double* W, const T* x, T* y, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                  int64_t dr, void* scratch, cudaStream_t st) {
  MixedLayout m;
  mixed_layout(chi_l, d, chi_r, dl, dr, align1024(scratch), &m);
  dim3 tb(32, 8);
  // B1[(s c)][a] = x[a][(s c)]
  split_transpose_kernel<T><<<tgrid(m.K1p, m.N1), tb, 0, st>>>(x, chi_l, m.N1, m.b1h, m.b1l, m.K1p);
  TNX_LAUNCH_CHECK();
  // step 1: T1 (FP32) = A1 . B1^T; 128 x 256 or 128 x 128 tiles, autotuned per shape
  {
    auto run = [&](int v) -> int {
      if (v == 0)
        return launch_gemm<256>(m.a1h, m.a1l, m.b1h, m.b1l, int(m.M1), int(m.N1), int(m.K1p), m.T1, m.N1, false,
                                m.flag, st, chi_l);
      return launch_gemm<128>(m.a1h, m.a1l, m.b1h, m.b1l, int(m.M1), int(m.N1), int(m.K1p), m.T1, m.N1, false,
                              m.flag, st, chi_l);
    };
    TNX_TRY(autotuned(TuneKey{3, m.M1, m.N1, m.K1p, 0, 0}, 2, m.N1 >= 256 ? 0 : 1, m.N1 >= 256, st, run));
  }
  // step 2: MPO contraction into the split A3 operand
  {
    int64_t total = chi_l * chi_r;
    int64_t blocks = (total + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    size_t smem = size_t(dl * dr * d * d) * sizeof(float);
    wcontract_split_kernel<<<unsigned(blocks), 128, smem, st>>>(m.T1, W, m.a3h, m.a3l, chi_l, int(d), chi_r,
                                                                 int(dl), int(dr), m.K3p);
    TNX_LAUNCH_CHECK();
  }
  // step 3: y = A3 . B3^T (FP32 accumulators written as T); tiles autotuned per shape
  {
    auto run = [&](int v) -> int {
      if (v == 0)
        return launch_gemm<256>(m.a3h, m.a3l, m.b3h, m.b3l, int(m.M3), int(m.N3), int(m.K3p), y, m.N3,
                                sizeof(T) == 8, m.flag, st, chi_r * dr);
      return launch_gemm<128>(m.a3h, m.a3l, m.b3h, m.b3l, int(m.M3), int(m.N3), int(m.K3p), y, m.N3,
                              sizeof(T) == 8, m.flag, st, chi_r * dr);
    };
    TNX_TRY(autotuned(TuneKey{3, m.M3, m.N3, m.K3p, int64_t(sizeof(T)), 0}, 2, 1, m.N3 >= 256, st, run));
  }
  return TNX_OK;
}

int mixed_apply(const double* W, const double* x, double* y, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                int64_t dr, void* scratch, cudaStream_t st) {
  return mixed_apply_t<double>(W, x, y, chi_l, d, chi_r, dl, dr, scratch, st);
}

int mixed_apply_f32(const double* W, const float* x, float* y, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                    int64_t dr, void* scratch, cudaStream_t st) {
  return mixed_apply_t<float>(W, x, y, chi_l, d, chi_r, dl, dr, scratch, st);
}

int mixed_flag(void* scratch, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, int** flag) {
  MixedLayout m;
  mixed_layout(chi_l, d, chi_r, dl, dr, align1024(scratch), &m);
  *flag = m.flag;
  return TNX_OK;
}

int matvec1_bf16x3(const double* L, const double* W, const double* R, const double* x, double* y, int64_t chi_l,
                   int64_t d, int64_t chi_r, int64_t dl, int64_t dr, void* scratch, size_t scratch_bytes,
                   cudaStream_t st) {
  if (!mixed_supported(chi_l, d, chi_r, dl, dr)) {
    set_error("split-BF16 matvec needs chi_l, chi_r >= 16 (got %lld, %lld)", (long long)chi_l, (long long)chi_r);
    return TNX_ERR_UNSUPPORTED;
  }
  if (scratch_bytes < matvec1_bf16x3_scratch_bytes(chi_l, d, chi_r, dl, dr) || !scratch) {
    set_error("split-BF16 matvec: scratch too small");
    return TNX_ERR_WORKSPACE;
  }
  TNX_TRY(mixed_prepare(L, R, chi_l, d, chi_r, dl, dr, scratch, st));
  return mixed_apply(W, x, y, chi_l, d, chi_r, dl, dr, scratch, st);
}


}  // namespace tnx

using namespace tnx;

extern "C" {

size_t tnx_gemm_bf16x3_workspace_bytes(int64_t m, int64_t n, int64_t k) {
  const int64_t kp = pad64(k);
  return 2 * align_up(size_t(m * kp * 2), 1024) + 2 * align_up(size_t(n * kp * 2), 1024) + 2048;
}

int tnx_gemm_bf16x3(int64_t m, int64_t n, int64_t k, const double* A, const double* B, double* C,
                    void* workspace, size_t workspace_bytes, void* stream) {
  TNX_CHECK_ARG(A && B && C, "null pointer");
  TNX_CHECK_ARG(m > 0 && n > 0 && k > 0, "non-positive size");
  TNX_CHECK_SHAPE(m < (1 << 30) && n < (1 << 30) && k < (1 << 28), "size too large");
  size_t need = tnx_gemm_bf16x3_workspace_bytes(m, n, k);
  if (workspace_bytes < need || !workspace) {
    set_error("tnx_gemm_bf16x3: workspace %zu bytes < required %zu", workspace_bytes, need);
    return TNX_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  const int64_t kp = pad64(k);
  char* b = static_cast<char*>(align1024(workspace));
  auto* ah = reinterpret_cast<__nv_bfloat16*>(b);
  auto* al = reinterpret_cast<__nv_bfloat16*>(b + align_up(size_t(m * kp * 2), 1024));
  auto* bh = reinterpret_cast<__nv_bfloat16*>(b + 2 * align_up(size_t(m * kp * 2), 1024));
  auto* bl = reinterpret_cast<__nv_bfloat16*>(b + 2 * align_up(size_t(m * kp * 2), 1024) +
                                              align_up(size_t(n * kp * 2), 1024));
  int* flag = reinterpret_cast<int*>(b + 2 * align_up(size_t(m * kp * 2), 1024) +
                                     2 * align_up(size_t(n * kp * 2), 1024));
  TNX_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
  split_pad_kernel<<<152 * 4, 256, 0, st>>>(A, m, k, ah, al, kp);
  TNX_LAUNCH_CHECK();
  split_pad_kernel<<<152 * 4, 256, 0, st>>>(B, n, k, bh, bl, kp);
  TNX_LAUNCH_CHECK();
  if (n >= 256)
    TNX_TRY(launch_gemm<256>(ah, al, bh, bl, int(m), int(n), int(kp), C, n, true, flag, st, k));
  else
    TNX_TRY(launch_gemm<128>(ah, al, bh, bl, int(m), int(n), int(kp), C, n, true, flag, st, k));
  int host_flag = 0;
  TNX_CUDA(cudaMemcpyAsync(&host_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  TNX_CUDA(cudaStreamSynchronize(st));
  if (host_flag) {
    set_error("tnx_gemm_bf16x3: a bounded device wait expired");
    return TNX_ERR_TIMEOUT;
  }
  return TNX_OK;
}

}  // extern "C"
