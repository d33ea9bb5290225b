// Double-FP32 cluster panel of the Householder QR, for the FP64-class precision modes.
//
// Same algorithm as the FP64 cluster panel in qr.cu (rows of the panel split over the CTAs of
// one thread-block cluster, one cluster barrier per column, exchange of partial sums through
// distributed shared memory, LAPACK dgeqr2 reflectors and the forward/columnwise dlarft T
// factor), with every per-element operation in double-FP32 arithmetic on the FP32 pipe. On
// this part the FP64 pipe issues about 2 FMA per clock per SM against 128 for FP32, and in the
// FP64 kernel the per-column update of the remaining panel columns is bound by it.
//
// Numbers are (hi, lo) float pairs (relative error ~2^-47 per operation, the standard model
// with u ~ 2^-47, so the factorisation stays backward stable at that level). The layout and
// schedule are chosen for short dependency chains on the FP32 pipe:
//   * 512 threads, 8 per panel column interleaved over rows, two independent accumulators,
//     (hi, lo) pairs interleaved in shared memory;
//     dot products accumulate compensated (hi, lo) sums renormalised once at the end;
//   * the CL partial sums of a column are added as a fixed binary tree (every CTA derives
//     bitwise-identical column scalars);
//   * the column scalars use 1 / norm from an rsqrtf seed refined by Newton steps in
//     double-FP32 (tau = 1 + |alpha| / norm needs no division; scale = sign / (norm tau) one
//     refined reciprocal), not FP64 square root and division;
//   * the T factor is distributed: CTA q extends rows a = q (mod CL) of T, so no CTA carries
//     a serial triangular product on the critical path.
// Columns are scaled by powers of two at load (largest entry of each panel column near 2^32)
// so that squares and products of small entries stay inside the FP32 exponent range; QR of
// A D with D a power-of-two diagonal has the same reflectors and R D, so R entries are
// rescaled on store and reflectors, tau and T are unaffected.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>

#ifdef TNX_PANEL_PROBE
#define PANEL_STAMP(k) \
  if (threadIdx.x == 0 && stamps) stamps[(q * 64 + jj) * 8 + (k)] = clock64()
#else
#define PANEL_STAMP(k)
#endif

namespace tnx {
namespace qrdf {

namespace cg = cooperative_groups;

constexpr int DPT = 512;  // threads per CTA

struct df2 {
  float h, l;
};

// Error-free transformations with explicit roundings (no contraction into FMA, no reassociation)
__device__ __forceinline__ df2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df2 fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df2 add(df2 x, df2 y) {
  const df2 s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(x.l, y.l)));
}
__device__ __forceinline__ df2 neg(df2 x) { return {-x.h, -x.l}; }
__device__ __forceinline__ df2 mul(df2 x, df2 y) {
  const float p = __fmul_rn(x.h, y.h);
  float e = fmaf(x.h, y.h, -p);
  e = fmaf(x.h, y.l, e);
  e = fmaf(x.l, y.h, e);
  return fast_two_sum(p, e);
}
// x - w v
__device__ __forceinline__ df2 fms(df2 x, df2 w, df2 v) {
  const float p = __fmul_rn(w.h, v.h);
  float pe = fmaf(w.h, v.h, -p);
  pe = fmaf(w.h, v.l, pe);
  pe = fmaf(w.l, v.h, pe);
  const df2 s = two_sum(x.h, -p);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fsub_rn(x.l, pe)));
}
// c += a b with c.l left unnormalised (long sums; renormalise with two_sum(c.h, c.l))
__device__ __forceinline__ void acc(df2& c, df2 a, df2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float pe = fmaf(a.h, b.h, -p);
  pe = fmaf(a.h, b.l, pe);
  pe = fmaf(a.l, b.h, pe);
  const df2 s = two_sum(c.h, p);
  c.h = s.h;
  c.l = __fadd_rn(c.l, __fadd_rn(s.l, pe));
}
__device__ __forceinline__ df2 norm(df2 c) { return two_sum(c.h, c.l); }
// 1 / sqrt(t), t > 0: rsqrtf seed, two Newton steps y += y (1 - t y^2) / 2 on the
// double-FP32 residual (seed error ~2^-22 -> ~2^-44 -> the format's ~2^-47)
__device__ __forceinline__ df2 rsqrt_df(df2 t) {
  df2 y = {rsqrtf(t.h), 0.f};
  for (int it = 0; it < 2; ++it) {
    const df2 e = fms({1.f, 0.f}, t, mul(y, y));
    y = add(y, {__fmul_rn(__fmul_rn(0.5f, y.h), e.h), 0.f});
  }
  return y;
}
// 1 / b: approximate FP32 reciprocal seed, two Newton steps z += z (1 - b z)
__device__ __forceinline__ df2 rcp_df(df2 b) {
  df2 z = {__fdividef(1.f, b.h), 0.f};
  for (int it = 0; it < 2; ++it) {
    const df2 e = fms({1.f, 0.f}, b, z);
    z = add(z, {__fmul_rn(z.h, e.h), 0.f});
  }
  return z;
}
__device__ __forceinline__ df2 shfl_xor(df2 x, int o) {
  return {__shfl_xor_sync(0xffffffffu, x.h, o), __shfl_xor_sync(0xffffffffu, x.l, o)};
}

// double (exponent lowered by e: x 2^-e, exact) -> (hi, lo); Inf and NaN stay non-finite
// (split_df gives (+-inf, 0) / (NaN, 0)) so that they propagate through the factorisation
__device__ __forceinline__ df2 split_scaled(double x, int e) {
  long long b = __double_as_longlong(x);
  const int ef = int((b >> 52) & 0x7ff);
  if (ef == 2047) {
    df2 r;
    split_df(x, r.h, r.l);
    return r;
  }
  if (ef == 0) {  // zero / subnormal (below 2^-1022: far below the split's range)
    b &= (1LL << 63);
  } else if (ef - e <= 0) {
    b &= (1LL << 63);
  } else {
    b -= (long long)e << 52;
  }
  df2 r;
  split_df(__longlong_as_double(b), r.h, r.l);
  return r;
}
// (hi, lo) -> double x 2^e
__device__ __forceinline__ double join_scaled(df2 x, int e) {
  const double d = join_df(x.h, x.l);
  long long b = __double_as_longlong(d);
  const int ef = int((b >> 52) & 0x7ff);
  if (ef == 0 || e == 0) return d;
  const int ne = ef + e;
  if (ne >= 2047) return __longlong_as_double((b & (1LL << 63)) | (0x7ffLL << 52));
  if (ne <= 0) return __longlong_as_double(b & (1LL << 63));
  return __longlong_as_double(b + ((long long)e << 52));
}

__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
  asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory");
}

// Sum of the CL partials slot(rank)[idx] over the cluster, as a fixed binary tree
template <int CL>
__device__ __forceinline__ df2 tree_sum(cg::cluster_group& cluster, const df2* slot, int idx) {
  df2 v[CL];
#pragma unroll
  for (int r = 0; r < CL; ++r) v[r] = cluster.map_shared_rank(slot, r)[idx];
#pragma unroll
  for (int s = 1; s < CL; s <<= 1)
#pragma unroll
    for (int r = 0; r + s < CL; r += 2 * s) v[r] = add(v[r], v[r + s]);
  return v[0];
}

// Dynamic shared memory bytes of one CTA: (hi, lo) pairs of the panel [NB][ld], of v and of
// the next column [ld] each (interleaved pairs: one 64-bit access per operand; with ld = TPC
// (mod 16) the two column groups of a half-warp fall on disjoint banks)
template <int NB>
constexpr size_t panel_df_smem_bytes(int ld) {
  return size_t(NB + 2) * size_t(ld) * sizeof(df2);
}

// Factor panel columns [j0, j0+nb) of the column-major m x n matrix F (ld = m), rows >= j0:
// on exit R on/above the diagonal, the reflectors below it (unit diagonal implicit), tau, and T
// (column-major, ld NB, upper triangular; zero outside [0, nb)) with H_j0..H_{j0+nb-1} =
// I - V T V^T. `ld` is the CTA's shared-memory row stride (>= rows per CTA).
template <int NB, int CL>
__global__ void __launch_bounds__(DPT) panel_df_kernel(double* __restrict__ F, int64_t m, int64_t j0, int nb, int ld,
                                                       double* __restrict__ tau_out, double* __restrict__ T_out
#ifdef TNX_PANEL_PROBE
                                                       ,
                                                       long long* stamps
#endif
) {
  constexpr int TPC = DPT / NB;  // threads per panel column
  constexpr int NR = NB / CL;    // rows of T held by each CTA
  static_assert(NB % CL == 0 && TPC >= 2 && TPC <= 32 && (TPC & (TPC - 1)) == 0, "panel shape");
  cg::cluster_group cluster = cg::this_cluster();
  const int q = int(cluster.block_rank());
  extern __shared__ df2 pd[];
  df2* X = pd;                        // [NB][ld] panel rows of this CTA, column-major
  df2* V = pd + NB * ld;              // reflector of the current column over this CTA's rows
  df2* N = V + ld;                    // next column after the current reflector
  __shared__ df2 slot[2][3][NB];      // exchange: partial dots, pivot row, partial T dots
  __shared__ unsigned long long smax[NB];
  __shared__ df2 S[NB], P[NB], Z[NB], taus[NB], sc[4];
  __shared__ df2 Tr[NR][NB];          // rows q, q + CL, ... of T
  __shared__ int cexp[NB];
  const int tid = threadIdx.x, ci = tid / TPC, h = tid % TPC, warp = tid >> 5, lane = tid & 31;
  const int64_t mp = m - j0;
  const int64_t rpc = (mp + CL - 1) / CL;
  const int64_t r0 = int64_t(q) * rpc;
  const int rows = int(r0 >= mp ? 0 : (mp - r0 < rpc ? mp - r0 : rpc));
#ifdef TNX_PANEL_PROBE
  int jj = 0;
#endif

  // ---- column scales: largest |entry| of each panel column over the cluster (integer max of
  // the magnitude bits), exponent chosen so that it lands in [2^31, 2^32)
  {
    unsigned long long mx = 0;
    if (ci < nb)
      for (int r = h; r < rows; r += TPC) {
        const unsigned long long b =
            static_cast<unsigned long long>(__double_as_longlong(F[(j0 + ci) * m + j0 + r0 + r])) & 0x7fffffffffffffffull;
        mx = b > mx ? b : mx;
      }
#pragma unroll
    for (int o = TPC / 2; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = t > mx ? t : mx;
    }
    if (h == 0 && ci < NB) smax[ci] = mx;
  }
  cluster_arrive_release();
  cluster_wait_acquire();
  if (tid < NB) {
    unsigned long long mx = 0;
#pragma unroll
    for (int r = 0; r < CL; ++r) {
      const unsigned long long t = cluster.map_shared_rank(smax, r)[tid];
      mx = t > mx ? t : mx;
    }
    const int ef = int(mx >> 52);  // biased exponent of the column maximum (0: zero column)
    cexp[tid] = ef == 0 ? 0 : ef - 1023 - 31;
  }
  __syncthreads();
  for (int e = tid; e < nb * rows; e += DPT) {
    const int c = e / rows, r = e % rows;
    X[c * ld + r] = split_scaled(F[(j0 + c) * m + j0 + r0 + r], cexp[c]);
  }
  for (int e = tid; e < NR * NB; e += DPT) Tr[e / NB][e % NB] = {0.f, 0.f};
  __syncthreads();
  // partials of pivot 0: x_0 . x_c below row 0, and pivot row 0 (rank 0)
  {
    df2 a0 = {0.f, 0.f};
    if (ci < nb) {
      const int rs = r0 > 0 ? 0 : 1;
      for (int r = rs + ((h - rs) % TPC + TPC) % TPC; r < rows; r += TPC)
        acc(a0, X[r], X[ci * ld + r]);
    }
    a0 = norm(a0);
#pragma unroll
    for (int o = TPC / 2; o > 0; o >>= 1) a0 = add(a0, shfl_xor(a0, o));
    if (ci < nb && h == 0) {
      slot[0][0][ci] = a0;
      if (r0 == 0 && rows > 0) slot[0][1][ci] = X[ci * ld];
    }
  }
  cluster_arrive_release();
  cluster_wait_acquire();

#ifndef TNX_PANEL_PROBE
  for (int jj = 0; jj < nb; ++jj) {
#else
  for (jj = 0; jj < nb; ++jj) {
#endif
    PANEL_STAMP(0);
    const int par = jj & 1;
    const int owner = int(jj / rpc);
    // ---- gather: S[c] (c >= jj), pivot row P[c], T dots Z[a] = v_a . v_{jj-1} (a < jj - 1)
    if (tid < NB) {
      const int c = tid;
      if (c >= jj && c < nb) {
        S[c] = tree_sum<CL>(cluster, &slot[par][0][0], c);
        P[c] = cluster.map_shared_rank(&slot[par][1][0], owner)[c];
      }
    } else if (tid < 2 * NB) {
      const int a = tid - NB;
      if (a < jj - 1) Z[a] = tree_sum<CL>(cluster, &slot[par][2][0], a);
    }
    __syncthreads();
    PANEL_STAMP(1);
    // ---- column scalars (one thread; every CTA derives the same bits)
    if (tid == 0) {
      const df2 sigma = S[jj], alpha = P[jj];
      df2 tj = {0.f, 0.f}, beta = alpha, scale = {0.f, 0.f};
      if (sigma.h != 0.f || sigma.l != 0.f) {
        // nrm = sqrt(alpha^2 + sigma) through y = 1 / nrm: tau = (beta - alpha) / beta =
        // 1 + |alpha| y, scale = 1 / (alpha - beta) = sign(alpha) y / tau
        const df2 t = add(mul(alpha, alpha), sigma);
        const df2 y = rsqrt_df(t);
        const df2 nrm = mul(t, y);
        const bool pos = alpha.h > 0.f || (alpha.h == 0.f && alpha.l >= 0.f);
        beta = pos ? neg(nrm) : nrm;
        tj = add({1.f, 0.f}, mul(pos ? alpha : neg(alpha), y));
        const df2 sy = mul(y, rcp_df(tj));
        scale = pos ? sy : neg(sy);
      }
      sc[0] = tj;
      sc[1] = beta;
      sc[2] = scale;
      sc[3] = jj + 1 < nb ? mul(tj, add(P[jj + 1], mul(scale, S[jj + 1]))) : df2{0.f, 0.f};
      taus[jj] = tj;
    }
    __syncthreads();
    PANEL_STAMP(2);
    const df2 tj = sc[0], scale = sc[2], wn = sc[3];
    const bool has_next = jj + 1 < nb;
    const int64_t lj = jj - r0;  // local row of pivot jj (outside [0, rows) on other CTAs)
    const int rA = int(lj > 0 ? lj : 0);
    df2* xj = X + jj * ld;
    // ---- phase A: v = scale x_jj below the pivot (1 at it), next column updated by it
    for (int r = rA + tid; r < rows; r += DPT) {
      const df2 v = r == lj ? df2{1.f, 0.f} : mul(scale, xj[r]);
      V[r] = v;
      if (has_next) N[r] = fms(xj[r + ld], wn, v);
    }
    __syncthreads();
    PANEL_STAMP(3);
    // ---- phase B: update columns c > jj + 1 and the partial dots of step jj + 1 (norm of
    // column jj + 1 below its pivot, its dots with c > jj + 1), pivot row jj + 1, T dots
    df2 a0 = {0.f, 0.f}, a1 = {0.f, 0.f};
    const int64_t ln = lj + 1;
    const bool own_ln = ln >= 0 && ln < rows && int(ln % TPC) == h;
    const int rB = int(lj + 2 > 0 ? lj + 2 : 0);
    const int rB0 = rB + ((h - rB) % TPC + TPC) % TPC;  // first row >= rB held by this thread
    df2(*nxt)[NB] = slot[par ^ 1];
    if (ci < nb && ci > jj + 1) {
      df2* xc = X + ci * ld;
      const df2 wc = mul(tj, add(P[ci], mul(scale, S[ci])));
      if (lj >= 0 && lj < rows && int(lj % TPC) == h) xc[lj] = add(xc[lj], neg(wc));  // v_jj[jj] = 1
      if (own_ln) {
        const df2 t = fms(xc[ln], wc, V[ln]);
        xc[ln] = t;
        nxt[1][ci] = t;
      }
      int r = rB0;
      for (; r + TPC < rows; r += 2 * TPC) {
        const df2 t0 = fms(xc[r], wc, V[r]);
        const df2 t1 = fms(xc[r + TPC], wc, V[r + TPC]);
        xc[r] = t0;
        xc[r + TPC] = t1;
        acc(a0, N[r], t0);
        acc(a1, N[r + TPC], t1);
      }
      if (r < rows) {
        const df2 t0 = fms(xc[r], wc, V[r]);
        xc[r] = t0;
        acc(a0, N[r], t0);
      }
    } else if (ci == jj + 1 && ci < nb) {
      if (own_ln) nxt[1][ci] = N[ln];
      int r = rB0;
      for (; r + TPC < rows; r += 2 * TPC) {
        acc(a0, N[r], N[r]);
        acc(a1, N[r + TPC], N[r + TPC]);
      }
      if (r < rows) acc(a0, N[r], N[r]);
    } else if (ci < jj) {
      const df2* xc = X + ci * ld;
      int r = rA + ((h - rA) % TPC + TPC) % TPC;
      for (; r + TPC < rows; r += 2 * TPC) {
        acc(a0, xc[r], V[r]);
        acc(a1, xc[r + TPC], V[r + TPC]);
      }
      if (r < rows) acc(a0, xc[r], V[r]);
    }
    df2 a = add(norm(a0), norm(a1));
#pragma unroll
    for (int o = TPC / 2; o > 0; o >>= 1) a = add(a, shfl_xor(a, o));
    if (h == 0 && ci < nb) {
      if (ci > jj) nxt[0][ci] = a;
      else if (ci < jj) nxt[2][ci] = a;
    }
    PANEL_STAMP(4);
    cluster_arrive_release();
    __syncthreads();
    // ---- phase C: store v_jj (beta at the pivot) and column jj + 1; extend the held rows of
    // T by column k = jj - 1: T[a][k] = -tau_k sum_{a <= c < k} T[a][c] z_c, T[k][k] = tau_k
    {
      const df2 beta = sc[1];
      for (int r = rA + tid; r < rows; r += DPT) {
        xj[r] = r == lj ? beta : V[r];
        if (has_next) xj[r + ld] = N[r];
      }
      const int k = jj - 1;
      if (k >= 0 && warp < NR) {
        const int a = q + CL * warp;
        if (a < k) {
          df2 t = {0.f, 0.f};
          for (int c = a + lane; c < k; c += 32) acc(t, Tr[warp][c], Z[c]);
          t = norm(t);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) t = add(t, shfl_xor(t, o));
          if (lane == 0) Tr[warp][k] = neg(mul(taus[k], t));
        } else if (a == k && lane == 0) {
          Tr[warp][k] = taus[k];
        }
      }
    }
    // the next gather rewrites S, P and Z, which phase C still reads
    __syncthreads();
    PANEL_STAMP(5);
    cluster_wait_acquire();
  }
  // last T column k = nb - 1 from the final exchange
  if (tid >= NB && tid < 2 * NB) {
    const int a = tid - NB;
    if (a < nb - 1) Z[a] = tree_sum<CL>(cluster, &slot[nb & 1][2][0], a);
  }
  __syncthreads();
  {
    const int k = nb - 1;
    if (warp < NR) {
      const int a = q + CL * warp;
      if (a < k) {
        df2 t = {0.f, 0.f};
        for (int c = a + lane; c < k; c += 32) acc(t, Tr[warp][c], Z[c]);
        t = norm(t);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = add(t, shfl_xor(t, o));
        if (lane == 0) Tr[warp][k] = neg(mul(taus[k], t));
      } else if (a == k && lane == 0) {
        Tr[warp][k] = taus[k];
      }
    }
  }
  __syncthreads();
  // T (column-major, ld NB): this CTA's rows; tau from rank 0
  for (int e = tid; e < NR * NB; e += DPT) {
    const int i = e / NB, b = e % NB, a = q + CL * i;
    T_out[b * NB + a] = (a <= b && b < nb) ? join_df(Tr[i][b].h, Tr[i][b].l) : 0.0;
  }
  if (q == 0)
    for (int b = tid; b < NB; b += DPT) tau_out[b] = b < nb ? join_df(taus[b].h, taus[b].l) : 0.0;
  // panel back to F: R entries (panel row <= column) rescaled, reflectors as they are
  for (int e = tid; e < nb * rows; e += DPT) {
    const int c = e / rows, r = e % rows;
    const df2 v = X[c * ld + r];
    F[(j0 + c) * m + j0 + r0 + r] = r0 + r <= c ? join_scaled(v, cexp[c]) : join_df(v.h, v.l);
  }
  // no CTA leaves while another may still read its slots
  cluster_arrive_release();
  cluster_wait_acquire();
}

}  // namespace qrdf
}  // namespace tnx

#undef PANEL_STAMP
