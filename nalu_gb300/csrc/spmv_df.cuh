// spmv_df.cuh -- FP64-accurate SpMV on the FP32 pipes for the Krylov solvers.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, so one FP64 multiply-add per
// stored entry makes the SELL-32 SpMV FP64-bound rather than HBM-bound.
// Here the matrix values and the search direction are stored as FP32 pairs
// (hi + lo, about 48 significant bits; same 8 bytes as an FP64 value) and
// every product is formed with an FMA-based TwoProd, summed with TwoSum
// (Ogita-Rump-Oishi compensated dot product); the row result is returned as
// an FP64 value.  Absolute error per row is about 2^-46 sum_j |a_ij p_j|.
#pragma once
#include <cuda_runtime.h>

#include "df64.h"

// gathers issued per group in the SELL row loops (all index and value loads of
// a group before its dependent gathers)
#ifndef NALU_SPMV_GROUP
#define NALU_SPMV_GROUP 8
#endif

namespace nalu_gb300 {

// FP32 pair of a double (hi nearest, lo the next 24 bits) with integer ops.
// Magnitudes at or above 2^128 (and infinities, NaN) give (+-inf or NaN, 0),
// so a breakdown stays visible; below 2^-100 gives 0.
__device__ __forceinline__ float2 split_df(double d) {
  const uint64_t b = (uint64_t)__double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e >= 1023 + 128) {
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint32_t nan = (e == 0x7ff && (b & 0xFFFFFFFFFFFFFull)) ? 0x400000u : 0u;
    return make_float2(__uint_as_float(sign | 0x7f800000u | nan), 0.0f);
  }
  const df64 s = df_split_bits(d);
  return make_float2(s.hi, s.lo);
}

// double -> float by truncating the significand (integer instructions only;
// the FP64 pipe is the scarce one on GB300).  |d| < 2^-126 gives 0.
__device__ __forceinline__ float narrow_f(double d) {
  const uint64_t b = (uint64_t)__double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < -126) return 0.0f;
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  if (e > 127) return __uint_as_float(sign | 0x7f800000u | (e == 1024 && (b & 0xFFFFFFFFFFFFFull) ? 0x400000u : 0u));
  return __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | (uint32_t)((b >> 29) & 0x7fffffu));
}

// scalars: fs[FS_BETA], fs[FS_ALPHA], fs[FS_PQ] (p . A p), fs[FS_RR] (r . r)
enum { FS_BETA = 0, FS_ALPHA = 1, FS_PQ = 2, FS_RR = 3 };

// z = M r (FP32 stencil values, FP32 residual); beta = -(z . q_old) / (p . q)_old by the last block

// exact widening of a float with integer ops only (float subnormals -> 0,
// infinities and NaN kept)
__device__ __forceinline__ double widen_f(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xff;
  const uint64_t sign = (uint64_t)(u >> 31) << 63;
  const uint64_t man = (uint64_t)(u & 0x7fffffu) << 29;
  const uint64_t exp = e == 0xff ? 0x7ffull : (uint64_t)(e + (1023 - 127));
  return __longlong_as_double((long long)(e == 0 ? sign : (sign | (exp << 52) | man)));
}

__device__ __forceinline__ double join_df(float2 v) { return widen_f(v.x) + widen_f(v.y); }

// a * b + c with a, b, c FP32 pairs (Dekker/QD style, FP32 instructions only)
__device__ __forceinline__ float2 fma_df(float2 a, float2 b, float2 c) {
  const float ph = __fmul_rn(a.x, b.x);
  const float pe = __fmaf_rn(a.x, b.x, -ph);
  const float pl = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, pe));
  const float t = __fadd_rn(ph, c.x);                           // TwoSum(ph, c.hi)
  const float bp = __fsub_rn(t, ph);
  const float er = __fadd_rn(__fsub_rn(ph, __fsub_rn(t, bp)), __fsub_rn(c.x, bp));
  const float lo = __fadd_rn(er, __fadd_rn(pl, c.y));
  const float hi = __fadd_rn(t, lo);                            // renormalise
  return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, t)));
}

// s += x * x * d for FP64 x and d, accumulated as an FP32 pair (about 46
// significant bits; no FP64 instruction)
__device__ __forceinline__ void acc_sq_df(float& sh, float& sl, float2 x, float d) {
  const float hh = __fmul_rn(x.x, x.x);
  const float he = __fmaf_rn(x.x, x.x, -hh);
  const float x2l = __fadd_rn(he, __fmul_rn(2.0f * x.x, x.y));    // x^2 = hh + x2l
  const float ph = __fmul_rn(hh, d);
  const float pe = __fmaf_rn(hh, d, -ph);
  const float lo = __fmaf_rn(x2l, d, pe);                          // x^2 d = ph + lo
  const float t = __fadd_rn(sh, ph);
  const float bp = __fsub_rn(t, sh);
  const float er = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(ph, bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(er, lo));
}

// s += a * b for FP32 pairs a, b: TwoProd of the high parts, the cross terms,
// TwoSum into (sh, sl)
__device__ __forceinline__ void acc_mul_df(float& sh, float& sl, float2 a, float2 b) {
  const float ph = __fmul_rn(a.x, b.x);
  const float pe = __fmaf_rn(a.x, b.x, -ph);                   // exact product error
  const float cr = __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x));   // cross terms
  const float t = __fadd_rn(sh, ph);                           // TwoSum(sh, ph)
  const float bp = __fsub_rn(t, sh);
  const float er = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(ph, bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(er, __fadd_rn(pe, cr)));
}

// (sh, sl) renormalised to an FP32 pair (FastTwoSum; |sl| is small against |sh|)
__device__ __forceinline__ float2 norm_df(float sh, float sl) {
  const float hi = __fadd_rn(sh, sl);
  return make_float2(hi, __fsub_rn(sl, __fsub_rn(hi, sh)));
}

// one SELL-32 row: sum_k val[base + 32 k] * p[col[base + 32 k]], as an FP32 pair
__device__ __forceinline__ float2 sell_row_df2(int64_t base, int len, const int32_t* __restrict__ scol,
                                               const float2* __restrict__ sval, const float2* __restrict__ p) {
  float sh = 0.0f, sl = 0.0f;
  auto add = [&](float2 a, float2 b) { acc_mul_df(sh, sl, a, b); };
  // groups of 8 (predicated past the row length): all index and value loads
  // of a group are issued before the dependent gathers, so each thread keeps
  // many DRAM requests in flight
  for (int k = 0; k < len; k += 8) {
    int32_t c[8];
    float2 a[8], b[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool in = k + u < len;
      c[u] = in ? __ldg(scol + base + (int64_t)(k + u) * 32) : -1;
      a[u] = in ? __ldg(sval + base + (int64_t)(k + u) * 32) : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) b[u] = c[u] >= 0 ? __ldg(p + c[u]) : make_float2(0.0f, 0.0f);
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (c[u] >= 0) add(a[u], b[u]);
  }
  return norm_df(sh, sl);
}

// one SELL-32 row with 16-bit column offsets from a per-(slice, entry) base:
// col = cbase[k] + col16[base + 32 k]
__device__ __forceinline__ float2 sell_row_df2_c16(int64_t base, int len, const uint16_t* __restrict__ col16,
                                                   const int32_t* __restrict__ cbase,
                                                   const float2* __restrict__ sval, const float2* __restrict__ p) {
  float sh = 0.0f, sl = 0.0f;
  constexpr int G = NALU_SPMV_GROUP;
  for (int k = 0; k < len; k += G) {
    int32_t c[G];
    float2 a[G], b[G];
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const bool in = k + u < len;
      c[u] = in ? __ldg(cbase + k + u) + (int32_t)__ldg(col16 + base + (int64_t)(k + u) * 32) : -1;
      a[u] = in ? __ldg(sval + base + (int64_t)(k + u) * 32) : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int u = 0; u < G; ++u) b[u] = c[u] >= 0 ? __ldg(p + c[u]) : make_float2(0.0f, 0.0f);
#pragma unroll
    for (int u = 0; u < G; ++u)
      if (c[u] >= 0) acc_mul_df(sh, sl, a[u], b[u]);
  }
  return norm_df(sh, sl);
}

// the same row as an FP64 value
__device__ __forceinline__ double sell_row_df(int64_t base, int len, const int32_t* __restrict__ scol,
                                              const float2* __restrict__ sval, const float2* __restrict__ p) {
  return join_df(sell_row_df2(base, len, scol, sval, p));
}

}  // namespace nalu_gb300
