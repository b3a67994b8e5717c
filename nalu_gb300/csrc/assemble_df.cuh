// assemble_df.cuh -- the double-float scalar assembly kernel template, shared
// by assemble_df.cu (dispatch) and the assemble_df_*.cu files that each
// instantiate a few variants (so they compile in parallel).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "hex8_elem_df.h"
#include "internal.h"

namespace nalu_gb300 {

constexpr int kAsmBlockDF = 64;
// resident blocks per SM the register allocation must allow (occupancy vs spills)
#ifndef NALU_DF_MINB
#define NALU_DF_MINB 5
#endif

struct AsmArgsDF {
  const int32_t* __restrict__ conn;
  const double* __restrict__ x;
  const df64* __restrict__ nodal;  // k [n] or w [n][3]
  const double* __restrict__ f_a;  // q (scalar diff) or pressure
  df64 inv_tau;
  const int64_t* __restrict__ rowptr;
  const uint8_t* __restrict__ slots;
  double* __restrict__ values;
  double* __restrict__ rhs;
  const int32_t* __restrict__ elems;
  int64_t count;
  int32_t* flags;
  double* cap_lhs;
  double* cap_rhs;
  int64_t cap_elem;
  int out;  // 0 atomic scatter, 1 coloured (plain RMW), 2 capture
};

struct SmemAccDF {
  df64 (*s)[kAsmBlockDF];   // [64 entries][threads]: element matrix
  df64 (*rs)[kAsmBlockDF];  // [8 rows][threads]: element rhs
  int t;
  __device__ __forceinline__ void set(int r, int c, df64 v) { s[r * 8 + c][t] = v; }
  __device__ __forceinline__ void add(int r, int c, df64 v) { s[r * 8 + c][t] = df_add(s[r * 8 + c][t], v); }
  __device__ __forceinline__ df64 get(int r, int c) const { return s[r * 8 + c][t]; }
  __device__ __forceinline__ void rset(int r, df64 v) { rs[r][t] = v; }
  __device__ __forceinline__ void radd(int r, df64 v) { rs[r][t] = df_add(rs[r][t], v); }
  __device__ __forceinline__ df64 rget(int r) const { return rs[r][t]; }
};

template <int KIND, int MODE, bool SHIFT, bool SMDOT>
__global__ void __launch_bounds__(kAsmBlockDF, NALU_DF_MINB) k_assemble_scalar_df(AsmArgsDF a) {
  const int OUT = a.out;
  __shared__ df64 s_lhs[64][kAsmBlockDF];
  __shared__ df64 s_rhs[8][kAsmBlockDF];
  const int t = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * kAsmBlockDF + t;
  if (i >= a.count) return;
  const int64_t e = (OUT == 2) ? a.cap_elem : (a.elems ? (int64_t)a.elems[i] : i);
  int nd[8];
  {
    const int4* c4 = reinterpret_cast<const int4*>(a.conn + 8 * e);
    const int4 p0 = __ldg(c4), p1 = __ldg(c4 + 1);
    nd[0] = p0.x; nd[1] = p0.y; nd[2] = p0.z; nd[3] = p0.w;
    nd[4] = p1.x; nd[5] = p1.y; nd[6] = p1.z; nd[7] = p1.w;
  }
  double x[8][3];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const double* px = a.x + 3 * (int64_t)nd[n];
    x[n][0] = __ldg(px);
    x[n][1] = __ldg(px + 1);
    x[n][2] = __ldg(px + 2);
  }
  SmemAccDF acc{s_lhs, s_rhs, t};
  double pv[8];
#pragma unroll
  for (int n = 0; n < 8; ++n) pv[n] = __ldg(a.f_a + nd[n]);
  df64 rhs_df[8];
  double mindet;
  int kexp;  // normalisation: lhs entries x 2^kexp, rhs (flux) entries x 2^(2 kexp)
  if constexpr (KIND == 0) {
    df64 k[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) k[n] = a.nodal[nd[n]];
    mindet = scalar_diff_lhs_df<SHIFT>(x, k, acc, kexp);
#pragma unroll
    for (int r = 0; r < 8; ++r) rhs_df[r] = df_zero();
  } else {
    df64 w[8][3];
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int d = 0; d < 3; ++d) w[n][d] = a.nodal[3 * (int64_t)nd[n] + d];
    df64 pd[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) pd[n] = df_split_bits(pv[n]);
    mindet = continuity_elem_df<MODE, SMDOT>(x, w, a.inv_tau, pd, acc, rhs_df, kexp);
  }
  if (!(mindet > 1.0e-50)) atomicAdd(a.flags + FLAG_NEG_JAC, 1);
  const bool rhs_from_lhs = (KIND == 0) || (MODE != 1);

  if (OUT == 2) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      double s = df_to_double_bits(rhs_df[r], 2 * kexp);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const double v = df_to_double_bits(acc.get(r, c), kexp);
        a.cap_lhs[r * 8 + c] = v;
        if (rhs_from_lhs) s -= v * pv[c];
      }
      a.cap_rhs[r] = s;
    }
    return;
  }
  const uint8_t* sl = a.slots + 64 * e;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int64_t base = __ldg(a.rowptr + nd[r]);
    const uint2 o2 = __ldg(reinterpret_cast<const uint2*>(sl + 8 * r));
    double s = df_to_double_bits(rhs_df[r], 2 * kexp);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const uint32_t word = c < 4 ? o2.x : o2.y;
      const int off = (word >> (8 * (c & 3))) & 0xff;
      const double v = df_to_double_bits(acc.get(r, c), kexp);
      if (rhs_from_lhs) s -= v * pv[c];
      double* dst = a.values + base + off;
      if (OUT == 0) atomicAdd(dst, v);
      else *dst += v;
    }
    if (OUT == 0) atomicAdd(a.rhs + nd[r], s);
    else a.rhs[nd[r]] += s;
  }
}

inline unsigned nblk_df(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

// launch one compiled variant; out: 0 atomic, 1 coloured, 2 capture
template <int KIND, int MODE, bool SHIFT, bool SMDOT>
void launch_df_variant(nalu_ctx* ctx, AsmArgsDF a, int out) {
  if (a.count <= 0) return;
  a.out = out;
  if (out == 2) k_assemble_scalar_df<KIND, MODE, SHIFT, SMDOT><<<1, 1, 0, ctx->stream>>>(a);
  else k_assemble_scalar_df<KIND, MODE, SHIFT, SMDOT><<<nblk_df(a.count, kAsmBlockDF), kAsmBlockDF, 0, ctx->stream>>>(a);
  ctx->launches++;
}

#define NALU_DF_VARIANTS(X) \
  X(0, 0, false, false) X(0, 0, true, false) X(1, 0, false, false) X(1, 0, false, true) \
  X(1, 1, false, false) X(1, 1, false, true) X(1, 2, false, false) X(1, 2, false, true)
#define NALU_DF_EXTERN(K, M, S, SM) extern template void launch_df_variant<K, M, S, SM>(nalu_ctx*, AsmArgsDF, int);

}  // namespace nalu_gb300
