// assemble_ip.cuh -- the double-float scalar assembly (ScalarDiffElemKernel,
// ContinuityAdvElemKernel) with one thread per (element, SCS integration
// point) instead of one thread per element.
//
// Why: the element-per-thread kernel holds an element's 8x8 matrix, its edge
// form and its 12-ip loop in one thread (168 registers, 576 B of shared
// memory per thread), which leaves 12 warps per SM and an issue-latency bound.
// Here a block of EPB elements runs in three phases:
//   0. gather (8 threads per element): node ids, coordinates relative to node
//      0 normalised by a power of two (rel_coords_df), nodal inputs; then the
//      edge-form coefficients of the Jacobian (9 threads per element) and the
//      trilinear coefficients of the nodal inputs (3 or 1 per element);
//   1. geometry (12 threads per element, one per SCS ip): Jacobian, cofactors,
//      area vector, G = adj(J)^T A, the eight lhs factors and the ip mass flow;
//   2. rows (8 threads per element): each row sums the factors of its three
//      ips in ascending ip order (the reference's order), converts to FP64,
//      forms the residual and scatters.
// Every lane of phase 1 runs the same instruction stream whatever its ip: the
// Jacobian is formed in a frame rotated cyclically so that the SCS normal
// axis comes first (an even permutation: det and the cofactor columns map onto
// each other), so the zero ip coordinate along the normal is known at compile
// time, and the per-ip constants come from bit tables, not branches.
// The arithmetic is that of hex8_elem_df.h (same error-free transforms, same
// summation order of the element matrix and rhs).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "assemble_df.cuh"
#include "hex8_elem_df.h"
#include "internal.h"

namespace nalu_gb300 {

// ---- per-ip constants as bit tables (compile-time, from hex8_elem.h) ------
// normal axis dd of each ip (2 bits per ip)
constexpr uint32_t ip_tab_dir() {
  uint32_t t = 0;
  for (int ip = 0; ip < 12; ++ip) t |= (uint32_t)ip_dir(ip) << (2 * ip);
  return t;
}
// sign bits of the ip location along t1 = dd+1 and t2 = dd+2 (mod 3), and of
// the area orientation (bit 0: s_t1 > 0, bit 1: s_t2 > 0, bit 2: ip_sign < 0)
constexpr uint64_t ip_tab_sign() {
  uint64_t t = 0;
  for (int ip = 0; ip < 12; ++ip) {
    const int dd = ip_dir(ip), t1 = (dd + 1) % 3, t2 = (dd + 2) % 3;
    const uint64_t b = (ip_loc(ip, t1, 1.0) > 0 ? 1u : 0u) | (ip_loc(ip, t2, 1.0) > 0 ? 2u : 0u) |
                       (ip_sign(ip) < 0 ? 4u : 0u);
    t |= b << (3 * ip);
  }
  return t;
}
// node index of rotated corner q (bit 0: sign along dd, bit 1: along t1,
// bit 2: along t2) for normal axis dd (3 bits per corner)
constexpr uint32_t ip_tab_node(int dd) {
  uint32_t t = 0;
  for (int q = 0; q < 8; ++q) {
    int sg[3] = {0, 0, 0};
    sg[dd] = (q & 1) ? 1 : -1;
    sg[(dd + 1) % 3] = (q & 2) ? 1 : -1;
    sg[(dd + 2) % 3] = (q & 4) ? 1 : -1;
    t |= (uint32_t)node_of(sg[0], sg[1], sg[2]) << (3 * q);
  }
  return t;
}
constexpr uint32_t kIpDir = ip_tab_dir();
constexpr uint64_t kIpSign = ip_tab_sign();
constexpr uint32_t kIpNode0 = ip_tab_node(0), kIpNode1 = ip_tab_node(1), kIpNode2 = ip_tab_node(2);

// shared-memory row strides (df64 words; odd strides spread elements over banks)
constexpr int kEfStride = 37;          // edge form [k][i][A,B,C,D] = 36
constexpr int kWcStride = 25;          // trilinear coefficients [comp][8] (or [8] for k)
constexpr int kXStride = 25;           // normalised coordinates [8][3]
constexpr int kFacRow = 9;             // factors of one ip: 8 (+1 pad)
constexpr int kFacStride = 12 * kFacRow + 1;

// registers the launch bounds allow per thread: 65536 / (12 EPB * blocks per
// SM).  The standard kernels (LIGHT) run at 40 registers and 48 warps per SM
// (continuity: an 8-byte spill; measured fastest at 128^3, 5% ahead of 64
// registers); the continuity variants with the pressure-stabilisation
// difference or shifted gradients (MODE 1, 2) and the shifted diffusion hold
// more live state and keep 85 (8 elements per block) or 64 registers (16),
// which they fill without spilling more than a word.
template <int EPB, bool LIGHT>
struct IpSched {
  static constexpr int kThreads = 12 * EPB;
  static constexpr int kMinBlocks = EPB == 8 ? (LIGHT ? 16 : 8) : (LIGHT ? 7 : 5);
};
template <int KIND, int MODE, bool SHIFT>
constexpr bool ip_light() { return MODE == 0 && !(KIND == 0 && SHIFT); }

// J' columns at the ip (rotated frame: column 0 = normal axis dd, 1 = t1,
// 2 = t2), from the edge form in shared memory.  s1, s2: ip coordinates along
// t1, t2 (the coordinate along dd is 0 at every SCS ip, standard or shifted).
__device__ __forceinline__ void jacobian_rot_df(const df64* EF, int dd, int t1, int t2, float s1, float s2,
                                                df64 j[3][3]) {
  // column dd: A + B s_u + C s_v + D s_u s_v over its own (u, v) = (t1, t2) in
  // ascending axis order
  const bool t1_first = t1 < t2;
  const float su = t1_first ? s1 : s2, sv = t1_first ? s2 : s1;
  // tangential columns: one ip coordinate (along dd) is zero, so one term
  // remains, the B (s_u) or C (s_v) coefficient of the other tangential axis
  const int q1 = ((t1 == 0 ? 1 : 0) == t2) ? 1 : 2;  // u(t1) == t2 ? B : C
  const int q2 = ((t2 == 0 ? 1 : 0) == t1) ? 1 : 2;
  const float suv = su * sv;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const df64* c0 = EF + 4 * (3 * dd + i);
    j[i][0] = df_sum4(c0[0], df_scale2(c0[1], su), df_scale2(c0[2], sv), df_scale2(c0[3], suv));
    const df64* c1 = EF + 4 * (3 * t1 + i);
    j[i][1] = df_add_lazy(c1[0], df_scale2(c1[q1], s2));
    const df64* c2 = EF + 4 * (3 * t2 + i);
    j[i][2] = df_add_lazy(c2[0], df_scale2(c2[q2], s1));
  }
}

// G'_k = sum_i C'[i][k] area[i]
__device__ __forceinline__ void g_of(const df64 c[3][3], const df64 area[3], df64 g[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) g[k] = df_dot3(c[0][k], area[0], c[1][k], area[1], c[2][k], area[2]);
}

// The eight lhs factors sum_k dN_c/ds_k g_k at an ip of the rotated frame
// (s along dd is 0, so h_dd = 1/2):
//   fac = c_dd h1 h2 g0 + (c1 h2 g1 + h1 c2 g2) / 2,   h = 1/2 + c s.
// The corners of one normal edge (c_dd = +-1) share the bracket X and the
// product Y: fac(+) = X + Y, fac(-) = X - Y.  f(node, value) receives them.
// The factors are formed as unnormalised pairs: the three products k g with
// exact float k (TwoProd error and low part folded into one FP32 term each),
// X by one TwoSum, X +- Y by one TwoSum each, the low terms added in FP32
// (33 FP32 operations per corner pair instead of 51).  Their consumers (the
// row sums and the widening to FP64, or the products of the pressure term)
// take unnormalised pairs.
template <class F>
__device__ __forceinline__ void factors_rot_df(const df64 g[3], float s1, float s2, uint32_t node_tab, F&& f) {
#pragma unroll
  for (int pr = 0; pr < 4; ++pr) {
    const float c1 = (pr & 1) ? 1.0f : -1.0f, c2 = (pr & 2) ? 1.0f : -1.0f;
    const float h1 = 0.5f + c1 * s1, h2 = 0.5f + c2 * s2;  // exact
    const float k1 = 0.5f * c1 * h2, k2 = 0.5f * c2 * h1, k0 = h1 * h2;  // exact
    const float p1 = f_mul(g[1].hi, k1), p2 = f_mul(g[2].hi, k2), p0 = f_mul(g[0].hi, k0);
    const float e1 = f_fma(g[1].lo, k1, f_fma(g[1].hi, k1, -p1));
    const float e2 = f_fma(g[2].lo, k2, f_fma(g[2].hi, k2, -p2));
    const float e0 = f_fma(g[0].lo, k0, f_fma(g[0].hi, k0, -p0));
    const df64 x = two_sum(p1, p2);                  // X = x.hi + xl
    const float xl = f_add(x.lo, f_add(e1, e2));
    const df64 sp = two_sum(x.hi, p0), sm = two_sum(x.hi, -p0);
    const int qm = 2 * pr, qp = 2 * pr + 1;  // rotated corner: bit 0 = sign along dd
    f((int)((node_tab >> (3 * qp)) & 7u), df64{sp.hi, f_add(sp.lo, f_add(xl, e0))});
    f((int)((node_tab >> (3 * qm)) & 7u), df64{sm.hi, f_add(sm.lo, f_sub(xl, e0))});
  }
}

// trilinear coefficients at an ip (monomials with s_dd vanish)
__device__ __forceinline__ df64 trilinear_rot_df(const df64* c, int t1, int t2, float s1, float s2) {
  return df_sum4(c[0], df_scale2(c[1 << t1], s1), df_scale2(c[1 << t2], s2),
                 df_scale2(c[(1 << t1) | (1 << t2)], s1 * s2));
}

template <int EPB, int KIND, int MODE, bool SHIFT, bool SMDOT>
__global__ void __launch_bounds__(IpSched<EPB, ip_light<KIND, MODE, SHIFT>()>::kThreads,
                                 IpSched<EPB, ip_light<KIND, MODE, SHIFT>()>::kMinBlocks)
    k_assemble_ip_df(AsmArgsDF a) {
  constexpr int NCOMP = KIND == 0 ? 1 : 3;
  __shared__ df64 s_ef[EPB][kEfStride];
  __shared__ df64 s_wc[EPB][kWcStride];
  __shared__ df64 s_fac[EPB][kFacStride];
  // the normalised coordinates live only in phases 0a-0b, the factors from
  // phase 1 on: they share storage (smaller blocks, one more block per SM)
  static_assert(kXStride <= kFacStride, "coordinates fit the factor rows");
  df64(*s_x)[kXStride] = reinterpret_cast<df64(*)[kXStride]>(&s_fac[0][0]);
  __shared__ df64 s_m[EPB][13];
  __shared__ df64 s_pd[EPB][MODE == 1 ? 9 : 1];
  __shared__ double s_p[EPB][9];
  __shared__ int s_nd[EPB][8];
  __shared__ int s_k[EPB];
  __shared__ int64_t s_e[EPB];
  const int OUT = a.out;
  const int t = threadIdx.x;
  const int64_t base_el = (int64_t)blockIdx.x * EPB;

  // ---- phase 0a: gather, 8 threads per element ----
  if (t < 8 * EPB) {
    const int el = t >> 3, n = t & 7;
    const int64_t gi = base_el + el;
    const bool valid = gi < a.count;
    const int64_t e = !valid ? 0 : (OUT == 2 ? a.cap_elem : (a.elems ? (int64_t)a.elems[gi] : gi));
    const int nd = __ldg(a.conn + 8 * e + n);
    double dx[3];
    int emax = -1023;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double xv = __ldg(a.x + 3 * (int64_t)nd + d);
      const double x0 = __shfl_sync(0xffffffffu, xv, 0, 8);  // node 0 of this element
      dx[d] = xv - x0;
      emax = max(emax, dexp(dx[d]));
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o, 8));
    const int kexp = min(max(emax, -kNormExpMax), kNormExpMax);
#pragma unroll
    for (int d = 0; d < 3; ++d) s_x[el][3 * n + d] = n == 0 ? df_zero() : df_split_bits(dx[d], kexp);
#pragma unroll
    for (int c = 0; c < NCOMP; ++c) s_wc[el][8 * c + n] = a.nodal[NCOMP * (int64_t)nd + c];
    const double pv = __ldg(a.f_a + nd);
    s_p[el][n] = pv;
    if (MODE == 1) s_pd[el][n] = df_split_bits(pv);
    s_nd[el][n] = nd;
    if (n == 0) {
      s_k[el] = kexp;
      s_e[el] = e;
    }
  }
  __syncthreads();

  // ---- phase 0b: edge form (9 per element) and trilinear coefficients ----
  if (t < 9 * EPB) {
    const int el = t / 9, ki = t - 9 * (t / 9);
    const int k = ki / 3, i = ki - 3 * (ki / 3);
    const int u = (k == 0) ? 1 : 0, v = (k == 2) ? 1 : 2;
    df64 ed[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int sg[3];
      sg[u] = (q & 1) ? 1 : -1;
      sg[v] = (q & 2) ? 1 : -1;
      sg[k] = -1;
      const int na = node_of(sg[0], sg[1], sg[2]);
      sg[k] = 1;
      const int nb = node_of(sg[0], sg[1], sg[2]);
      ed[q] = df_add_lazy(s_x[el][3 * nb + i], df_neg(s_x[el][3 * na + i]));
    }
    // unnormalised pairs throughout: the Jacobian sums (df_sum4,
    // df_add_lazy) and the cofactor products take them
    const df64 p01 = df_add_lazy(ed[0], ed[1]), m01 = df_add_lazy(ed[1], df_neg(ed[0]));
    const df64 p23 = df_add_lazy(ed[2], ed[3]), m23 = df_add_lazy(ed[3], df_neg(ed[2]));
    df64* o = &s_ef[el][4 * ki];
    o[0] = df_scale2(df_add_lazy(p01, p23), 0.25f);
    o[1] = df_scale2(df_add_lazy(m01, m23), 0.5f);
    o[2] = df_scale2(df_add_lazy(p23, df_neg(p01)), 0.5f);
    o[3] = df_add_lazy(m23, df_neg(m01));
  } else if (t < (9 + NCOMP) * EPB) {
    const int tt = t - 9 * EPB;
    const int el = tt / NCOMP, comp = tt - NCOMP * (tt / NCOMP);
    df64* w = &s_wc[el][8 * comp];
    df64 v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = w[node_of((m & 1) ? 1 : -1, (m & 2) ? 1 : -1, (m & 4) ? 1 : -1)];
#pragma unroll
    for (int kb = 0; kb < 3; ++kb) {
      const int bit = 1 << kb;
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        if (m & bit) continue;
        const df64 lo = v[m], hi = v[m | bit];
        v[m] = df_scale2(df_add_lazy(lo, hi), 0.5f);
        v[m | bit] = df_add_lazy(hi, df_neg(lo));
      }
    }
#pragma unroll
    for (int m = 0; m < 8; ++m) w[m] = v[m];
  }
  __syncthreads();

  // ---- phase 1: one thread per (element, ip) ----
  {
    const int el = t / 12, ip = t - 12 * (t / 12);
    const bool valid = base_el + el < a.count;
    if (valid) {
      const int dd = (int)((kIpDir >> (2 * ip)) & 3u);
      const int t1 = dd == 2 ? 0 : dd + 1, t2 = dd == 0 ? 2 : dd - 1;
      const uint32_t sb = (uint32_t)((kIpSign >> (3 * ip)) & 7u);
      const float g1 = (sb & 1u) ? 1.0f : -1.0f, g2 = (sb & 2u) ? 1.0f : -1.0f;
      const float sc = (sb & 4u) ? -0.25f : 0.25f;  // ip_sign / 4
      const uint32_t ntab = dd == 0 ? kIpNode0 : (dd == 1 ? kIpNode1 : kIpNode2);
      const df64* EF = s_ef[el];
      df64* FAC = &s_fac[el][kFacRow * ip];
      const float s1 = 0.25f * g1, s2 = 0.25f * g2;  // standard ip location along t1, t2
      df64 area[3], gstd[3], det;
      {
        df64 j[3][3], c[3][3];
        jacobian_rot_df(EF, dd, t1, t2, s1, s2, j);
        cofactor_df(j, c, det);
#pragma unroll
        for (int i = 0; i < 3; ++i) area[i] = df_scale2(c[i][0], sc);
        g_of(c, area, gstd);
      }
      float mindet = det.hi;
      constexpr bool SH = (KIND == 0) ? SHIFT : (MODE != 0);
      df64 gl[3], detl = det;
      if (SH) {
        df64 j[3][3], c[3][3];
        jacobian_rot_df(EF, dd, t1, t2, 2.0f * s1, 2.0f * s2, j);
        cofactor_df(j, c, detl);
        g_of(c, area, gl);
        mindet = fminf(mindet, detl.hi);
      } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) gl[k] = gstd[k];
      }
      if (!(mindet > 0.0f)) atomicAdd(a.flags + FLAG_NEG_JAC, 1);
      df64 scale = df_neg(df_rcp(detl));
      if (KIND == 0) scale = df_mul(trilinear_rot_df(s_wc[el], t1, t2, s1, s2), scale);  // -k_ip / det
#pragma unroll
      for (int k = 0; k < 3; ++k) gl[k] = df_mul_lazy(gl[k], scale);
      const float l1 = SH ? 2.0f * s1 : s1, l2 = SH ? 2.0f * s2 : s2;
      factors_rot_df(gl, l1, l2, ntab, [&](int node, df64 v) { FAC[node] = v; });
      if (KIND == 1) {
        const float m1 = SMDOT ? 2.0f * s1 : s1, m2 = SMDOT ? 2.0f * s2 : s2;
        const df64 wx = trilinear_rot_df(s_wc[el], t1, t2, m1, m2);
        const df64 wy = trilinear_rot_df(s_wc[el] + 8, t1, t2, m1, m2);
        const df64 wz = trilinear_rot_df(s_wc[el] + 16, t1, t2, m1, m2);
        df64 m = df_mul(df_dot3(wx, area[0], wy, area[1], wz, area[2]), a.inv_tau);
        if (MODE == 1) {
          // reduced sensitivities: the standard-location pressure term joins mdot
          const df64 sstd = df_neg(df_rcp(det));
          df64 gs[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) gs[k] = df_mul(gstd[k], sstd);
          df64 dpa = df_zero();
          const df64* PD = s_pd[el];
          factors_rot_df(gs, s1, s2, ntab, [&](int node, df64 v) { dpa = df_fma(v, PD[node], dpa); });
          m = df_add(m, df_scale2(dpa, pow2f(-s_k[el])));
        }
        s_m[el][ip] = m;
      }
    }
  }
  __syncthreads();

  // ---- phase 2: one thread per (element, row) ----
  if (t >= 8 * EPB) return;
  const int el = t >> 3, r = t & 7;
  if (base_el + el >= a.count) return;
  const int rb = r & 4, rq = r & 3;
  int ips[3];
  ips[0] = rb + (rq == 0 ? 0 : rq - 1);
  ips[1] = rb + (rq == 0 ? 3 : rq);
  ips[2] = 8 + rq;
  const int kexp = s_k[el];
  // each entry sums its three ips' factors (ascending ip) as one unnormalised
  // pair; the widening to FP64 below renormalises it
  const bool l0 = ip_left(ips[0]) == r, l1 = ip_left(ips[1]) == r, l2 = ip_left(ips[2]) == r;
  const df64* F0 = &s_fac[el][kFacRow * ips[0]];
  const df64* F1 = &s_fac[el][kFacRow * ips[1]];
  const df64* F2 = &s_fac[el][kFacRow * ips[2]];
  df64 v[8];
#pragma unroll
  for (int c = 0; c < 8; ++c)
    v[c] = df_sum3_lazy(l0 ? F0[c] : df_neg(F0[c]), l1 ? F1[c] : df_neg(F1[c]), l2 ? F2[c] : df_neg(F2[c]));
  df64 rs = df_zero();
  if (KIND == 1) {
    const df64 m0 = s_m[el][ips[0]], m1 = s_m[el][ips[1]], m2 = s_m[el][ips[2]];
    rs = df_sum3_lazy(l0 ? df_neg(m0) : m0, l1 ? df_neg(m1) : m1, l2 ? df_neg(m2) : m2);
  }
  const bool rhs_from_lhs = (KIND == 0) || (MODE != 1);
  double s = KIND == 1 ? df_to_double_bits(rs, 2 * kexp) : 0.0;
  double vd[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    vd[c] = df_to_double_bits(v[c], kexp);
    if (rhs_from_lhs) s -= vd[c] * s_p[el][c];
  }
  if (OUT == 2) {
#pragma unroll
    for (int c = 0; c < 8; ++c) a.cap_lhs[r * 8 + c] = vd[c];
    a.cap_rhs[r] = s;
    return;
  }
  const int nd = s_nd[el][r];
  const int64_t e = s_e[el];
  const int64_t base = __ldg(a.rowptr + nd);
  const uint2 o2 = __ldg(reinterpret_cast<const uint2*>(a.slots + 64 * e + 8 * r));
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const uint32_t word = c < 4 ? o2.x : o2.y;
    const int off = (word >> (8 * (c & 3))) & 0xff;
    double* dst = a.values + base + off;
    if (OUT == 0) atomicAdd(dst, vd[c]);
    else *dst += vd[c];
  }
  if (OUT == 0) atomicAdd(a.rhs + nd, s);
  else a.rhs[nd] += s;
}

// launch one compiled variant; out: 0 atomic, 1 coloured, 2 capture
template <int EPB, int KIND, int MODE, bool SHIFT, bool SMDOT>
void launch_ip_variant(nalu_ctx* ctx, AsmArgsDF a, int out) {
  if (a.count <= 0) return;
  a.out = out;
  const unsigned grid = (unsigned)((a.count + EPB - 1) / EPB);
  k_assemble_ip_df<EPB, KIND, MODE, SHIFT, SMDOT><<<grid, 12 * EPB, 0, ctx->stream>>>(a);
  ctx->launches++;
}

#define NALU_IP_VARIANTS(X, EPB) \
  X(EPB, 0, 0, false, false) X(EPB, 0, 0, true, false) X(EPB, 1, 0, false, false) X(EPB, 1, 0, false, true) \
  X(EPB, 1, 1, false, false) X(EPB, 1, 1, false, true) X(EPB, 1, 2, false, false) X(EPB, 1, 2, false, true)
#define NALU_IP_EXTERN(E, K, M, S, SM) extern template void launch_ip_variant<E, K, M, S, SM>(nalu_ctx*, AsmArgsDF, int);

}  // namespace nalu_gb300
