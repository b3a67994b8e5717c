// hex8_elem_df.h -- the Hex8 element math of hex8_elem.h in double-float
// (df64) arithmetic on the FP32 pipes.
//
// Same formulation (edge-form Jacobian, areas from cofactor columns, lhs
// factors from adj(J)^T A) and the same summation order of the element matrix
// as hex8_elem.h.  Unlike the FP64 version the 12 integration points run as a
// loop with their constants computed from the ip index: the unrolled df64 body
// is too large for the instruction cache (measured: warps stalled on
// instruction fetch).  All ip constants are dyadic rationals, exact in FP32.
//
// Precision: coordinates enter as FP64 differences to node 0 of the element
// (their full relative precision survives the split into hi + lo), nodal
// fields enter pre-split per node; every operation is an error-free-transform
// sequence with ~2^-48 relative rounding, about 32x the FP64 unit, well inside
// the 1e-12 parity tolerance (checked on the CPU against the oracle by
// tests/test_elem_math.py and on the GPU by the parity tests).
#pragma once

#include "df64.h"
#include "hex8_elem.h"

namespace nalu_gb300 {

struct EdgeFormDF {
  df64 A[3][3], B[3][3], C[3][3], D[3][3];  // [k][component]
};

// Bound of the per-element normalisation exponent: 2^(2k) and 2^(-k) stay
// normal floats, so kernels can move area- and length-scaled quantities
// back to physical units in df64 as well as in FP64.
constexpr int kNormExpMax = 62;

// x relative to node 0 (FP64 differences), scaled by 2^-k and split into
// df64, where 2^k bounds the largest difference: the element math then runs
// on O(1) numbers whatever the mesh's units.  Products of three or four
// lengths (det J, adj(J)^T A) would otherwise leave the FP32 exponent range
// for element sizes below about 1e-9 or above 1e9.  Lengths in the results
// carry the factor 2^k exactly (a power of two): the caller rescales them.
NALU_HD int rel_coords_df(const double x[8][3], df64 d[8][3]) {
  double dx[8][3];
  int emax = -1023;
#pragma unroll
  for (int n = 1; n < 8; ++n)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dx[n][i] = x[n][i] - x[0][i];
      const int e = dexp(dx[n][i]);
      emax = e > emax ? e : emax;
    }
  const int k = emax < -kNormExpMax ? -kNormExpMax : (emax > kNormExpMax ? kNormExpMax : emax);
#pragma unroll
  for (int i = 0; i < 3; ++i) d[0][i] = df_zero();
#pragma unroll
  for (int n = 1; n < 8; ++n)
#pragma unroll
    for (int i = 0; i < 3; ++i) d[n][i] = df_split_bits(dx[n][i], k);
  return k;
}

NALU_HD void edge_form_df(const df64 d[8][3], EdgeFormDF& f) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int u = (k == 0) ? 1 : 0;
    const int v = (k == 2) ? 1 : 2;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      df64 e[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int sg[3];
        sg[u] = (q & 1) ? 1 : -1;
        sg[v] = (q & 2) ? 1 : -1;
        sg[k] = -1;
        const int a = node_of(sg[0], sg[1], sg[2]);
        sg[k] = 1;
        const int b = node_of(sg[0], sg[1], sg[2]);
        e[q] = (a == 0) ? d[b][i] : df_sub(d[b][i], d[a][i]);
      }
      const df64 p01 = df_add(e[0], e[1]), m01 = df_sub(e[1], e[0]);
      const df64 p23 = df_add(e[2], e[3]), m23 = df_sub(e[3], e[2]);
      f.A[k][i] = df_scale2(df_add(p01, p23), 0.25f);
      f.B[k][i] = df_scale2(df_add(m01, m23), 0.5f);
      f.C[k][i] = df_scale2(df_sub(p23, p01), 0.5f);
      f.D[k][i] = df_sub(m23, m01);
    }
  }
}

// ip location in FP32 arithmetic (a = 0.25 standard, 0.5 shifted); the same
// table as ip_loc() in hex8_elem.h, evaluated without FP64 instructions
NALU_HD float ip_loc_f(int ip, int k, float a) {
  if (ip >= 8) return k == 2 ? 0.0f : (float)corner_sign(ip - 8, k) * a;
  if (k == 2) return ip < 4 ? -a : a;
  const int m = ip & 3;
  if (m == 0) return k == 0 ? 0.0f : -a;
  if (m == 1) return k == 0 ? a : 0.0f;
  if (m == 2) return k == 0 ? 0.0f : a;
  return k == 0 ? -a : 0.0f;
}
NALU_HD void ip_location(int ip, float a, float s[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) s[k] = ip_loc_f(ip, k, a);
}

// J at a runtime ip location s (all entries exact dyadic in FP32)
NALU_HD void jacobian_df(const EdgeFormDF& f, const float s[3], df64 j[3][3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int u = (k == 0) ? 1 : 0;
    const int v = (k == 2) ? 1 : 2;
    const float su = s[u], sv = s[v];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      df64 r = f.A[k][i];
      if (su != 0.0f) r = df_add(r, df_scale2(f.B[k][i], su));
      if (sv != 0.0f) r = df_add(r, df_scale2(f.C[k][i], sv));
      if (su != 0.0f && sv != 0.0f) r = df_add(r, df_scale2(f.D[k][i], su * sv));
      j[i][k] = r;
    }
  }
}

// cofactors as unnormalised pairs (every consumer is a product or a dot
// product, which take them); det renormalised
NALU_HD void cofactor_df(const df64 j[3][3], df64 adj[3][3], df64& det) {
  adj[0][0] = df_cross_lazy(j[1][1], j[2][2], j[2][1], j[1][2]);
  adj[0][1] = df_cross_lazy(j[1][2], j[2][0], j[2][2], j[1][0]);
  adj[0][2] = df_cross_lazy(j[1][0], j[2][1], j[2][0], j[1][1]);
  adj[1][0] = df_cross_lazy(j[0][2], j[2][1], j[2][2], j[0][1]);
  adj[1][1] = df_cross_lazy(j[0][0], j[2][2], j[2][0], j[0][2]);
  adj[1][2] = df_cross_lazy(j[0][1], j[2][0], j[2][1], j[0][0]);
  adj[2][0] = df_cross_lazy(j[0][1], j[1][2], j[1][1], j[0][2]);
  adj[2][1] = df_cross_lazy(j[0][2], j[1][0], j[1][2], j[0][0]);
  adj[2][2] = df_cross_lazy(j[0][0], j[1][1], j[1][0], j[0][1]);
  det = df_dot3(j[0][0], adj[0][0], j[1][0], adj[1][0], j[2][0], adj[2][0]);
}

struct IpGeomDF {
  df64 area[3];
  df64 G[3];
  df64 det;
};

NALU_HD void ip_geometry_df(const EdgeFormDF& f, int ip, IpGeomDF& g) {
  float s[3];
  ip_location(ip, 0.25f, s);
  df64 j[3][3], adj[3][3], det;
  jacobian_df(f, s, j);
  cofactor_df(j, adj, det);
  const int dd = ip_dir(ip);
  const float sc = (ip < 8 && (ip & 3) == 2) ? -0.25f : 0.25f;  // 1/4 ip_sign(ip)
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    // adj[i][dd] with a runtime column index, without dynamic register indexing
    const df64 col = dd == 0 ? adj[i][0] : (dd == 1 ? adj[i][1] : adj[i][2]);
    g.area[i] = df_scale2(col, sc);
  }
#pragma unroll
  for (int jj = 0; jj < 3; ++jj)
    g.G[jj] = df_dot3(adj[0][jj], g.area[0], adj[1][jj], g.area[1], adj[2][jj], g.area[2]);
  g.det = det;
}

NALU_HD void ip_shifted_G_df(const EdgeFormDF& f, int ip, const df64 area[3], df64 G[3], df64& det) {
  float s[3];
  ip_location(ip, 0.5f, s);
  df64 j[3][3], adj[3][3];
  jacobian_df(f, s, j);
  cofactor_df(j, adj, det);
#pragma unroll
  for (int jj = 0; jj < 3; ++jj)
    G[jj] = df_dot3(adj[0][jj], area[0], adj[1][jj], area[1], adj[2][jj], area[2]);
}

// fac[c] = sum_j dN_c/ds_j(s) * (G_j * scale)
//        = c0 h1 h2 g0 + h0 (c1 h2 g1 + c2 h1 g2),   h_k = 1/2 + c_k s_k;
// the two corners of an x-edge share h1, h2 and the bracket, so each pair
// costs one bracket and two short products.
NALU_HD void lhs_factors_df(const df64 G[3], df64 scale, const float s[3], df64 fac[8]) {
  const df64 g0 = df_mul(G[0], scale), g1 = df_mul(G[1], scale), g2 = df_mul(G[2], scale);
  const float hp = 0.5f + s[0], hm = 0.5f - s[0];  // h0 for c0 = +1, -1 (exact)
#pragma unroll
  for (int pr = 0; pr < 4; ++pr) {
    const int cp = node_of(1, (pr & 1) ? 1 : -1, (pr & 2) ? 1 : -1);   // c0 = +1
    const int cm = node_of(-1, (pr & 1) ? 1 : -1, (pr & 2) ? 1 : -1);  // c0 = -1
    const float c1 = (float)corner_sign(cp, 1), c2 = (float)corner_sign(cp, 2);
    const float h1 = 0.5f + c1 * s[1], h2 = 0.5f + c2 * s[2];
    const df64 t = df_add(df_mul_f(g1, c1 * h2), df_mul_f(g2, c2 * h1));  // exact float factors
    const df64 u = df_mul_f(g0, h1 * h2);
    fac[cp] = df_add(u, df_mul_f(t, hp));
    fac[cm] = df_add(df_neg(u), df_mul_f(t, hm));
  }
}

// Trilinear coefficients of a nodal scalar: f(s) = sum_m c_m s^m over the 8
// monomials (index bit k set = factor s_{k+1}); nodal values sit at s = +-1/2.
NALU_HD void trilinear_coeffs_df(const df64 v[8], df64 c[8]) {
  df64 t[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) t[m] = v[node_of((m & 1) ? 1 : -1, (m & 2) ? 1 : -1, (m & 4) ? 1 : -1)];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int bit = 1 << k;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      if (m & bit) continue;
      const df64 a = t[m], b = t[m | bit];
      t[m] = df_scale2(df_add(a, b), 0.5f);
      t[m | bit] = df_sub(b, a);
    }
  }
#pragma unroll
  for (int m = 0; m < 8; ++m) c[m] = t[m];
}

// evaluate trilinear coefficients at s (every monomial weight is a power of two or 0)
NALU_HD df64 trilinear_eval_df(const df64 c[8], const float s[3]) {
  df64 r = c[0];
#pragma unroll
  for (int m = 1; m < 8; ++m) {
    float w = 1.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (m & (1 << k)) w *= s[k];
    if (w != 0.0f) r = df_add(r, df_scale2(c[m], w));
  }
  return r;
}

// element-matrix accumulation for one ip: first touch of a row stores
template <class Acc>
NALU_HD void accumulate_ip_df(Acc& acc, int ip, const df64 fac[8]) {
  const int il = ip_left(ip), ir = ip_right(ip);
  const bool fl = first_ip_of_row(il) == ip;
  const bool fr = first_ip_of_row(ir) == ip;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    if (fl) acc.set(il, c, fac[c]); else acc.add(il, c, fac[c]);
    if (fr) acc.set(ir, c, df_neg(fac[c])); else acc.add(ir, c, df_neg(fac[c]));
  }
}

// ---------------------------------------------------------------------------
// ScalarDiffElemKernel in df64 (k given per node as df64)
// ---------------------------------------------------------------------------
// The element matrix comes out in normalised units: entries times 2^kexp
// are the physical ones (a diffusion matrix scales like a length).
template <bool SHIFT, class Acc>
NALU_HD double scalar_diff_lhs_df(const double x[8][3], const df64 k[8], Acc& acc, int& kexp) {
  EdgeFormDF f;
  {
    df64 d[8][3];
    kexp = rel_coords_df(x, d);
    edge_form_df(d, f);
  }
  df64 kc[8];
  trilinear_coeffs_df(k, kc);
  float mindet = 3.0e38f;
#pragma unroll 1
  for (int ip = 0; ip < 12; ++ip) {
    IpGeomDF g;
    ip_geometry_df(f, ip, g);
    df64 G[3] = {g.G[0], g.G[1], g.G[2]};
    df64 det = g.det;
    if (SHIFT) ip_shifted_G_df(f, ip, g.area, G, det);
    mindet = fminf(mindet, det.hi);
    float s[3];
    ip_location(ip, 0.25f, s);
    const df64 kIp = trilinear_eval_df(kc, s);
    float sg[3];
    ip_location(ip, SHIFT ? 0.5f : 0.25f, sg);
    df64 fac[8];
    lhs_factors_df(G, df_neg(df_mul(kIp, df_rcp(det))), sg, fac);
    accumulate_ip_df(acc, ip, fac);
  }
  return f2d_bits(mindet);
}

// ---------------------------------------------------------------------------
// ContinuityAdvElemKernel in df64 (MODE as in hex8_elem.h).  The caller adds
// -lhs . p in FP64 for MODE 0/2.  Normalised units: lhs entries times
// 2^kexp and rhs entries (mass flow rates, area-scaled) times 2^(2 kexp) are
// the physical ones.
// ---------------------------------------------------------------------------
template <int MODE, bool SMDOT, class Acc>
NALU_HD double continuity_elem_df(const double x[8][3], const df64 w[8][3], df64 inv_tau, const df64 p[8],
                                  Acc& acc, df64 rhs[8], int& kexp) {
  EdgeFormDF f;
  {
    df64 d[8][3];
    kexp = rel_coords_df(x, d);
    edge_form_df(d, f);
  }
  const float inv_len = pow2f(-kexp);  // the length-scaled pressure term joins an area-scaled flux
  df64 wc[3][8];
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    df64 v[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) v[n] = w[n][comp];
    trilinear_coeffs_df(v, wc[comp]);
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) acc.rset(r, df_zero());
  float mindet = 3.0e38f;
#pragma unroll 1
  for (int ip = 0; ip < 12; ++ip) {
    IpGeomDF g;
    ip_geometry_df(f, ip, g);
    mindet = fminf(mindet, g.det.hi);
    df64 fac[8];
    float s_std[3], s_sh[3];
    ip_location(ip, 0.25f, s_std);
    ip_location(ip, 0.5f, s_sh);
    if (MODE == 0) {
      lhs_factors_df(g.G, df_neg(df_rcp(g.det)), s_std, fac);
    } else {
      df64 Gs[3], dets;
      ip_shifted_G_df(f, ip, g.area, Gs, dets);
      mindet = fminf(mindet, dets.hi);
      lhs_factors_df(Gs, df_neg(df_rcp(dets)), s_sh, fac);
    }
    accumulate_ip_df(acc, ip, fac);
    const float* sm = SMDOT ? s_sh : s_std;
    const df64 wx = trilinear_eval_df(wc[0], sm);
    const df64 wy = trilinear_eval_df(wc[1], sm);
    const df64 wz = trilinear_eval_df(wc[2], sm);
    df64 m = df_mul(df_dot3(wx, g.area[0], wy, g.area[1], wz, g.area[2]), inv_tau);
    if (MODE == 1) {
      df64 fs[8];
      lhs_factors_df(g.G, df_neg(df_rcp(g.det)), s_std, fs);
      df64 dpa = df_zero();
#pragma unroll
      for (int c = 0; c < 8; ++c) dpa = df_fma(fs[c], p[c], dpa);
      m = df_add(m, df_scale2(dpa, inv_len));
    }
    // rhs[il] -= m ; rhs[ir] += m, accumulated beside the element matrix
    // (runtime row index; registers cannot be indexed at run time)
    acc.radd(ip_left(ip), df_neg(m));
    acc.radd(ip_right(ip), m);
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) rhs[r] = acc.rget(r);
  return f2d_bits(mindet);
}

// ---------------------------------------------------------------------------
// Mass flow rate at the SCS in df64 (ComputeMdotElemAlgorithm.C:200-245):
//   mdot_ip = (rho u + tau Gp)_ip . A - tau (dN/dx . A) . p
// SMDOT: shifted shape functions for the interpolation; SPOIS: shifted grad
// op for the pressure gradient.  Writes out[ip] (12 values) as FP64.
// ---------------------------------------------------------------------------
template <bool SMDOT, bool SPOIS>
NALU_HD double mdot_elem_df(const double x[8][3], const df64 w[8][3], const df64 p[8], df64 tau, double* out) {
  EdgeFormDF f;
  int kexp;
  {
    df64 d[8][3];
    kexp = rel_coords_df(x, d);
    edge_form_df(d, f);
  }
  const float inv_len = pow2f(-kexp);
  df64 wc[3][8];
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    df64 v[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) v[n] = w[n][comp];
    trilinear_coeffs_df(v, wc[comp]);
  }
  float mindet = 3.0e38f;
#pragma unroll 1
  for (int ip = 0; ip < 12; ++ip) {
    IpGeomDF g;
    ip_geometry_df(f, ip, g);
    mindet = fminf(mindet, g.det.hi);
    float s_std[3], s_sh[3];
    ip_location(ip, 0.25f, s_std);
    ip_location(ip, 0.5f, s_sh);
    const float* sm = SMDOT ? s_sh : s_std;
    const df64 wx = trilinear_eval_df(wc[0], sm);
    const df64 wy = trilinear_eval_df(wc[1], sm);
    const df64 wz = trilinear_eval_df(wc[2], sm);
    const df64 m0 = df_dot3(wx, g.area[0], wy, g.area[1], wz, g.area[2]);
    df64 fs[8];
    if (SPOIS) {
      df64 Gs[3], dets;
      ip_shifted_G_df(f, ip, g.area, Gs, dets);
      mindet = fminf(mindet, dets.hi);
      lhs_factors_df(Gs, df_rcp(dets), s_sh, fs);  // = dN_c/dx . A
    } else {
      lhs_factors_df(g.G, df_rcp(g.det), s_std, fs);
    }
    df64 dpa = df_zero();
#pragma unroll
    for (int c = 0; c < 8; ++c) dpa = df_fma(fs[c], p[c], dpa);
    out[ip] = df_to_double_bits(df_sub(m0, df_scale2(df_mul(tau, dpa), inv_len)), 2 * kexp);
  }
  return f2d_bits(mindet);
}

// plain array accumulator (host check)
struct ArrayAccDF {
  df64* m;
  df64* rhs;  // [8], used by the continuity kernel
  NALU_HD void set(int r, int c, df64 v) { m[r * 8 + c] = v; }
  NALU_HD void add(int r, int c, df64 v) { m[r * 8 + c] = df_add(m[r * 8 + c], v); }
  NALU_HD void rset(int r, df64 v) { rhs[r] = v; }
  NALU_HD void radd(int r, df64 v) { rhs[r] = df_add(rhs[r], v); }
  NALU_HD df64 rget(int r) const { return rhs[r]; }
};

}  // namespace nalu_gb300
