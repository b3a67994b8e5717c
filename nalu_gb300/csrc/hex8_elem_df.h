// hex8_elem_df.h -- the Hex8 element math of hex8_elem.h in double-float
// (df64) arithmetic on the FP32 pipes.
//
// Same formulation (edge-form Jacobian, areas from cofactor columns,
// lhs factors from adj(J)^T A), same summation order of the element matrix.
// Precision: coordinates enter as FP64 differences to node 0 of the element
// (so their full relative precision survives the split into hi + lo), nodal
// fields enter pre-split per node; every operation is an error-free-transform
// sequence with ~2^-48 relative rounding, i.e. about 32x the FP64 rounding
// unit, well inside the 1e-12 parity tolerance (checked on the CPU against the
// oracle by tests/test_elem_math.py and on the GPU by the parity tests).
#pragma once

#include "df64.h"
#include "hex8_elem.h"

namespace nalu_gb300 {

struct EdgeFormDF {
  df64 A[3][3], B[3][3], C[3][3], D[3][3];  // [k][component]
};

// x relative to node 0 (FP64 differences), split into df64
NALU_HD void rel_coords_df(const double x[8][3], df64 d[8][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) d[0][i] = df_zero();
#pragma unroll
  for (int n = 1; n < 8; ++n)
#pragma unroll
    for (int i = 0; i < 3; ++i) d[n][i] = df_from_double(x[n][i] - x[0][i]);
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

template <int IP, bool SHIFT>
NALU_HD void jacobian_ip_df(const EdgeFormDF& f, df64 j[3][3]) {
  constexpr double a = SHIFT ? 0.5 : 0.25;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int u = (k == 0) ? 1 : 0;
    const int v = (k == 2) ? 1 : 2;
    const double su = ip_loc(IP, u, a), sv = ip_loc(IP, v, a);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      df64 r = f.A[k][i];
      if (su != 0.0) r = df_add(r, df_scale2(f.B[k][i], (float)su));
      if (sv != 0.0) r = df_add(r, df_scale2(f.C[k][i], (float)sv));
      if (su * sv != 0.0) r = df_add(r, df_scale2(f.D[k][i], (float)(su * sv)));
      j[i][k] = r;
    }
  }
}

NALU_HD void cofactor_df(const df64 j[3][3], df64 adj[3][3], df64& det) {
  adj[0][0] = df_cross(j[1][1], j[2][2], j[2][1], j[1][2]);
  adj[0][1] = df_cross(j[1][2], j[2][0], j[2][2], j[1][0]);
  adj[0][2] = df_cross(j[1][0], j[2][1], j[2][0], j[1][1]);
  adj[1][0] = df_cross(j[0][2], j[2][1], j[2][2], j[0][1]);
  adj[1][1] = df_cross(j[0][0], j[2][2], j[2][0], j[0][2]);
  adj[1][2] = df_cross(j[0][1], j[2][0], j[2][1], j[0][0]);
  adj[2][0] = df_cross(j[0][1], j[1][2], j[1][1], j[0][2]);
  adj[2][1] = df_cross(j[0][2], j[1][0], j[1][2], j[0][0]);
  adj[2][2] = df_cross(j[0][0], j[1][1], j[1][0], j[0][1]);
  det = df_fma(j[2][0], adj[2][0], df_fma(j[1][0], adj[1][0], df_mul(j[0][0], adj[0][0])));
}

struct IpGeomDF {
  df64 area[3];
  df64 G[3];
  df64 det;
};

template <int IP>
NALU_HD void ip_geometry_df(const EdgeFormDF& f, IpGeomDF& g) {
  df64 j[3][3], adj[3][3], det;
  jacobian_ip_df<IP, false>(f, j);
  cofactor_df(j, adj, det);
  constexpr int dd = ip_dir(IP);
  constexpr float s = (float)(0.25 * ip_sign(IP));
#pragma unroll
  for (int i = 0; i < 3; ++i) g.area[i] = df_scale2(adj[i][dd], s);
#pragma unroll
  for (int jj = 0; jj < 3; ++jj)
    g.G[jj] = df_fma(adj[2][jj], g.area[2], df_fma(adj[1][jj], g.area[1], df_mul(adj[0][jj], g.area[0])));
  g.det = det;
}

template <int IP>
NALU_HD void ip_shifted_G_df(const EdgeFormDF& f, const df64 area[3], df64 G[3], df64& det) {
  df64 j[3][3], adj[3][3];
  jacobian_ip_df<IP, true>(f, j);
  cofactor_df(j, adj, det);
#pragma unroll
  for (int jj = 0; jj < 3; ++jj)
    G[jj] = df_fma(adj[2][jj], area[2], df_fma(adj[1][jj], area[1], df_mul(adj[0][jj], area[0])));
}

// fac[c] = sum_j dN_c/ds_j(ip) * (G_j * scale)
template <int IP, bool SHIFT>
NALU_HD void lhs_factors_df(const df64 G[3], df64 scale, df64 fac[8]) {
  constexpr double a = SHIFT ? 0.5 : 0.25;
  const df64 g0 = df_mul(G[0], scale), g1 = df_mul(G[1], scale), g2 = df_mul(G[2], scale);
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const double d0 = dshape_ip(IP, c, 0, a), d1 = dshape_ip(IP, c, 1, a), d2 = dshape_ip(IP, c, 2, a);
    df64 r = df_zero();
    bool first = true;
    if (d0 != 0.0) { r = df_mul_f(g0, (float)d0); first = false; }
    if (d1 != 0.0) { r = first ? df_mul_f(g1, (float)d1) : df_add(r, df_mul_f(g1, (float)d1)); first = false; }
    if (d2 != 0.0) { r = first ? df_mul_f(g2, (float)d2) : df_add(r, df_mul_f(g2, (float)d2)); first = false; }
    fac[c] = r;
  }
}

// Trilinear coefficients of a nodal scalar: f(s) = sum_m c_m s^m over the 8
// monomials {1, s1, s2, s1 s2, s3, s1 s3, s2 s3, s1 s2 s3} (index bit k set =
// factor s_{k+1}); nodal values live at the corners s = +-1/2.
NALU_HD void trilinear_coeffs_df(const df64 v[8], df64 c[8]) {
  // reorder corners to bit order: bit0 = s1 sign, bit1 = s2 sign, bit2 = s3 sign
  df64 t[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) t[m] = v[node_of((m & 1) ? 1 : -1, (m & 2) ? 1 : -1, (m & 4) ? 1 : -1)];
  // along each axis: f(-1/2) = a, f(+1/2) = b  ->  f(s) = (a+b)/2 + (b-a) s
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

// evaluate trilinear coefficients at an ip (location a = 1/4 or 1/2)
template <int IP, bool SHIFT>
NALU_HD df64 trilinear_eval_df(const df64 c[8]) {
  constexpr double a = SHIFT ? 0.5 : 0.25;
  const double s[3] = {ip_loc(IP, 0, a), ip_loc(IP, 1, a), ip_loc(IP, 2, a)};
  df64 r = c[0];
#pragma unroll
  for (int m = 1; m < 8; ++m) {
    double w = 1.0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (m & (1 << k)) w *= s[k];
    if (w != 0.0) r = df_add(r, df_scale2(c[m], (float)w));
  }
  return r;
}

// element matrix accumulator in df64 (first touch stores, later ips add)
template <int IP, class Acc>
NALU_HD void accumulate_ip_df(Acc& acc, const df64 fac[8]) {
  constexpr int il = ip_left(IP), ir = ip_right(IP);
  constexpr bool fl = first_ip_of_row(il) == IP;
  constexpr bool fr = first_ip_of_row(ir) == IP;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    if (fl) acc.set(il, c, fac[c]); else acc.add(il, c, fac[c]);
    if (fr) acc.set(ir, c, df_neg(fac[c])); else acc.add(ir, c, df_neg(fac[c]));
  }
}

// ---------------------------------------------------------------------------
// ScalarDiffElemKernel in df64: k given per node as df64
// ---------------------------------------------------------------------------
template <bool SHIFT, class Acc>
struct ScalarDiffBodyDF {
  const EdgeFormDF& f;
  const df64* kc;  // trilinear coefficients of the diffusion coefficient
  Acc& acc;
  double mindet;
  template <int IP>
  NALU_HD void apply() {
    IpGeomDF g;
    ip_geometry_df<IP>(f, g);
    df64 G[3] = {g.G[0], g.G[1], g.G[2]};
    df64 det = g.det;
    if (SHIFT) ip_shifted_G_df<IP>(f, g.area, G, det);
    const double dd = df_to_double(det);
    mindet = dd < mindet ? dd : mindet;
    const df64 kIp = trilinear_eval_df<IP, false>(kc);
    df64 fac[8];
    lhs_factors_df<IP, SHIFT>(G, df_neg(df_mul(kIp, df_rcp(det))), fac);
    accumulate_ip_df<IP>(acc, fac);
  }
};

template <bool SHIFT, class Acc>
NALU_HD double scalar_diff_lhs_df(const double x[8][3], const df64 k[8], Acc& acc) {
  EdgeFormDF f;
  {
    df64 d[8][3];
    rel_coords_df(x, d);
    edge_form_df(d, f);
  }
  df64 kc[8];
  trilinear_coeffs_df(k, kc);
  ScalarDiffBodyDF<SHIFT, Acc> body{f, kc, acc, 1.0e300};
  IpLoop<0, 12>::run(body);
  return body.mindet;
}

// ---------------------------------------------------------------------------
// ContinuityAdvElemKernel in df64 (MODE as in hex8_elem.h).  wc: trilinear
// coefficients of w = rho u + tau Gpdx per component; the caller adds
// -lhs . p in FP64 for MODE 0/2.
// ---------------------------------------------------------------------------
template <int MODE, bool SMDOT, class Acc>
struct ContinuityBodyDF {
  const EdgeFormDF& f;
  const df64 (*wc)[8];  // [3][8]
  df64 inv_tau;
  const double* p;
  Acc& acc;
  df64* rhs;
  double mindet;
  template <int IP>
  NALU_HD void apply() {
    IpGeomDF g;
    ip_geometry_df<IP>(f, g);
    constexpr int il = ip_left(IP), ir = ip_right(IP);
    double dd = df_to_double(g.det);
    mindet = dd < mindet ? dd : mindet;
    df64 fac[8];
    if (MODE == 0) {
      lhs_factors_df<IP, false>(g.G, df_neg(df_rcp(g.det)), fac);
    } else {
      df64 Gs[3], dets;
      ip_shifted_G_df<IP>(f, g.area, Gs, dets);
      dd = df_to_double(dets);
      mindet = dd < mindet ? dd : mindet;
      lhs_factors_df<IP, true>(Gs, df_neg(df_rcp(dets)), fac);
    }
    accumulate_ip_df<IP>(acc, fac);
    const df64 wx = trilinear_eval_df<IP, SMDOT>(wc[0]);
    const df64 wy = trilinear_eval_df<IP, SMDOT>(wc[1]);
    const df64 wz = trilinear_eval_df<IP, SMDOT>(wc[2]);
    df64 m = df_mul(df_fma(wz, g.area[2], df_fma(wy, g.area[1], df_mul(wx, g.area[0]))), inv_tau);
    if (MODE == 1) {
      df64 fs[8];
      lhs_factors_df<IP, false>(g.G, df_neg(df_rcp(g.det)), fs);
      df64 dpa = df_zero();
#pragma unroll
      for (int c = 0; c < 8; ++c) dpa = df_add(dpa, df_mul(fs[c], df_from_double(p[c])));
      m = df_add(m, dpa);
    }
    rhs[il] = df_sub(rhs[il], m);
    rhs[ir] = df_add(rhs[ir], m);
  }
};

template <int MODE, bool SMDOT, class Acc>
NALU_HD double continuity_elem_df(const double x[8][3], const df64 w[8][3], df64 inv_tau, const double p[8],
                                  Acc& acc, df64 rhs[8]) {
  EdgeFormDF f;
  {
    df64 d[8][3];
    rel_coords_df(x, d);
    edge_form_df(d, f);
  }
  df64 wc[3][8];
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    df64 v[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) v[n] = w[n][comp];
    trilinear_coeffs_df(v, wc[comp]);
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) rhs[r] = df_zero();
  ContinuityBodyDF<MODE, SMDOT, Acc> body{f, wc, inv_tau, p, acc, rhs, 1.0e300};
  IpLoop<0, 12>::run(body);
  return body.mindet;
}

// plain array accumulator (host check)
struct ArrayAccDF {
  df64* m;
  NALU_HD void set(int r, int c, df64 v) { m[r * 8 + c] = v; }
  NALU_HD void add(int r, int c, df64 v) { m[r * 8 + c] = df_add(m[r * 8 + c], v); }
};

}  // namespace nalu_gb300
