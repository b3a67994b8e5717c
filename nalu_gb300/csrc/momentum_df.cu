// momentum_df.cu -- the 24x24 momentum element kernels
// (MomentumAdvDiffElemKernel, src/kernel/MomentumAdvDiffElemKernel.C:72-185;
// MomentumUpwAdvDiffElemKernel, src/kernel/MomentumUpwAdvDiffElemKernel.C:90-320)
// with the element math in double-float (FP32-pair) arithmetic.
//
// Same three phases and the same summation order as momentum.cu:
//   0. gather: coordinates relative to node 0 of the element (FP64
//      differences, then split), nodal fields split into FP32 pairs; nine
//      threads per element form the edge-form Jacobian coefficients;
//   1. one thread per (element, SCS ip): Jacobian from the edge form,
//      cofactors, area vector, grad op, the per-ip sums and the upwind /
//      Peclet blending of the blended kernel;
//   2. one thread per (element, matrix row): the 24 entries summed over the
//      row node's three ips, converted to FP64 and scattered.
// Shape-function values and derivatives at the ip locations are products of
// 1/2 +- s with s in {0, +-1/4, +-1/2}: exact in FP32.
#include <cuda_runtime.h>

#include <cstdint>

#include "hex8_elem_df.h"
#include "internal.h"
#include "momentum.cuh"

namespace nalu_gb300 {
namespace {

// shared-memory layout per element in df64 words: MomLayout, then the edge
// form, padded so that the element stride (2 SIZE 32-bit words) is 2 mod 32:
// equal offsets of the 16 elements of a block fall in different banks
struct MomLayoutDF {
  static constexpr int EF = MomLayout::ALHS + 24;  // [k][i][A,B,C,D]
  static constexpr int SIZE = EF + 36 + 1;    // 689
};
static_assert((2 * MomLayoutDF::SIZE) % 32 == 2, "element stride");

__device__ __forceinline__ float shape_f(int n, const float s[3]) {
  return (0.5f + (float)corner_sign(n, 0) * s[0]) * (0.5f + (float)corner_sign(n, 1) * s[1]) *
         (0.5f + (float)corner_sign(n, 2) * s[2]);
}
__device__ __forceinline__ float dshape_f(int n, int k, const float s[3]) {
  float v = (float)corner_sign(n, k);
#pragma unroll
  for (int m = 0; m < 3; ++m)
    if (m != k) v *= 0.5f + (float)corner_sign(n, m) * s[m];
  return v;
}
__device__ __forceinline__ int node_of_rt(int s0, int s1, int s2) {
  // STK Hex8 numbering from corner signs (runtime form of node_of)
  const int lo = s1 < 0 ? (s0 < 0 ? 0 : 1) : (s0 < 0 ? 3 : 2);
  return lo + (s2 < 0 ? 0 : 4);
}

// edge-form coefficients of column k, component i (the bilinear interpolation
// of the four element edges along axis k): J[i][k](s) = A + B s_u + C s_v + D s_u s_v
__device__ void edge_entry_df(const df64* X, int k, int i, df64* out) {
  const int u = (k == 0) ? 1 : 0, v = (k == 2) ? 1 : 2;
  df64 e[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int sg[3];
    sg[u] = (q & 1) ? 1 : -1;
    sg[v] = (q & 2) ? 1 : -1;
    sg[k] = -1;
    const int a = node_of_rt(sg[0], sg[1], sg[2]);
    sg[k] = 1;
    const int b = node_of_rt(sg[0], sg[1], sg[2]);
    e[q] = df_sub(X[3 * b + i], X[3 * a + i]);
  }
  const df64 p01 = df_add(e[0], e[1]), m01 = df_sub(e[1], e[0]);
  const df64 p23 = df_add(e[2], e[3]), m23 = df_sub(e[3], e[2]);
  out[0] = df_scale2(df_add(p01, p23), 0.25f);
  out[1] = df_scale2(df_add(m01, m23), 0.5f);
  out[2] = df_scale2(df_sub(p23, p01), 0.5f);
  out[3] = df_sub(m23, m01);
}

// J at location s from the edge form in shared memory
__device__ void jacobian_ef_df(const df64* EF, const float s[3], df64 j[3][3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int u = (k == 0) ? 1 : 0, v = (k == 2) ? 1 : 2;
    const float su = s[u], sv = s[v];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const df64* c = EF + 4 * (3 * k + i);
      df64 r = c[0];
      if (su != 0.0f) r = df_add(r, df_mul_f(c[1], su));
      if (sv != 0.0f) r = df_add(r, df_mul_f(c[2], sv));
      if (su != 0.0f && sv != 0.0f) r = df_add(r, df_mul_f(c[3], su * sv));
      j[i][k] = r;
    }
  }
}

__device__ __forceinline__ double dbl(df64 v) { return df_to_double_bits(v); }
__device__ __forceinline__ df64 spl(double v) { return df_split_bits(v); }
__device__ __forceinline__ df64 df_div(df64 a, df64 b) { return df_mul(a, df_rcp(b)); }
__device__ __forceinline__ df64 df_abs(df64 a) { return a.hi < 0.0f ? df_neg(a) : a; }

template <bool UPW, bool SHIFT, bool SKEW, int OUT>
__global__ void __launch_bounds__(kMomThreads) k_assemble_momentum_df(MomArgs a) {
  extern __shared__ df64 smd[];
  __shared__ int s_nodes[kMomElems][8];
  __shared__ int64_t s_elem[kMomElems];
  __shared__ int s_kexp[kMomElems][8];  // per node: exponent of its largest coordinate difference
  const int t = threadIdx.x;
  const int el = t / 12, sub = t % 12;
  const int64_t gi = (int64_t)blockIdx.x * kMomElems + el;
  const bool valid = gi < a.count;
  df64* S = smd + el * MomLayoutDF::SIZE;

  // ---- phase 0: gather ----
  // Coordinates relative to node 0 are normalised by 2^-k, 2^k bounding the
  // element's largest difference (as rel_coords_df): the geometry then runs on
  // O(1) numbers, and areas (x 2^2k), grad ops (x 2^-k) and lengths (x 2^k)
  // return to physical units right after it.
  double dxv[3] = {0.0, 0.0, 0.0};
  if (valid) {
    const int64_t e = (OUT == 2) ? a.cap_elem : (a.elems ? (int64_t)a.elems[gi] : gi);
    if (sub == 0) s_elem[el] = e;
    if (sub < 8) {
      const int n = __ldg(a.conn + 8 * e + sub);
      const int n0 = __ldg(a.conn + 8 * e);
      s_nodes[el][sub] = n;
      int emax = -1023;
      for (int d = 0; d < 3; ++d) {
        dxv[d] = sub == 0 ? 0.0 : __ldg(a.x + 3 * (int64_t)n + d) - __ldg(a.x + 3 * (int64_t)n0 + d);
        emax = max(emax, dexp(dxv[d]));
        S[MomLayout::U + 3 * sub + d] = spl(__ldg(a.u + 3 * (int64_t)n + d));
      }
      s_kexp[el][sub] = emax;
      S[MomLayout::MU + sub] = spl(__ldg(a.mu + n));
      if (UPW) {
        for (int d = 0; d < 3; ++d) S[MomLayout::VR + 3 * sub + d] = spl(__ldg(a.vrtm + 3 * (int64_t)n + d));
        S[MomLayout::RHO + sub] = spl(__ldg(a.rho + n));
        for (int k = 0; k < 9; ++k) S[MomLayout::GJU + 9 * sub + k] = spl(__ldg(a.gju + 9 * (int64_t)n + k));
      }
    }
    S[MomLayout::MD + sub] = spl(__ldg(a.mdot + 12 * e + sub));
  }
  __syncthreads();
  int kexp = 0;
  if (valid) {
    int emax = s_kexp[el][0];
#pragma unroll
    for (int q = 1; q < 8; ++q) emax = max(emax, s_kexp[el][q]);
    kexp = min(max(emax, -kNormExpMax), kNormExpMax);
    if (sub < 8)
      for (int d = 0; d < 3; ++d) S[MomLayout::X + 3 * sub + d] = df_split_bits(dxv[d], kexp);
  }
  __syncthreads();
  if (valid && sub < 9) edge_entry_df(S + MomLayout::X, sub / 3, sub % 3, S + MomLayoutDF::EF + 4 * sub);
  __syncthreads();

  // ---- phase 1: per ip ----
  if (valid) {
    const int ip = sub;
    float s[3], g[3], av[3];
    ip_location(ip, 0.25f, s);
    const df64* X = S + MomLayout::X;
    const df64* EF = S + MomLayoutDF::EF;
    df64 j[3][3], adj[3][3], det;
    jacobian_ef_df(EF, s, j);
    cofactor_df(j, adj, det);
    const int dd = ip_dir(ip);
    const float sg4 = (ip < 8 && (ip & 3) == 2) ? -0.25f : 0.25f;
    df64 A[3];  // physical area vector: normalised cofactor column x 2^2k
    const float sgA = sg4 * pow2f(2 * kexp);
#pragma unroll
    for (int i = 0; i < 3; ++i) A[i] = df_scale2(dd == 0 ? adj[i][0] : (dd == 1 ? adj[i][1] : adj[i][2]), sgA);
    float mindet = det.hi;
#pragma unroll
    for (int k = 0; k < 3; ++k) g[k] = s[k];
    if (SHIFT) {
      ip_location(ip, 0.5f, g);
      jacobian_ef_df(EF, g, j);
      cofactor_df(j, adj, det);
      mindet = fminf(mindet, det.hi);
    }
    if (!(mindet > 1.0e-37f)) atomicAdd(a.flags + FLAG_NEG_JAC, 1);  // det <= 0 (or below FP32 range)
    const df64 inv = df_scale2(df_rcp(det), pow2f(-kexp));  // adj / det in physical units (x 2^-k)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) adj[i][k] = df_mul(adj[i][k], inv);
    df64* DN = S + MomLayout::DNDX + 24 * ip;
    const df64* Un = S + MomLayout::U;
    const df64* MUn = S + MomLayout::MU;
    const df64 tmdot = S[MomLayout::MD + ip];
    ip_location(ip, SKEW ? 0.5f : 0.25f, av);
    df64 muIp = df_zero(), uIp[3] = {df_zero(), df_zero(), df_zero()}, cIp[3] = {df_zero(), df_zero(), df_zero()};
    df64 divU = df_zero(), dA[8], vr[3] = {df_zero(), df_zero(), df_zero()};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float d0 = dshape_f(c, 0, g), d1 = dshape_f(c, 1, g), d2 = dshape_f(c, 2, g);
      df64 dn[3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
        dn[i] = df_add(df_add(df_mul_f(adj[i][0], d0), df_mul_f(adj[i][1], d1)), df_mul_f(adj[i][2], d2));
      DN[3 * c] = dn[0];
      DN[3 * c + 1] = dn[1];
      DN[3 * c + 2] = dn[2];
      const float r = shape_f(c, s), rAdv = shape_f(c, av);
      muIp = df_add(muIp, df_mul_f(MUn[c], r));
      const df64 uc0 = Un[3 * c], uc1 = Un[3 * c + 1], uc2 = Un[3 * c + 2];
      uIp[0] = df_add(uIp[0], df_mul_f(uc0, rAdv));
      uIp[1] = df_add(uIp[1], df_mul_f(uc1, rAdv));
      uIp[2] = df_add(uIp[2], df_mul_f(uc2, rAdv));
      if (UPW) {
        cIp[0] = df_add(cIp[0], df_mul_f(X[3 * c], rAdv));
        cIp[1] = df_add(cIp[1], df_mul_f(X[3 * c + 1], rAdv));
        cIp[2] = df_add(cIp[2], df_mul_f(X[3 * c + 2], rAdv));
      }
      divU = df_fma(uc2, dn[2], df_fma(uc1, dn[1], df_fma(uc0, dn[0], divU)));
      dA[c] = df_dot3(dn[0], A[0], dn[1], A[1], dn[2], A[2]);
      const df64 Au = df_dot3(A[0], uc0, A[1], uc1, A[2], uc2);
      vr[0] = df_fma(dA[c], uc0, df_fma(dn[0], Au, vr[0]));
      vr[1] = df_fma(dA[c], uc1, df_fma(dn[1], Au, vr[1]));
      vr[2] = df_fma(dA[c], uc2, df_fma(dn[2], Au, vr[2]));
    }
    const df64 nmu = df_neg(muIp);
    df64* AA = S + MomLayout::AA + 3 * ip;
    AA[0] = df_mul(nmu, A[0]);
    AA[1] = df_mul(nmu, A[1]);
    AA[2] = df_mul(nmu, A[2]);
    df64 advscale = df64{1.0f, 0.0f};
    df64 aflux[3] = {df_mul(tmdot, uIp[0]), df_mul(tmdot, uIp[1]), df_mul(tmdot, uIp[2])};
    df64 alhsL = df_zero(), alhsR = df_zero();
    if (UPW) {
      // upwind / central blending (MomentumUpwAdvDiffElemKernel.C, classic Peclet
      // function, optional van Leer limiter), in FP32 pairs like the rest
      const int il = ip_left(ip), ir = ip_right(ip);
      const df64 small_ = spl(1.0e-16);
      const df64* VR = S + MomLayout::VR;
      const df64* RHO = S + MomLayout::RHO;
      const df64* GJ = S + MomLayout::GJU;
      df64 udotx = df_zero(), duL[3], duR[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const df64 dxi = df_sub(X[3 * ir + i], X[3 * il + i]);
        const df64 ui = df_scale2(df_add(VR[3 * il + i], VR[3 * ir + i]), 0.5f);
        udotx = df_fma(ui, dxi, udotx);
        duL[i] = df_zero();
        duR[i] = df_zero();
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          duL[i] = df_fma(df_sub(cIp[jj], X[3 * il + jj]), GJ[9 * il + 3 * i + jj], duL[i]);
          duR[i] = df_fma(df_sub(X[3 * ir + jj], cIp[jj]), GJ[9 * ir + 3 * i + jj], duR[i]);
        }
      }
      const float len = pow2f(kexp);  // normalised lengths back to physical units
      udotx = df_scale2(udotx, len);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        duL[i] = df_scale2(duL[i], len);
        duR[i] = df_scale2(duR[i], len);
      }
      const df64 diffIp = df_scale2(df_add(df_div(MUn[il], RHO[il]), df_div(MUn[ir], RHO[ir])), 0.5f);
      const df64 pe = df_div(df_abs(udotx), df_add(diffIp, small_));
      const df64 mpe = df_mul(spl(a.hf), pe);
      const df64 mpe2 = df_mul(mpe, mpe);
      const df64 pecfac = df_div(mpe2, df_add(df64{5.0f, 0.0f}, mpe2));
      const df64 one = df64{1.0f, 0.0f};
      const df64 om_pecfac = df_sub(one, pecfac);
      const df64 alpha = spl(a.alpha), alpha_upw = spl(a.alpha_upw), upw = spl(a.upw);
      const df64 om_alpha = df_sub(one, alpha), om_alphaUpw = df_sub(one, alpha_upw);
      const bool pos = tmdot.hi > 0.0f;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        df64 limL = one, limR = one;
        const df64 uil = Un[3 * il + i], uir = Un[3 * ir + i];
        if (a.use_limiter) {
          const df64 dq = df_sub(uir, uil);
          const df64 dqMl = df_sub(df_scale2(duL[i], 4.0f), dq);
          const df64 dqMr = df_sub(df_scale2(duR[i], 4.0f), dq);
          const df64 pl = df_mul(dqMl, dq), pr = df_mul(dqMr, dq);
          const df64 sl = df_add(dqMl, dq), sr = df_add(dqMr, dq);
          limL = df_div(df_scale2(df_add(pl, df_abs(pl)), 2.0f), df_add(df_mul(sl, sl), small_));
          limR = df_div(df_scale2(df_add(pr, df_abs(pr)), 2.0f), df_add(df_mul(sr, sr), small_));
        }
        const df64 uL = df_fma(df_mul(duL[i], upw), limL, uil);
        const df64 uR = df_sub(uir, df_mul(df_mul(duR[i], upw), limR));
        const df64 uiUpw = df_fma(om_alphaUpw, uIp[i], df_mul(alpha_upw, pos ? uL : uR));
        const df64 hatL = df_fma(om_alpha, uIp[i], df_mul(alpha, uL));
        const df64 hatR = df_fma(om_alpha, uIp[i], df_mul(alpha, uR));
        const df64 uCds = df_scale2(df_add(hatL, hatR), 0.5f);
        aflux[i] = df_mul(tmdot, df_fma(om_pecfac, uCds, df_mul(pecfac, uiUpw)));
      }
      const df64 atm = df_abs(tmdot);
      const df64 cen = df_mul(df_scale2(df_mul(alpha, om_pecfac), 0.5f), tmdot);
      alhsL = df_fma(df_scale2(df_add(tmdot, atm), 0.5f), df_mul(pecfac, alpha_upw), cen);
      alhsR = df_fma(df_scale2(df_sub(tmdot, atm), 0.5f), df_mul(pecfac, alpha_upw), cen);
      advscale = df_fma(om_pecfac, om_alpha, df_mul(pecfac, om_alphaUpw));
    }
    df64* DG = S + MomLayout::DIAG + 8 * ip;
    const df64 tmsc = UPW ? df_mul(tmdot, advscale) : tmdot;
#pragma unroll
    for (int c = 0; c < 8; ++c) DG[c] = df_fma(nmu, dA[c], df_mul_f(tmsc, shape_f(c, av)));
    df64* RI = S + MomLayout::RIP + 3 * ip;
    const df64 dstress = spl(2.0 / 3.0 * dbl(muIp) * dbl(divU) * a.include_divu);
#pragma unroll
    for (int i = 0; i < 3; ++i) RI[i] = df_fma(nmu, vr[i], df_fma(dstress, A[i], aflux[i]));
    S[MomLayout::ALHS + 2 * ip] = alhsL;
    S[MomLayout::ALHS + 2 * ip + 1] = alhsR;
  }
  __syncthreads();

  // ---- phase 2: rows; each thread owns rows sub and sub+12 of its element.
  // The entries accumulate as unnormalised pairs (lazy products and sums);
  // the widening to FP64 renormalises them ----
  if (!valid) return;
  for (int h = 0; h < 2; ++h) {
    const int row = sub + 12 * h;  // = 3 r + i
    const int r = row / 3, i = row % 3;
    df64 v[8][3];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c][0] = v[c][1] = v[c][2] = df_zero();
    df64 rs = df_zero();
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int ip = node_ip(r, k);
      const int il = ip_left(ip), ir = ip_right(ip);
      const bool left = il == r;
      const df64* DN = S + MomLayout::DNDX + 24 * ip;
      const df64* AA = S + MomLayout::AA + 3 * ip;
      const df64* DG = S + MomLayout::DIAG + 8 * ip;
      const df64 aa0 = left ? AA[0] : df_neg(AA[0]), aa1 = left ? AA[1] : df_neg(AA[1]),
                 aa2 = left ? AA[2] : df_neg(AA[2]);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const df64 di = DN[3 * c + i];
        v[c][0] = df_fma_lazy(di, aa0, v[c][0]);
        v[c][1] = df_fma_lazy(di, aa1, v[c][1]);
        v[c][2] = df_fma_lazy(di, aa2, v[c][2]);
        const df64 dg = left ? DG[c] : df_neg(DG[c]);
        if (i == 0) v[c][0] = df_add_lazy(v[c][0], dg);
        else if (i == 1) v[c][1] = df_add_lazy(v[c][1], dg);
        else v[c][2] = df_add_lazy(v[c][2], dg);
      }
      if (UPW) {
        const df64 aL = S[MomLayout::ALHS + 2 * ip], aR = S[MomLayout::ALHS + 2 * ip + 1];
        const df64 sL = left ? aL : df_neg(aL), sR = left ? aR : df_neg(aR);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          if (c == il) {
            if (i == 0) v[c][0] = df_add_lazy(v[c][0], sL);
            else if (i == 1) v[c][1] = df_add_lazy(v[c][1], sL);
            else v[c][2] = df_add_lazy(v[c][2], sL);
          }
          if (c == ir) {
            if (i == 0) v[c][0] = df_add_lazy(v[c][0], sR);
            else if (i == 1) v[c][1] = df_add_lazy(v[c][1], sR);
            else v[c][2] = df_add_lazy(v[c][2], sR);
          }
        }
      }
      const df64 ri = S[MomLayout::RIP + 3 * ip + i];
      rs = df_add_lazy(rs, left ? df_neg(ri) : ri);
    }
    if (OUT == 2) {
#pragma unroll
      for (int c = 0; c < 8; ++c)
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) a.cap_lhs[row * 24 + 3 * c + jj] = dbl(v[c][jj]);
      a.cap_rhs[row] = dbl(rs);
      continue;
    }
    const int64_t e = s_elem[el];
    const int64_t grow = 3 * (int64_t)s_nodes[el][r] + i;
    const int64_t base = __ldg(a.rowptr + grow);
    const uint2 o2 = __ldg(reinterpret_cast<const uint2*>(a.slots + 64 * e + 8 * r));
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const uint32_t word = c < 4 ? o2.x : o2.y;
      const int off = (word >> (8 * (c & 3))) & 0xff;
      double* dst = a.values + base + 3 * off;
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) {
        if (OUT == 0) atomicAdd(dst + jj, dbl(v[c][jj]));
        else dst[jj] += dbl(v[c][jj]);
      }
    }
    if (OUT == 0) atomicAdd(a.rhs + grow, dbl(rs));
    else a.rhs[grow] += dbl(rs);
  }
}

template <bool UPW, bool SHIFT, bool SKEW, int OUT>
void launch_mom_df_variant(nalu_ctx* ctx, const MomArgs& a, int64_t count) {
  const size_t smem = sizeof(df64) * MomLayoutDF::SIZE * kMomElems;
  cudaFuncSetAttribute(k_assemble_momentum_df<UPW, SHIFT, SKEW, OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  const unsigned grid = (unsigned)((count + kMomElems - 1) / kMomElems);
  if (grid == 0) return;
  k_assemble_momentum_df<UPW, SHIFT, SKEW, OUT><<<grid, kMomThreads, smem, ctx->stream>>>(a);
  ctx->launches++;
}

template <int OUT>
void launch_mom_df_out(nalu_ctx* ctx, bool upw, bool shift, bool skew, const MomArgs& a, int64_t count) {
  if (upw) {
    if (shift) {
      if (skew) launch_mom_df_variant<true, true, true, OUT>(ctx, a, count);
      else launch_mom_df_variant<true, true, false, OUT>(ctx, a, count);
    } else {
      if (skew) launch_mom_df_variant<true, false, true, OUT>(ctx, a, count);
      else launch_mom_df_variant<true, false, false, OUT>(ctx, a, count);
    }
  } else {
    if (shift) {
      if (skew) launch_mom_df_variant<false, true, true, OUT>(ctx, a, count);
      else launch_mom_df_variant<false, true, false, OUT>(ctx, a, count);
    } else {
      if (skew) launch_mom_df_variant<false, false, true, OUT>(ctx, a, count);
      else launch_mom_df_variant<false, false, false, OUT>(ctx, a, count);
    }
  }
}

}  // namespace

int launch_momentum_df(nalu_ctx* ctx, int kernel, const MomArgs& a, int scatter, int64_t cap_elem, bool shift,
                       bool skew) {
  const bool upw = kernel == NALU_KERNEL_MOMENTUM_UPW_ADV_DIFF;
  if (cap_elem >= 0) {
    MomArgs ac = a;
    ac.count = 1;
    launch_mom_df_out<2>(ctx, upw, shift, skew, ac, 1);
  } else if (scatter == NALU_SCATTER_COLOURED) {
    const int nc = (int)ctx->colour_offsets.size() - 1;
    for (int c = 0; c < nc; ++c) {
      MomArgs ac = a;
      ac.elems = ctx->d_colour_elems.p + ctx->colour_offsets[c];
      ac.count = ctx->colour_offsets[c + 1] - ctx->colour_offsets[c];
      launch_mom_df_out<1>(ctx, upw, shift, skew, ac, ac.count);
    }
  } else {
    MomArgs ac = a;
    ac.count = ctx->n_elems;
    launch_mom_df_out<0>(ctx, upw, shift, skew, ac, ac.count);
  }
  return cuda_check(ctx, cudaGetLastError(), "momentum (df64) launch");
}

}  // namespace nalu_gb300
