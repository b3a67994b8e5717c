// momentum.cu -- sm_103a kernels for the 24x24 Hex8 momentum element
// matrices: MomentumAdvDiffElemKernel (src/kernel/MomentumAdvDiffElemKernel.C:72-185)
// and MomentumUpwAdvDiffElemKernel (src/kernel/MomentumUpwAdvDiffElemKernel.C:90-320),
// fused with the gather and with LinearSystem::sumInto for numDof = 3
// (sum_into_row_vec_3, src/TpetraLinearSystem.C:1378-1414).
//
// A block owns kMomElems elements and works in three phases:
//   0. gather node data of its elements into shared memory;
//   1. one thread per (element, SCS ip): Jacobian, area vector, grad op and
//      the per-ip factors of the element matrix and residual;
//   2. one thread per (element, matrix row): sums the three ips adjacent to
//      the row's node and scatters the 24 entries into the CRS row.
// The residual uses  rhs(row) = -sum_ip (aflux + divU stress + viscous flux),
// exactly the reference's rhs updates regrouped per ip.
#include <cuda_runtime.h>

#include <cstdint>

#include "hex8_elem.h"
#include "internal.h"
#include "momentum.cuh"

namespace nalu_gb300 {

template <bool UPW, bool SHIFT, bool SKEW, int OUT>
__global__ void __launch_bounds__(kMomThreads) k_assemble_momentum(MomArgs a) {
  extern __shared__ double sm[];
  __shared__ int s_nodes[kMomElems][8];
  __shared__ int64_t s_elem[kMomElems];
  const int t = threadIdx.x;
  const int el = t / 12, sub = t % 12;
  const int64_t gi = (int64_t)blockIdx.x * kMomElems + el;
  const bool valid = gi < a.count;
  double* S = sm + el * MomLayout::SIZE;

  // ---- phase 0: gather ----
  if (valid) {
    const int64_t e = (OUT == 2) ? a.cap_elem : (a.elems ? (int64_t)a.elems[gi] : gi);
    if (sub == 0) s_elem[el] = e;
    if (sub < 8) {
      const int n = __ldg(a.conn + 8 * e + sub);
      s_nodes[el][sub] = n;
      for (int d = 0; d < 3; ++d) {
        S[MomLayout::X + 3 * sub + d] = __ldg(a.x + 3 * (int64_t)n + d);
        S[MomLayout::U + 3 * sub + d] = __ldg(a.u + 3 * (int64_t)n + d);
      }
      S[MomLayout::MU + sub] = __ldg(a.mu + n);
      if (UPW) {
        for (int d = 0; d < 3; ++d) S[MomLayout::VR + 3 * sub + d] = __ldg(a.vrtm + 3 * (int64_t)n + d);
        S[MomLayout::RHO + sub] = __ldg(a.rho + n);
        for (int k = 0; k < 9; ++k) S[MomLayout::GJU + 9 * sub + k] = __ldg(a.gju + 9 * (int64_t)n + k);
      }
    }
    S[MomLayout::MD + sub] = __ldg(a.mdot + 12 * e + sub);
  }
  __syncthreads();

  // ---- phase 1: per ip ----
  if (valid) {
    const int ip = sub;
    const double s0 = ip_loc(ip, 0, 0.25), s1 = ip_loc(ip, 1, 0.25), s2 = ip_loc(ip, 2, 0.25);
    const double* X = S + MomLayout::X;
    double j[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double c0 = 0.0, c1 = 0.0, c2 = 0.0;
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        const double w = dshape(n, k, s0, s1, s2);
        c0 += w * X[3 * n];
        c1 += w * X[3 * n + 1];
        c2 += w * X[3 * n + 2];
      }
      j[0][k] = c0; j[1][k] = c1; j[2][k] = c2;
    }
    double adj[3][3], det;
    cofactor(j, adj, det);
    const int dd = ip_dir(ip);
    const double sg = 0.25 * ip_sign(ip);
    const double A[3] = {sg * adj[0][dd], sg * adj[1][dd], sg * adj[2][dd]};
    double mindet = det;
    // grad op (standard or shifted location)
    double g0 = s0, g1 = s1, g2 = s2;
    if (SHIFT) {
      g0 = ip_loc(ip, 0, 0.5); g1 = ip_loc(ip, 1, 0.5); g2 = ip_loc(ip, 2, 0.5);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double c0 = 0.0, c1 = 0.0, c2 = 0.0;
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          const double w = dshape(n, k, g0, g1, g2);
          c0 += w * X[3 * n];
          c1 += w * X[3 * n + 1];
          c2 += w * X[3 * n + 2];
        }
        j[0][k] = c0; j[1][k] = c1; j[2][k] = c2;
      }
      cofactor(j, adj, det);
      mindet = det < mindet ? det : mindet;
    }
    if (!(mindet > 1.0e-50)) atomicAdd(a.flags + FLAG_NEG_JAC, 1);
    const double inv = 1.0 / det;
    double* DN = S + MomLayout::DNDX + 24 * ip;
    const double* Un = S + MomLayout::U;
    const double* MUn = S + MomLayout::MU;
    const double tmdot = S[MomLayout::MD + ip];
    // ip values
    const double sa = SKEW ? 0.5 : 0.25;
    const double a0 = ip_loc(ip, 0, sa), a1 = ip_loc(ip, 1, sa), a2 = ip_loc(ip, 2, sa);
    double muIp = 0.0, uIp[3] = {0.0, 0.0, 0.0}, cIp[3] = {0.0, 0.0, 0.0}, divU = 0.0;
    double dA[8];
    double vr[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const double d0 = dshape(c, 0, g0, g1, g2), d1 = dshape(c, 1, g0, g1, g2), d2 = dshape(c, 2, g0, g1, g2);
      double dn[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) dn[i] = (adj[i][0] * d0 + adj[i][1] * d1 + adj[i][2] * d2) * inv;
      DN[3 * c] = dn[0]; DN[3 * c + 1] = dn[1]; DN[3 * c + 2] = dn[2];
      const double r = shape(c, s0, s1, s2);
      const double rAdv = shape(c, a0, a1, a2);
      muIp += r * MUn[c];
      const double uc0 = Un[3 * c], uc1 = Un[3 * c + 1], uc2 = Un[3 * c + 2];
      uIp[0] += rAdv * uc0; uIp[1] += rAdv * uc1; uIp[2] += rAdv * uc2;
      if (UPW) {
        cIp[0] += rAdv * X[3 * c]; cIp[1] += rAdv * X[3 * c + 1]; cIp[2] += rAdv * X[3 * c + 2];
      }
      divU += uc0 * dn[0] + uc1 * dn[1] + uc2 * dn[2];
      dA[c] = dn[0] * A[0] + dn[1] * A[1] + dn[2] * A[2];
      const double Au = A[0] * uc0 + A[1] * uc1 + A[2] * uc2;
      vr[0] += dn[0] * Au + dA[c] * uc0;
      vr[1] += dn[1] * Au + dA[c] * uc1;
      vr[2] += dn[2] * Au + dA[c] * uc2;
    }
    const double nmu = -muIp;
    double* AA = S + MomLayout::AA + 3 * ip;
    AA[0] = nmu * A[0]; AA[1] = nmu * A[1]; AA[2] = nmu * A[2];
    double advscale = 1.0;
    double aflux[3] = {tmdot * uIp[0], tmdot * uIp[1], tmdot * uIp[2]};
    double alhsL = 0.0, alhsR = 0.0;
    if (UPW) {
      const int il = ip_left(ip), ir = ip_right(ip);
      const double small_ = 1.0e-16;
      const double* VR = S + MomLayout::VR;
      const double* RHO = S + MomLayout::RHO;
      const double* GJ = S + MomLayout::GJU;
      double udotx = 0.0, duL[3], duR[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const double dxi = X[3 * ir + i] - X[3 * il + i];
        const double ui = 0.5 * (VR[3 * il + i] + VR[3 * ir + i]);
        udotx += ui * dxi;
        duL[i] = 0.0;
        duR[i] = 0.0;
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          duL[i] += (cIp[jj] - X[3 * il + jj]) * GJ[9 * il + 3 * i + jj];
          duR[i] += (X[3 * ir + jj] - cIp[jj]) * GJ[9 * ir + 3 * i + jj];
        }
      }
      const double diffIp = 0.5 * (MUn[il] / RHO[il] + MUn[ir] / RHO[ir]);
      const double pe = fabs(udotx) / (diffIp + small_);
      const double mpe = a.hf * pe;
      const double pecfac = mpe * mpe / (5.0 + mpe * mpe);
      const double om_pecfac = 1.0 - pecfac;
      const double om_alpha = 1.0 - a.alpha, om_alphaUpw = 1.0 - a.alpha_upw;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        double limL = 1.0, limR = 1.0;
        if (a.use_limiter) {
          const double dq = Un[3 * ir + i] - Un[3 * il + i];
          const double dqMl = 2.0 * 2.0 * duL[i] - dq;
          const double dqMr = 2.0 * 2.0 * duR[i] - dq;
          limL = (2.0 * (dqMl * dq + fabs(dqMl * dq))) / ((dqMl + dq) * (dqMl + dq) + small_);
          limR = (2.0 * (dqMr * dq + fabs(dqMr * dq))) / ((dqMr + dq) * (dqMr + dq) + small_);
        }
        const double uL = Un[3 * il + i] + duL[i] * a.upw * limL;
        const double uR = Un[3 * ir + i] - duR[i] * a.upw * limR;
        const double uiUpw = tmdot > 0 ? a.alpha_upw * uL + om_alphaUpw * uIp[i] : a.alpha_upw * uR + om_alphaUpw * uIp[i];
        const double hatL = a.alpha * uL + om_alpha * uIp[i];
        const double hatR = a.alpha * uR + om_alpha * uIp[i];
        const double uCds = 0.5 * (hatL + hatR);
        aflux[i] = tmdot * (pecfac * uiUpw + om_pecfac * uCds);
      }
      alhsL = 0.5 * (tmdot + fabs(tmdot)) * pecfac * a.alpha_upw + 0.5 * a.alpha * om_pecfac * tmdot;
      alhsR = 0.5 * (tmdot - fabs(tmdot)) * pecfac * a.alpha_upw + 0.5 * a.alpha * om_pecfac * tmdot;
      advscale = pecfac * om_alphaUpw + om_pecfac * om_alpha;
    }
    double* DG = S + MomLayout::DIAG + 8 * ip;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const double rAdv = shape(c, a0, a1, a2);
      DG[c] = rAdv * tmdot * advscale + nmu * dA[c];
    }
    double* RI = S + MomLayout::RIP + 3 * ip;
    const double dstress = 2.0 / 3.0 * muIp * divU * a.include_divu;
#pragma unroll
    for (int i = 0; i < 3; ++i) RI[i] = aflux[i] + dstress * A[i] + nmu * vr[i];
    S[MomLayout::ALHS + 2 * ip] = alhsL;
    S[MomLayout::ALHS + 2 * ip + 1] = alhsR;
  }
  __syncthreads();

  // ---- phase 2: rows; each thread owns rows sub and sub+12 of its element ----
  if (!valid) return;
  for (int h = 0; h < 2; ++h) {
    const int row = sub + 12 * h;  // = 3 r + i
    const int r = row / 3, i = row % 3;
    double v[8][3];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c][0] = v[c][1] = v[c][2] = 0.0;
    double rs = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int ip = node_ip(r, k);
      const int il = ip_left(ip), ir = ip_right(ip);
      const double sg = (il == r) ? 1.0 : -1.0;
      const double* DN = S + MomLayout::DNDX + 24 * ip;
      const double* AA = S + MomLayout::AA + 3 * ip;
      const double* DG = S + MomLayout::DIAG + 8 * ip;
      const double aa0 = sg * AA[0], aa1 = sg * AA[1], aa2 = sg * AA[2];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const double di = DN[3 * c + i];
        v[c][0] += di * aa0;
        v[c][1] += di * aa1;
        v[c][2] += di * aa2;
        v[c][i] += sg * DG[c];
      }
      if (UPW) {
        const double aL = S[MomLayout::ALHS + 2 * ip], aR = S[MomLayout::ALHS + 2 * ip + 1];
        v[il][i] += sg * aL;
        v[ir][i] += sg * aR;
      }
      rs -= sg * S[MomLayout::RIP + 3 * ip + i];
    }
    if (OUT == 2) {
#pragma unroll
      for (int c = 0; c < 8; ++c)
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) a.cap_lhs[row * 24 + 3 * c + jj] = v[c][jj];
      a.cap_rhs[row] = rs;
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
        if (OUT == 0) atomicAdd(dst + jj, v[c][jj]);
        else dst[jj] += v[c][jj];
      }
    }
    if (OUT == 0) atomicAdd(a.rhs + grow, rs);
    else a.rhs[grow] += rs;
  }
}

namespace {
template <bool UPW, bool SHIFT, bool SKEW, int OUT>
void launch_mom_variant(nalu_ctx* ctx, const MomArgs& a, int64_t count) {
  const size_t smem = sizeof(double) * MomLayout::SIZE * kMomElems;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_assemble_momentum<UPW, SHIFT, SKEW, OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    attr = true;
  }
  const unsigned grid = (unsigned)((count + kMomElems - 1) / kMomElems);
  if (grid == 0) return;
  k_assemble_momentum<UPW, SHIFT, SKEW, OUT><<<grid, kMomThreads, smem, ctx->stream>>>(a);
  ctx->launches++;
}

template <int OUT>
void launch_mom_out(nalu_ctx* ctx, bool upw, bool shift, bool skew, const MomArgs& a, int64_t count) {
  if (upw) {
    if (shift) { if (skew) launch_mom_variant<true, true, true, OUT>(ctx, a, count); else launch_mom_variant<true, true, false, OUT>(ctx, a, count); }
    else { if (skew) launch_mom_variant<true, false, true, OUT>(ctx, a, count); else launch_mom_variant<true, false, false, OUT>(ctx, a, count); }
  } else {
    if (shift) { if (skew) launch_mom_variant<false, true, true, OUT>(ctx, a, count); else launch_mom_variant<false, true, false, OUT>(ctx, a, count); }
    else { if (skew) launch_mom_variant<false, false, true, OUT>(ctx, a, count); else launch_mom_variant<false, false, false, OUT>(ctx, a, count); }
  }
}
}  // namespace

int launch_momentum(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int scatter, int64_t cap_elem,
                    double* cap_lhs, double* cap_rhs) {
  MomArgs a{};
  a.conn = ctx->d_conn.p;
  a.x = ctx->fields[NALU_FIELD_COORDINATES].d.p;
  a.u = ctx->fields[NALU_FIELD_VELOCITY].d.p;
  a.mu = ctx->fields[NALU_FIELD_VISCOSITY].d.p;
  a.mdot = ctx->fields[NALU_FIELD_MDOT_SCS].d.p;
  const bool upw = kernel == NALU_KERNEL_MOMENTUM_UPW_ADV_DIFF;
  if (upw) {
    a.vrtm = ctx->fields[NALU_FIELD_VELOCITY_RTM].d.p;
    a.rho = ctx->fields[NALU_FIELD_DENSITY].d.p;
    a.gju = ctx->fields[NALU_FIELD_DUDX].d.p;
  }
  a.include_divu = o.include_divu;
  a.alpha = o.alpha;
  a.alpha_upw = o.alpha_upw;
  a.upw = o.upw_factor;
  a.hf = o.hybrid_factor;
  a.use_limiter = o.use_limiter;
  a.rowptr = ctx->d_rowptr.p;
  a.slots = ctx->d_slots.p;
  a.values = ctx->d_values.p;
  a.rhs = ctx->d_rhs.p;
  a.flags = ctx->d_flags.p;
  const bool shift = o.shifted_grad_op != 0, skew = o.skew_symmetric != 0;
  if (o.arith == NALU_ARITH_DF64) {
    a.cap_elem = cap_elem;
    a.cap_lhs = cap_lhs;
    a.cap_rhs = cap_rhs;
    return launch_momentum_df(ctx, kernel, a, scatter, cap_elem, shift, skew);
  }
  if (cap_elem >= 0) {
    a.cap_elem = cap_elem;
    a.cap_lhs = cap_lhs;
    a.cap_rhs = cap_rhs;
    a.count = 1;
    launch_mom_out<2>(ctx, upw, shift, skew, a, 1);
  } else if (scatter == NALU_SCATTER_COLOURED) {
    const int nc = (int)ctx->colour_offsets.size() - 1;
    for (int c = 0; c < nc; ++c) {
      MomArgs ac = a;
      ac.elems = ctx->d_colour_elems.p + ctx->colour_offsets[c];
      ac.count = ctx->colour_offsets[c + 1] - ctx->colour_offsets[c];
      launch_mom_out<1>(ctx, upw, shift, skew, ac, ac.count);
    }
  } else {
    a.count = ctx->n_elems;
    launch_mom_out<0>(ctx, upw, shift, skew, a, a.count);
  }
  return cuda_check(ctx, cudaGetLastError(), "momentum launch");
}

}  // namespace nalu_gb300
