// mass.cu -- time terms of the continuity and momentum equations.
//
//   ContinuityMassElemKernel::execute (src/kernel/ContinuityMassElemKernel.C:84-120)
//     rhs(ip) -= (g1 rho^{n+1} + g2 rho^n + g3 rho^{n-1})_ip scV / dt / (dt / g1)
//   MomentumMassElemKernel::execute (src/kernel/MomentumMassElemKernel.C:100-171)
//     rhs(3 ip + j) -= (g1 rho^{n+1} u^{n+1} + g2 rho^n u^n + g3 rho^{n-1} u^{n-1})_j scV / dt
//                      + Gjp_j scV densFac
//     lhs(3 ip + j, 3 ic + j) += N_ic(ip) g1 rho^{n+1} scV / dt
//
// ip runs over the eight sub-control volumes; ip i belongs to node i
// (HexSCV::ipNodeMap), so every element row is produced by exactly one ip and
// one thread owns it.  Values at the ip come from the shape functions at the
// SCV centroids (+-1/4 in the [-1/2, 1/2] parent cube), or, lumped, at the
// nodes, where they are 1 at node ip and 0 elsewhere.  Each product rho_ip u_ip
// is formed from separately interpolated factors, as the reference does.
//
// Layout: 16 elements per 128-thread block, thread = (element, ip).  The
// element's nodal states go to shared memory; the SCV volume comes from the
// context's per-element volume cache (HexSCV::determinant of the current
// coordinates, refreshed when they change); the thread interpolates and
// scatters its row: for continuity
// only the rhs entry, for momentum 3 rows x 8 (lumped: 1) diagonal-block
// entries through the per-element slot table, FP64 atomics or, per colour,
// plain adds.
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace nalu_gb300 {
namespace {

constexpr int kMassElems = 16;

struct MassArgs {
  const int32_t* conn;
  const double* scv;     // [E][8] HexSCV volumes
  const int32_t* elems;  // element list of one colour, or null (all elements)
  int64_t count;
  const double* rho[3];  // states N-1, N, N+1
  const double* u[3];
  const double* gjp;
  double dt, g1, g2, g3;
  double dens_on, dens_off;  // densFac = rho^{n+1} dens_on + dens_off
  const int64_t* rowptr;
  const uint8_t* slots;
  double* values;
  double* rhs;
  int64_t cap_elem;
  double* cap_lhs;
  double* cap_rhs;
};

// N_c at the centroid of SCV ip: per axis 3/4 on the node's side, 1/4 across
__device__ __forceinline__ double scv_weight(int ip, int c) {
  const int diff = ip ^ c;
  // node bits: x flips between (0,1),(3,2); y = bit 1; z = bit 2
  const int xi = ((ip & 1) ^ ((ip >> 1) & 1)), xc = ((c & 1) ^ ((c >> 1) & 1));
  const double fx = xi == xc ? 0.75 : 0.25;
  const double fy = (diff & 2) ? 0.25 : 0.75;
  const double fz = (diff & 4) ? 0.25 : 0.75;
  return fx * fy * fz;
}

template <bool MOM, bool LUMPED, int OUT>
__global__ void __launch_bounds__(kMassElems * 8) k_assemble_mass(MassArgs a) {
  __shared__ double s_rho[kMassElems][3][8];
  __shared__ double s_u[MOM ? kMassElems : 1][3][8][3];
  __shared__ double s_g[MOM ? kMassElems : 1][8][3];
  const int el = threadIdx.x / 8, ip = threadIdx.x % 8;
  const int64_t k = OUT == 2 ? 0 : (int64_t)blockIdx.x * kMassElems + el;
  const bool valid = OUT == 2 ? el == 0 : k < a.count;
  int64_t e = 0;
  int node = 0;
  if (valid) {
    e = OUT == 2 ? a.cap_elem : (a.elems ? __ldg(a.elems + k) : k);
    node = __ldg(a.conn + 8 * e + ip);
#pragma unroll
    for (int t = 0; t < 3; ++t) s_rho[el][t][ip] = __ldg(a.rho[t] + node);
    if (MOM) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int t = 0; t < 3; ++t) s_u[el][t][ip][d] = __ldg(a.u[t] + 3 * (int64_t)node + d);
        s_g[el][ip][d] = __ldg(a.gjp + 3 * (int64_t)node + d);
      }
    }
  }
  __syncthreads();
  if (!valid) return;
  const double scV = __ldg(a.scv + 8 * e + ip);
  double r[3] = {0.0, 0.0, 0.0}, uu[3][3] = {}, g[3] = {0.0, 0.0, 0.0};
  if (LUMPED) {
#pragma unroll
    for (int t = 0; t < 3; ++t) r[t] = s_rho[el][t][ip];
    if (MOM) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int t = 0; t < 3; ++t) uu[t][d] = s_u[el][t][ip][d];
        g[d] = s_g[el][ip][d];
      }
    }
  } else {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const double w = scv_weight(ip, c);
#pragma unroll
      for (int t = 0; t < 3; ++t) r[t] += w * s_rho[el][t][c];
      if (MOM) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
#pragma unroll
          for (int t = 0; t < 3; ++t) uu[t][d] += w * s_u[el][t][c][d];
          g[d] += w * s_g[el][c][d];
        }
      }
    }
  }
  if (!MOM) {
    const double v = -(a.g1 * r[2] + a.g2 * r[1] + a.g3 * r[0]) * scV / a.dt / (a.dt / a.g1);
    if (OUT == 2) {
#pragma unroll
      for (int c = 0; c < 8; ++c) a.cap_lhs[ip * 8 + c] = 0.0;
      a.cap_rhs[ip] = v;
    } else if (OUT == 0) {
      atomicAdd(a.rhs + node, v);
    } else {
      a.rhs[node] += v;
    }
    return;
  }
  const double dens_fac = r[2] * a.dens_on + a.dens_off;
  const double lhs_base = a.g1 * r[2] * scV / a.dt;  // times N_ic(ip)
  uint2 o2 = make_uint2(0u, 0u);
  if (OUT != 2) o2 = __ldg(reinterpret_cast<const uint2*>(a.slots + 64 * e + 8 * ip));
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const double v = -(a.g1 * r[2] * uu[2][j] + a.g2 * r[1] * uu[1][j] + a.g3 * r[0] * uu[0][j]) * scV / a.dt -
                     g[j] * scV * dens_fac;
    const int row = 3 * ip + j;
    if (OUT == 2) {
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const double lf = LUMPED ? (c == ip ? lhs_base : 0.0) : scv_weight(ip, c) * lhs_base;
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) a.cap_lhs[row * 24 + 3 * c + jj] = jj == j ? lf : 0.0;
      }
      a.cap_rhs[row] = v;
      continue;
    }
    const int64_t grow = 3 * (int64_t)node + j;
    double* vrow = a.values + __ldg(a.rowptr + grow) + j;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (LUMPED && c != ip) continue;
      const uint32_t word = c < 4 ? o2.x : o2.y;
      const int off = (word >> (8 * (c & 3))) & 0xff;
      const double lf = LUMPED ? lhs_base : scv_weight(ip, c) * lhs_base;
      if (OUT == 0) atomicAdd(vrow + 3 * off, lf);
      else vrow[3 * off] += lf;
    }
    if (OUT == 0) atomicAdd(a.rhs + grow, v);
    else a.rhs[grow] += v;
  }
}

template <bool MOM, int OUT>
void launch_variant(nalu_ctx* ctx, bool lumped, const MassArgs& a, int64_t count) {
  const unsigned grid = (unsigned)((count + kMassElems - 1) / kMassElems);
  if (grid == 0) return;
  if (lumped) k_assemble_mass<MOM, true, OUT><<<grid, kMassElems * 8, 0, ctx->stream>>>(a);
  else k_assemble_mass<MOM, false, OUT><<<grid, kMassElems * 8, 0, ctx->stream>>>(a);
  ctx->launches++;
}

template <int OUT>
void launch_out(nalu_ctx* ctx, bool mom, bool lumped, const MassArgs& a, int64_t count) {
  if (mom) launch_variant<true, OUT>(ctx, lumped, a, count);
  else launch_variant<false, OUT>(ctx, lumped, a, count);
}

}  // namespace

int launch_mass(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int scatter, int64_t cap_elem,
                double* cap_lhs, double* cap_rhs) {
  const bool mom = kernel == NALU_KERNEL_MOMENTUM_MASS;
  int rc = ensure_scv_cache(ctx);
  if (rc) return rc;
  MassArgs a{};
  a.conn = ctx->d_conn.p;
  a.scv = ctx->d_scv.p;
  const Field& rn = ctx->fields[NALU_FIELD_DENSITY_N];
  const Field& rnm1 = ctx->fields[NALU_FIELD_DENSITY_NM1];
  a.rho[0] = rnm1.set ? rnm1.d.p : rn.d.p;
  a.rho[1] = rn.d.p;
  a.rho[2] = ctx->fields[NALU_FIELD_DENSITY].d.p;
  if (mom) {
    const Field& un = ctx->fields[NALU_FIELD_VELOCITY_N];
    const Field& unm1 = ctx->fields[NALU_FIELD_VELOCITY_NM1];
    a.u[0] = unm1.set ? unm1.d.p : un.d.p;
    a.u[1] = un.d.p;
    a.u[2] = ctx->fields[NALU_FIELD_VELOCITY].d.p;
    a.gjp = ctx->fields[NALU_FIELD_DPDX].d.p;
  }
  a.dt = o.dt;
  a.g1 = o.gamma1;
  a.g2 = o.gamma2;
  a.g3 = o.gamma3;
  a.dens_on = o.balanced_force ? 1.0 : 0.0;
  a.dens_off = o.balanced_force ? 0.0 : 1.0;
  a.rowptr = ctx->d_rowptr.p;
  a.slots = ctx->d_slots.p;
  a.values = ctx->d_values.p;
  a.rhs = ctx->d_rhs.p;
  const bool lumped = o.lumped_mass != 0;
  if (cap_elem >= 0) {
    a.cap_elem = cap_elem;
    a.cap_lhs = cap_lhs;
    a.cap_rhs = cap_rhs;
    a.count = 1;
    launch_out<2>(ctx, mom, lumped, a, 1);
  } else if (scatter == NALU_SCATTER_COLOURED) {
    const int nc = (int)ctx->colour_offsets.size() - 1;
    for (int c = 0; c < nc; ++c) {
      MassArgs ac = a;
      ac.elems = ctx->d_colour_elems.p + ctx->colour_offsets[c];
      ac.count = ctx->colour_offsets[c + 1] - ctx->colour_offsets[c];
      launch_out<1>(ctx, mom, lumped, ac, ac.count);
    }
  } else {
    a.count = ctx->n_elems;
    launch_out<0>(ctx, mom, lumped, a, a.count);
  }
  return cuda_check(ctx, cudaGetLastError(), "mass launch");
}

}  // namespace nalu_gb300
