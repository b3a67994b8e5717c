// geometry.cu -- nodal geometry and gradients on the Hex8 mesh.
//
//   dual nodal volume  ComputeGeometryInteriorAlgorithm
//                      (src/ComputeGeometryInteriorAlgorithm.C): the eight
//                      sub-control volumes of HexSCV::determinant
//                      (src/master_element/Hex8CVFEM.C:149-180), each the
//                      Grandy volume (Hex8GeometryFunctions.h:78-163) of a
//                      sub-hexahedron of the 27-point subdivision
//                      (:263-322), summed into their nodes
//   projected nodal    AssembleNodalGradElemAlgorithm
//   gradient           (src/AssembleNodalGradElemAlgorithm.C) and its
//                      velocity form (AssembleNodalGradUElemAlgorithm):
//                      grad[il] += qIp A / V_il, grad[ir] -= qIp A / V_ir
//
// Both are one-off geometry passes in FP64.  The volume kernel runs one
// thread per (element, sub-control volume) with the element's corners in
// shared memory; the gradient kernel one thread per element, areas from the
// cofactor identity of hex8_elem.h (equal to the reference's triangulated
// areas up to rounding).  Scatter by FP64 atomics.
#include <cuda_runtime.h>

#include <cstdint>

#include "hex8_elem.h"
#include "hex8_elem_df.h"
#include "internal.h"
#include "scv.cuh"

namespace nalu_gb300 {
namespace {

constexpr int kVolElems = 16;  // elements per block, 8 threads each

// vol (node field, optional) += sub-control volumes; scv (optional) [E][8]
// gets them per element; cap (one element) gets its eight volumes
__global__ void __launch_bounds__(kVolElems * 8) k_dual_volume(int64_t n_elems, const int32_t* __restrict__ conn,
                                                               const double* __restrict__ x, double* vol,
                                                               double* scv_out, int64_t cap_elem, double* cap) {
  __shared__ double sc[kVolElems][8][3];
  const int el = threadIdx.x / 8, scv = threadIdx.x % 8;
  const int64_t e = cap_elem >= 0 ? cap_elem : (int64_t)blockIdx.x * kVolElems + el;
  const bool valid = cap_elem >= 0 ? (el == 0) : e < n_elems;
  int node = 0;
  if (valid) {
    node = __ldg(conn + 8 * e + scv);
#pragma unroll
    for (int d = 0; d < 3; ++d) sc[el][scv][d] = __ldg(x + 3 * (int64_t)node + d);
  }
  __syncthreads();
  if (!valid) return;
  const double v = scv_volume(sc[el], scv);
  if (cap) {
    cap[scv] = v;
    return;
  }
  if (scv_out) scv_out[8 * e + scv] = v;
  if (vol) atomicAdd(vol + node, v);
}

// SCS area vector of ip (runtime index): +-1/4 of a cofactor column of J at
// the standard ip location
__device__ void scs_area(const EdgeForm& f, int ip, double area[3]) {
  const double s[3] = {ip_loc(ip, 0, 0.25), ip_loc(ip, 1, 0.25), ip_loc(ip, 2, 0.25)};
  double j[3][3], adj[3][3], det;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int u = (k == 0) ? 1 : 0, v = (k == 2) ? 1 : 2;
    const double su = s[u], sv = s[v];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double r = f.A[k][i];
      if (su != 0.0) r = r + f.B[k][i] * su;
      if (sv != 0.0) r = r + f.C[k][i] * sv;
      if (su * sv != 0.0) r = r + f.D[k][i] * (su * sv);
      j[i][k] = r;
    }
  }
  cofactor(j, adj, det);
  const int d = ip_dir(ip);
  const double sc = 0.25 * ip_sign(ip);
#pragma unroll
  for (int i = 0; i < 3; ++i) area[i] = sc * (d == 0 ? adj[i][0] : (d == 1 ? adj[i][1] : adj[i][2]));
}

// projected nodal gradient, element part; q [n][NC], grad [n][NC][3].  The
// twelve SCS area vectors are formed once; per component, the three SCS
// contributions of each node are summed in registers (q_ip A, + to the left
// node, - to the right) and leave as 8 x 3 atomics, scaled by 1/V of the node.
template <int NC, bool SHIFT>
__global__ void __launch_bounds__(128) k_nodal_grad(int64_t n_elems, const int32_t* __restrict__ conn,
                                                    const double* __restrict__ x, const double* __restrict__ q,
                                                    const double* __restrict__ dvol, double* grad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  int nd[8];
  double xc[8][3];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    nd[n] = __ldg(conn + 8 * e + n);
#pragma unroll
    for (int d = 0; d < 3; ++d) xc[n][d] = __ldg(x + 3 * (int64_t)nd[n] + d);
  }
  double area[12][3];
  {
    EdgeForm f;
    edge_form(xc, f);
#pragma unroll
    for (int ip = 0; ip < 12; ++ip) scs_area(f, ip, area[ip]);
  }
  constexpr double a = SHIFT ? 0.5 : 0.25;
#pragma unroll 1
  for (int k = 0; k < NC; ++k) {
    double qn[8], acc[8][3];
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      qn[n] = __ldg(q + (int64_t)nd[n] * NC + k);
      acc[n][0] = acc[n][1] = acc[n][2] = 0.0;
    }
#pragma unroll
    for (int ip = 0; ip < 12; ++ip) {
      double qip = 0.0;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const double w = shape_ip(ip, c, a);
        if (w != 0.0) qip += w * qn[c];
      }
      const int il = ip_left(ip), ir = ip_right(ip);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double fac = qip * area[ip][j];
        acc[il][j] += fac;
        acc[ir][j] -= fac;
      }
    }
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const double inv = 1.0 / __ldg(dvol + nd[n]);
#pragma unroll
      for (int j = 0; j < 3; ++j) atomicAdd(grad + ((int64_t)nd[n] * NC + k) * 3 + j, acc[n][j] * inv);
    }
  }
}

// the three SCS ips of each node (lrscv: node left (+) or right (-) of the ip)
__constant__ int8_t c_node_ip[8][3] = {{0, 3, 8}, {0, 1, 9}, {1, 2, 10}, {2, 3, 11},
                                       {4, 7, 8}, {4, 5, 9}, {5, 6, 10}, {6, 7, 11}};

// Element part of the projected nodal gradient in df64: node by node (a
// warp-uniform loop), the node's three SCS contributions +-q_ip A summed as
// FP32 pairs in registers, then NC x 3 FP64 atomics scaled by 1/V.  Areas
// are formed per (node, ip), i.e. twice per ip, on the FP32 pipes.
template <int NC, bool SHIFT>
__global__ void __launch_bounds__(128) k_nodal_grad_df(int64_t n_elems, const int32_t* __restrict__ conn,
                                                       const double* __restrict__ x, const double* __restrict__ q,
                                                       const double* __restrict__ dvol, double* grad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  int nd[8];
  double xc[8][3];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    nd[n] = __ldg(conn + 8 * e + n);
#pragma unroll
    for (int d = 0; d < 3; ++d) xc[n][d] = __ldg(x + 3 * (int64_t)nd[n] + d);
  }
  EdgeFormDF f;
  int kexp;  // normalised areas: x 2^(2 kexp)
  {
    df64 dd[8][3];
    kexp = rel_coords_df(xc, dd);
    edge_form_df(dd, f);
  }
  df64 qn[8][NC];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int k = 0; k < NC; ++k) qn[n][k] = df_split_bits(__ldg(q + (int64_t)nd[n] * NC + k));
#pragma unroll 1
  for (int r = 0; r < 8; ++r) {
    df64 acc[NC][3];
#pragma unroll
    for (int k = 0; k < NC; ++k) acc[k][0] = acc[k][1] = acc[k][2] = df_zero();
#pragma unroll 1
    for (int t = 0; t < 3; ++t) {
      const int ip = c_node_ip[r][t];
      IpGeomDF g;
      ip_geometry_df(f, ip, g);
      float s[3];
      ip_location(ip, SHIFT ? 0.5f : 0.25f, s);
      const float sg = ip_left(ip) == r ? 1.0f : -1.0f;
#pragma unroll
      for (int k = 0; k < NC; ++k) {
        df64 qi = df_zero();
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const float w = (0.5f + corner_sign(c, 0) * s[0]) * (0.5f + corner_sign(c, 1) * s[1]) *
                          (0.5f + corner_sign(c, 2) * s[2]);  // exact
          qi = df_add(qi, df_mul_f(qn[c][k], w));
        }
        qi = df_mul_f(qi, sg);
#pragma unroll
        for (int j = 0; j < 3; ++j) acc[k][j] = df_fma(qi, g.area[j], acc[k][j]);
      }
    }
    const double inv = 1.0 / __ldg(dvol + nd[r]);
#pragma unroll
    for (int k = 0; k < NC; ++k)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        atomicAdd(grad + ((int64_t)nd[r] * NC + k) * 3 + j, df_to_double_bits(acc[k][j], 2 * kexp) * inv);
  }
}

__global__ void k_zero(int64_t n, double* p) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.0;
}

}  // namespace

int launch_dual_volume(nalu_ctx* ctx, double* vol, int64_t cap_elem, double* cap) {
  const int64_t E = ctx->n_elems;
  if (E <= 0 || ctx->n_nodes <= 0) return NALU_OK;
  double* scv_out = nullptr;
  if (cap_elem < 0) {
    if (vol) {
      k_zero<<<(unsigned)((ctx->n_nodes + 255) / 256), 256, 0, ctx->stream>>>(ctx->n_nodes, vol);
      ctx->launches++;
    }
    // the per-element volumes refresh the cache on the way
    if (ctx->d_scv.n != 8 * E) NALU_CUDA(ctx, ctx->d_scv.alloc(8 * E));
    scv_out = ctx->d_scv.p;
  }
  const unsigned grid = cap_elem >= 0 ? 1u : (unsigned)((E + kVolElems - 1) / kVolElems);
  k_dual_volume<<<grid, kVolElems * 8, 0, ctx->stream>>>(E, ctx->d_conn.p, ctx->fields[NALU_FIELD_COORDINATES].d.p,
                                                          vol, scv_out, cap_elem, cap);
  ctx->launches++;
  const int rc = cuda_check(ctx, cudaGetLastError(), "dual volume");
  if (rc == NALU_OK && scv_out) ctx->scv_version = ctx->coords_version;
  return rc;
}

int ensure_scv_cache(nalu_ctx* ctx) {
  if (ctx->scv_version == ctx->coords_version && ctx->d_scv.n == 8 * ctx->n_elems) return NALU_OK;
  return launch_dual_volume(ctx, nullptr, -1, nullptr);
}

int launch_nodal_grad(nalu_ctx* ctx, const double* q, int ncomp, const double* dvol, double* grad, bool shifted,
                      int arith) {
  const int64_t E = ctx->n_elems;
  const int64_t total = ctx->n_nodes * 3 * ncomp;
  if (E <= 0 || total <= 0) return NALU_OK;
  k_zero<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(total, grad);
  const unsigned grid = (unsigned)((E + 127) / 128);
  const double* x = ctx->fields[NALU_FIELD_COORDINATES].d.p;
  if (arith == NALU_ARITH_DF64) {
    if (ncomp == 1) {
      if (shifted) k_nodal_grad_df<1, true><<<grid, 128, 0, ctx->stream>>>(E, ctx->d_conn.p, x, q, dvol, grad);
      else k_nodal_grad_df<1, false><<<grid, 128, 0, ctx->stream>>>(E, ctx->d_conn.p, x, q, dvol, grad);
    } else {
      if (shifted) k_nodal_grad_df<3, true><<<grid, 128, 0, ctx->stream>>>(E, ctx->d_conn.p, x, q, dvol, grad);
      else k_nodal_grad_df<3, false><<<grid, 128, 0, ctx->stream>>>(E, ctx->d_conn.p, x, q, dvol, grad);
    }
  } else if (ncomp == 1) {
    if (shifted) k_nodal_grad<1, true><<<grid, 128, 0, ctx->stream>>>(E, ctx->d_conn.p, x, q, dvol, grad);
    else k_nodal_grad<1, false><<<grid, 128, 0, ctx->stream>>>(E, ctx->d_conn.p, x, q, dvol, grad);
  } else {
    if (shifted) k_nodal_grad<3, true><<<grid, 128, 0, ctx->stream>>>(E, ctx->d_conn.p, x, q, dvol, grad);
    else k_nodal_grad<3, false><<<grid, 128, 0, ctx->stream>>>(E, ctx->d_conn.p, x, q, dvol, grad);
  }
  ctx->launches += 2;
  return cuda_check(ctx, cudaGetLastError(), "nodal gradient");
}

}  // namespace nalu_gb300
