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
#include "internal.h"

namespace nalu_gb300 {
namespace {

constexpr int kVolElems = 16;  // elements per block, 8 threads each

// point k (0..26) of the 27-point subdivision, component d
__device__ double subpoint(const double (*c)[3], int k, int d) {
  auto m2 = [&](int a, int b) { return 0.5 * (c[a][d] + c[b][d]); };
  auto m4 = [&](int a, int b, int e, int f) { return 0.25 * (c[a][d] + c[b][d] + c[e][d] + c[f][d]); };
  switch (k) {
    case 8: return m2(0, 1);
    case 9: return m2(1, 2);
    case 10: return m2(2, 3);
    case 11: return m2(3, 0);
    case 12: return m4(0, 1, 2, 3);
    case 13: return m2(4, 5);
    case 14: return m2(5, 6);
    case 15: return m2(6, 7);
    case 16: return m2(7, 4);
    case 17: return m4(4, 5, 6, 7);
    case 18: return m2(1, 5);
    case 19: return m2(0, 4);
    case 20: return m4(0, 1, 4, 5);
    case 21: return m2(3, 7);
    case 22: return m2(2, 6);
    case 23: return m4(2, 3, 6, 7);
    case 24: return m4(1, 2, 5, 6);
    case 25: return m4(0, 3, 4, 7);
    case 26: {
      double s = 0.0;
      for (int n = 0; n < 8; ++n) s += c[n][d];
      return s * 0.125;
    }
    default: return c[k][d];
  }
}

__constant__ int8_t c_sub[8][8] = {{0, 8, 12, 11, 19, 20, 26, 25},  {8, 1, 9, 12, 20, 18, 24, 26},
                                   {12, 9, 2, 10, 26, 24, 22, 23},  {11, 12, 10, 3, 25, 26, 23, 21},
                                   {19, 20, 26, 25, 4, 13, 17, 16}, {20, 18, 24, 26, 13, 5, 14, 17},
                                   {26, 24, 22, 23, 17, 14, 6, 15}, {25, 26, 23, 21, 16, 17, 15, 7}};
__constant__ int8_t c_gface[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {2, 3, 7, 6}, {1, 2, 6, 5}, {0, 4, 3, 7}};
__constant__ int8_t c_gtri[24][3] = {{0, 8, 1},  {8, 2, 1},   {3, 2, 8},   {3, 8, 0},  {6, 9, 5},   {7, 9, 6},
                                     {4, 9, 7},  {4, 5, 9},   {10, 0, 1},  {5, 10, 1}, {4, 10, 5},  {4, 0, 10},
                                     {7, 6, 11}, {6, 2, 11},  {2, 3, 11},  {3, 7, 11}, {6, 12, 2},  {5, 12, 6},
                                     {5, 1, 12}, {1, 2, 12},  {0, 4, 13},  {4, 7, 13}, {7, 3, 13},  {3, 0, 13}};

// Grandy's hexahedron volume: six face centroids, 24 triangles
__device__ double grandy_volume(const double (&h)[8][3]) {
  double cv[14][3];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int d = 0; d < 3; ++d) cv[n][d] = h[n][d];
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      cv[k + 8][d] = 0.25 * (cv[c_gface[k][0]][d] + cv[c_gface[k][1]][d] + cv[c_gface[k][2]][d] + cv[c_gface[k][3]][d]);
  double volume = 0.0;
#pragma unroll
  for (int k = 0; k < 24; ++k) {
    const int p = c_gtri[k][0], q = c_gtri[k][1], r = c_gtri[k][2];
    const double m0 = cv[p][0] + cv[q][0] + cv[r][0], m1 = cv[p][1] + cv[q][1] + cv[r][1],
                 m2 = cv[p][2] + cv[q][2] + cv[r][2];
    const double d0 = (cv[q][1] - cv[p][1]) * (cv[r][2] - cv[p][2]) - (cv[r][1] - cv[p][1]) * (cv[q][2] - cv[p][2]);
    const double d1 = (cv[r][0] - cv[p][0]) * (cv[q][2] - cv[p][2]) - (cv[q][0] - cv[p][0]) * (cv[r][2] - cv[p][2]);
    const double d2 = (cv[q][0] - cv[p][0]) * (cv[r][1] - cv[p][1]) - (cv[r][0] - cv[p][0]) * (cv[q][1] - cv[p][1]);
    volume += m0 * d0 + m1 * d1 + m2 * d2;
  }
  return volume / 18.0;
}

// vol (node field) += sub-control volumes; cap (optional, one element) gets the eight volumes
__global__ void __launch_bounds__(kVolElems * 8) k_dual_volume(int64_t n_elems, const int32_t* __restrict__ conn,
                                                               const double* __restrict__ x, double* vol,
                                                               int64_t cap_elem, double* cap) {
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
  double h[8][3];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int d = 0; d < 3; ++d) h[n][d] = subpoint(sc[el], c_sub[scv][n], d);
  const double v = grandy_volume(h);
  if (cap) cap[scv] = v;
  else atomicAdd(vol + node, v);
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

// projected nodal gradient, element part; q [n][NC], grad [n][NC][3]
template <int NC, bool SHIFT>
__global__ void __launch_bounds__(128) k_nodal_grad(int64_t n_elems, const int32_t* __restrict__ conn,
                                                    const double* __restrict__ x, const double* __restrict__ q,
                                                    const double* __restrict__ dvol, double* grad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  int nd[8];
  double xc[8][3], qn[8][NC], inv[8];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    nd[n] = __ldg(conn + 8 * e + n);
#pragma unroll
    for (int d = 0; d < 3; ++d) xc[n][d] = __ldg(x + 3 * (int64_t)nd[n] + d);
#pragma unroll
    for (int k = 0; k < NC; ++k) qn[n][k] = __ldg(q + (int64_t)nd[n] * NC + k);
    inv[n] = 1.0 / __ldg(dvol + nd[n]);
  }
  EdgeForm f;
  edge_form(xc, f);
  const double a = SHIFT ? 0.5 : 0.25;
#pragma unroll 1
  for (int ip = 0; ip < 12; ++ip) {
    double area[3];
    scs_area(f, ip, area);
    const int il = ip_left(ip), ir = ip_right(ip);
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      double qip = 0.0;
#pragma unroll
      for (int c = 0; c < 8; ++c) qip += shape(c, ip_loc(ip, 0, a), ip_loc(ip, 1, a), ip_loc(ip, 2, a)) * qn[c][k];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double fac = qip * area[j];
        atomicAdd(grad + ((int64_t)nd[il] * NC + k) * 3 + j, fac * inv[il]);
        atomicAdd(grad + ((int64_t)nd[ir] * NC + k) * 3 + j, -fac * inv[ir]);
      }
    }
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
  if (cap_elem < 0) {
    k_zero<<<(unsigned)((ctx->n_nodes + 255) / 256), 256, 0, ctx->stream>>>(ctx->n_nodes, vol);
    ctx->launches++;
  }
  const unsigned grid = cap_elem >= 0 ? 1u : (unsigned)((E + kVolElems - 1) / kVolElems);
  k_dual_volume<<<grid, kVolElems * 8, 0, ctx->stream>>>(E, ctx->d_conn.p, ctx->fields[NALU_FIELD_COORDINATES].d.p,
                                                          vol, cap_elem, cap);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "dual volume");
}

int launch_nodal_grad(nalu_ctx* ctx, const double* q, int ncomp, const double* dvol, double* grad, bool shifted) {
  const int64_t E = ctx->n_elems;
  const int64_t total = ctx->n_nodes * 3 * ncomp;
  if (E <= 0 || total <= 0) return NALU_OK;
  k_zero<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(total, grad);
  const unsigned grid = (unsigned)((E + 127) / 128);
  const double* x = ctx->fields[NALU_FIELD_COORDINATES].d.p;
  if (ncomp == 1) {
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
