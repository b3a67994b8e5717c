// master_element.cu -- the Hex8 master element (src/master_element/Hex8CVFEM.C)
// as batched device calls: the MasterElement surface that kernels and
// algorithms call per element, evaluated here for many elements at once.
//
//   HexSCS::determinant     SCS area vectors [12][3] (Hex8CVFEM.C:547-580);
//                           here as +-1/4 of a cofactor column of J at the ip,
//                           equal to the reference's triangulated sub-face
//                           sum up to rounding
//   HexSCS::grad_op         dN/dx [12][8][3] and dN/ds [12][8][3]
//   (shifted_grad_op)       (generic_grad_op, MasterElementFunctions.h:51-108)
//   HexSCV::determinant     the eight sub-control volumes (scv.cuh)
//   HexSCS::face_grad_op    dN/dx at the four exposed-face ips of a side
//   (shifted_face_grad_op)  (Hex8CVFEM.C:668-684)
//   adjacentNodes, shape_fcn, side_node_ordinals: the constant tables.
//
// One thread per element; coordinates [nelem][8][3] in the element's node
// order, outputs per element in the reference's layouts.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "hex8_elem.h"
#include "internal.h"
#include "scv.cuh"

namespace nalu_gb300 {
namespace {

enum MePoints { ME_SCS = 0, ME_SCV = 1, ME_FACE = 2 };

__constant__ int8_t c_me_side[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
__constant__ int8_t c_me_side_axis[6] = {1, 0, 1, 0, 2, 2};

// parent coordinates of integration point k of the given point set
__device__ void me_point(int kind, int k, int side, bool shifted, double s[3]) {
  const double a = shifted ? 0.5 : 0.25;
  if (kind == ME_SCS) {
#pragma unroll
    for (int d = 0; d < 3; ++d) s[d] = ip_loc(k, d, a);
  } else if (kind == ME_SCV) {
#pragma unroll
    for (int d = 0; d < 3; ++d) s[d] = corner_sign(k, d) * a;
  } else {
    const int node = c_me_side[side][k];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double xn = 0.5 * corner_sign(node, d);
      s[d] = (shifted || d == c_me_side_axis[side]) ? xn : 0.5 * xn;
    }
  }
}

// J[i][k] = sum_n dN_n/ds_k x_n,i at s, its cofactor matrix and determinant
__device__ void me_jacobian(const double x[8][3], const double s[3], double adj[3][3], double& det) {
  double j[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double r = 0.0;
#pragma unroll
      for (int n = 0; n < 8; ++n) r += dshape(n, k, s[0], s[1], s[2]) * x[n][i];
      j[i][k] = r;
    }
  cofactor(j, adj, det);
}

__device__ __forceinline__ void me_load(const double* __restrict__ coords, int64_t e, double x[8][3]) {
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int d = 0; d < 3; ++d) x[n][d] = coords[24 * e + 3 * n + d];
}

__global__ void k_me_scs_areav(int64_t nelem, const double* __restrict__ coords, double* __restrict__ areav) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  double x[8][3];
  me_load(coords, e, x);
#pragma unroll 1
  for (int ip = 0; ip < 12; ++ip) {
    double s[3], adj[3][3], det;
    me_point(ME_SCS, ip, 0, false, s);
    me_jacobian(x, s, adj, det);
    const int d = ip_dir(ip);
    const double sc = 0.25 * ip_sign(ip);
#pragma unroll
    for (int i = 0; i < 3; ++i) areav[36 * e + 3 * ip + i] = sc * (d == 0 ? adj[i][0] : (d == 1 ? adj[i][1] : adj[i][2]));
  }
}

// grad op at the points of `kind`; side indexes a per-element side array for
// faces; counts elements whose det(J) <= 0 at some point
__global__ void k_me_grad_op(int64_t nelem, const double* __restrict__ coords, int kind, const int32_t* __restrict__ side,
                             int shifted, double* __restrict__ gradop, double* __restrict__ deriv, int* nbad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  const int npts = kind == ME_SCS ? 12 : (kind == ME_SCV ? 8 : 4);
  const int sd = kind == ME_FACE ? side[e] : 0;
  double x[8][3];
  me_load(coords, e, x);
  bool bad = false;
#pragma unroll 1
  for (int k = 0; k < npts; ++k) {
    double s[3], adj[3][3], det;
    me_point(kind, k, sd, shifted != 0, s);
    me_jacobian(x, s, adj, det);
    if (!(det > 1.0e-300)) bad = true;
    const double inv = 1.0 / det;
    const int64_t o = ((int64_t)e * npts + k) * 24;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const double d0 = dshape(n, 0, s[0], s[1], s[2]), d1 = dshape(n, 1, s[0], s[1], s[2]),
                   d2 = dshape(n, 2, s[0], s[1], s[2]);
#pragma unroll
      for (int i = 0; i < 3; ++i) gradop[o + 3 * n + i] = (adj[i][0] * d0 + adj[i][1] * d1 + adj[i][2] * d2) * inv;
      if (deriv) {
        deriv[o + 3 * n + 0] = d0;
        deriv[o + 3 * n + 1] = d1;
        deriv[o + 3 * n + 2] = d2;
      }
    }
  }
  if (bad) atomicAdd(nbad, 1);
}

__global__ void k_me_scv_volume(int64_t nelem, const double* __restrict__ coords, double* __restrict__ vol) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  double x[8][3];
  me_load(coords, e, x);
#pragma unroll 1
  for (int ip = 0; ip < 8; ++ip) vol[8 * e + ip] = scv_volume(x, ip);
}

unsigned me_grid(int64_t n) { return (unsigned)((n + 127) / 128); }

// device copies of host arrays (or the caller's device arrays as they are)
struct MeIo {
  nalu_ctx* ctx;
  bool on_device;
  DBuf<double> in, out, out2;
  DBuf<int32_t> side;
  int rc = NALU_OK;
  const double* coords_in(const double* coords, int64_t n) {
    if (on_device) return coords;
    if ((rc = cuda_check(ctx, in.alloc(24 * n), "me alloc"))) return nullptr;
    rc = cuda_check(ctx, cudaMemcpyAsync(in.p, coords, sizeof(double) * 24 * n, cudaMemcpyHostToDevice, ctx->stream),
                    "me copy");
    return in.p;
  }
  double* buf(DBuf<double>& b, double* user, int64_t count) {
    if (!user) return nullptr;
    if (on_device) return user;
    if ((rc = cuda_check(ctx, b.alloc(count), "me alloc"))) return nullptr;
    return b.p;
  }
  int back(double* user, const double* dev, int64_t count) {
    if (rc || on_device || !user) return rc;
    return cuda_check(ctx, cudaMemcpyAsync(user, dev, sizeof(double) * count, cudaMemcpyDeviceToHost, ctx->stream),
                      "me copy back");
  }
};

int me_finish(nalu_ctx* ctx, const char* what) {
  int rc = cuda_check(ctx, cudaGetLastError(), what);
  if (rc) return rc;
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), what);
}

}  // namespace
}  // namespace nalu_gb300

using namespace nalu_gb300;

extern "C" {

int nalu_hex_scs_determinant(nalu_ctx* ctx, int64_t nelem, const double* coords, double* areav, int on_device) {
  if (!ctx || nelem < 0 || (nelem > 0 && (!coords || !areav))) return set_error(ctx, NALU_ERR_ARG, "scs determinant args");
  if (nelem == 0) return NALU_OK;
  cudaSetDevice(ctx->device);
  MeIo io{ctx, on_device != 0};
  const double* c = io.coords_in(coords, nelem);
  double* a = io.buf(io.out, areav, 36 * nelem);
  if (io.rc) return io.rc;
  k_me_scs_areav<<<me_grid(nelem), 128, 0, ctx->stream>>>(nelem, c, a);
  ctx->launches++;
  int rc = io.back(areav, a, 36 * nelem);
  return rc ? rc : me_finish(ctx, "scs determinant");
}

static int grad_op_common(nalu_ctx* ctx, int kind, int64_t nelem, const int32_t* side, const double* coords,
                          int shifted, double* gradop, double* deriv, int on_device) {
  if (!ctx || nelem < 0 || (nelem > 0 && (!coords || !gradop)) || (kind == 2 && nelem > 0 && !side))
    return set_error(ctx, NALU_ERR_ARG, "grad op args");
  if (nelem == 0) return NALU_OK;
  cudaSetDevice(ctx->device);
  const int npts = kind == 0 ? 12 : (kind == 1 ? 8 : 4);
  MeIo io{ctx, on_device != 0};
  const double* c = io.coords_in(coords, nelem);
  double* g = io.buf(io.out, gradop, (int64_t)npts * 24 * nelem);
  double* d = io.buf(io.out2, deriv, (int64_t)npts * 24 * nelem);
  const int32_t* sd = nullptr;
  if (kind == 2) {
    if (on_device) {
      sd = side;
    } else {
      if ((io.rc = cuda_check(ctx, io.side.alloc(nelem), "me alloc")) == NALU_OK)
        io.rc = cuda_check(ctx, cudaMemcpyAsync(io.side.p, side, sizeof(int32_t) * nelem, cudaMemcpyHostToDevice,
                                                ctx->stream), "me copy");
      sd = io.side.p;
    }
  }
  if (io.rc) return io.rc;
  DBuf<int> nbad;
  NALU_CUDA(ctx, nbad.alloc(1));
  NALU_CUDA(ctx, cudaMemsetAsync(nbad.p, 0, sizeof(int), ctx->stream));
  k_me_grad_op<<<me_grid(nelem), 128, 0, ctx->stream>>>(nelem, c, kind, sd, shifted, g, d, nbad.p);
  ctx->launches++;
  int rc = io.back(gradop, g, (int64_t)npts * 24 * nelem);
  if (!rc) rc = io.back(deriv, d, (int64_t)npts * 24 * nelem);
  if (rc) return rc;
  int hb = 0;
  NALU_CUDA(ctx, cudaMemcpyAsync(&hb, nbad.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  rc = me_finish(ctx, "grad op");
  if (rc) return rc;
  if (hb) return set_error(ctx, NALU_ERR_NEG_JACOBIAN, std::to_string(hb) + " element(s) with det(J) <= 0");
  return NALU_OK;
}

int nalu_hex_scs_grad_op(nalu_ctx* ctx, int64_t nelem, const double* coords, int shifted, double* gradop,
                         double* deriv, int on_device) {
  return grad_op_common(ctx, 0, nelem, nullptr, coords, shifted, gradop, deriv, on_device);
}

int nalu_hex_scv_grad_op(nalu_ctx* ctx, int64_t nelem, const double* coords, int shifted, double* gradop,
                         double* deriv, int on_device) {
  return grad_op_common(ctx, 1, nelem, nullptr, coords, shifted, gradop, deriv, on_device);
}

int nalu_hex_face_grad_op(nalu_ctx* ctx, int64_t nelem, const int32_t* side, const double* coords, int shifted,
                          double* gradop, int on_device) {
  if (side && !on_device)
    for (int64_t i = 0; i < nelem; ++i)
      if (side[i] < 0 || side[i] > 5) return set_error(ctx, NALU_ERR_ARG, "side ordinal out of range");
  return grad_op_common(ctx, 2, nelem, side, coords, shifted, gradop, nullptr, on_device);
}

int nalu_hex_scv_determinant(nalu_ctx* ctx, int64_t nelem, const double* coords, double* vol, int on_device) {
  if (!ctx || nelem < 0 || (nelem > 0 && (!coords || !vol))) return set_error(ctx, NALU_ERR_ARG, "scv determinant args");
  if (nelem == 0) return NALU_OK;
  cudaSetDevice(ctx->device);
  MeIo io{ctx, on_device != 0};
  const double* c = io.coords_in(coords, nelem);
  double* v = io.buf(io.out, vol, 8 * nelem);
  if (io.rc) return io.rc;
  k_me_scv_volume<<<me_grid(nelem), 128, 0, ctx->stream>>>(nelem, c, v);
  ctx->launches++;
  int rc = io.back(vol, v, 8 * nelem);
  return rc ? rc : me_finish(ctx, "scv determinant");
}

void nalu_hex_scs_adjacent_nodes(int32_t* lrscv) {
  if (!lrscv) return;
  for (int ip = 0; ip < 12; ++ip) {
    lrscv[2 * ip] = ip_left(ip);
    lrscv[2 * ip + 1] = ip_right(ip);
  }
}

void nalu_hex_scs_shape_fcn(int shifted, double* shp) {
  if (!shp) return;
  const double a = shifted ? 0.5 : 0.25;
  for (int ip = 0; ip < 12; ++ip)
    for (int n = 0; n < 8; ++n) shp[8 * ip + n] = shape_ip(ip, n, a);
}

void nalu_hex_side_node_ordinals(int side, int32_t* nodes4) {
  static const int32_t t[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
  if (!nodes4 || side < 0 || side > 5) return;
  std::memcpy(nodes4, t[side], sizeof(t[side]));
}

}  // extern "C"
