// faces.cu -- boundary faces of the Hex8 mesh: side sets, their exposed-face
// geometry, the boundary closure of the projected nodal gradient, and the
// continuity inflow / open face kernels.
//
//   side set           a list of (element, side ordinal); side s of an element
//                      has the nodes sideNodeOrdinals_[s]
//                      (src/master_element/Hex8CVFEM.C:415-422), which is also
//                      the face ip -> node map HexSCS::ipNodeMap(s)
//   exposed area       Quad3DSCS::determinant = quad3d_scs_det
//                      (MasterElementWork.F:1467-1590): four sub-faces, each
//                      the quad (corner, edge midpoint, centre, edge midpoint)
//                      with area vector (c - p_k) x (e_{k-1} - e_k) / 2
//   gradient closure   AssembleNodalGradBoundaryAlgorithm::execute
//                      (src/AssembleNodalGradBoundaryAlgorithm.C:75-153)
//   inflow             ContinuityInflowElemKernel::execute
//                      (src/kernel/ContinuityInflowElemKernel.C:73-108)
//   open               ContinuityOpenElemKernel::execute
//                      (src/kernel/ContinuityOpenElemKernel.C:107-199) with
//                      HexSCS::face_grad_op at the exposed-face ips
//                      (Hex8CVFEM.C:668-684, intgExpFace_ :348-373)
//
// One thread per face; rows are the face's nodes, columns the element's (the
// face-element algorithm sums into the element's connectivity), through the
// element slot table with FP64 atomics.  The exposed-face skin of a mesh is
// found with an exact hash of each side (its smallest node and the node
// diagonally across from it, which identify a quad of a conforming mesh).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "hex8_elem.h"
#include "internal.h"

namespace nalu_gb300 {
namespace {

__constant__ int8_t c_side[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
// parent axis normal to each side
__constant__ int8_t c_side_axis[6] = {1, 0, 1, 0, 2, 2};

constexpr double kPenaltyFac = 2.0;  // ContinuityOpenElemKernel penaltyFac_
constexpr int kFaceThreads = 128;

// quad3d_scs_det: sub-face k of the quad p (side order)
__device__ void quad_areas(const double p[4][3], double a[4][3]) {
  double e[4][3], c[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int k = 0; k < 4; ++k) e[k][d] = (p[k][d] + p[(k + 1) & 3][d]) * 0.5;
    c[d] = (p[0][d] + p[1][d] + p[2][d] + p[3][d]) * 0.25;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int prev = (k + 3) & 3;
    const double dx13 = c[0] - p[k][0], dx24 = e[prev][0] - e[k][0];
    const double dy13 = c[1] - p[k][1], dy24 = e[prev][1] - e[k][1];
    const double dz13 = c[2] - p[k][2], dz24 = e[prev][2] - e[k][2];
    a[k][0] = 0.5 * (dz24 * dy13 - dz13 * dy24);
    a[k][1] = 0.5 * (dx24 * dz13 - dx13 * dz24);
    a[k][2] = 0.5 * (dy24 * dx13 - dy13 * dx24);
  }
}

// Quad3DSCS shape function of face node ic at face ip (quad3d_shape_fcn at
// +-1/4): 9/16 own corner, 3/16 the two neighbours, 1/16 across; shifted: 1, 0
__device__ __forceinline__ double face_w(int ip, int ic, bool shifted) {
  if (shifted) return ip == ic ? 1.0 : 0.0;
  const int d = (ip - ic) & 3;
  return d == 0 ? 0.5625 : (d == 2 ? 0.0625 : 0.1875);
}

// dN_n/dx . A for all eight nodes at the parent point s (generic grad op,
// contracted with A through G = adj(J)^T A)
__device__ void dndx_dot(const double x[8][3], const double s[3], const double A[3], double out[8]) {
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
  double adj[3][3], det;
  cofactor(j, adj, det);
  double G[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) G[k] = (adj[0][k] * A[0] + adj[1][k] * A[1] + adj[2][k] * A[2]) / det;
#pragma unroll
  for (int n = 0; n < 8; ++n)
    out[n] = dshape(n, 0, s[0], s[1], s[2]) * G[0] + dshape(n, 1, s[0], s[1], s[2]) * G[1] +
             dshape(n, 2, s[0], s[1], s[2]) * G[2];
}

// exposed-face ip k of side s: the face node's parent point, in-plane
// coordinates halved unless shifted
__device__ void face_ip_point(int s, int k, bool shifted, double pt[3]) {
  const int node = c_side[s][k];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double x = 0.5 * corner_sign(node, d);
    pt[d] = (shifted || d == c_side_axis[s]) ? x : 0.5 * x;
  }
}

// ---- skin -------------------------------------------------------------------
constexpr unsigned long long kEmpty = ~0ull;

__device__ __forceinline__ unsigned long long side_key(const int32_t* conn, int64_t e, int s) {
  int32_t nd[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) nd[k] = __ldg(conn + 8 * e + c_side[s][k]);
  int m = 0;
#pragma unroll
  for (int k = 1; k < 4; ++k)
    if (nd[k] < nd[m]) m = k;
  return ((unsigned long long)(uint32_t)nd[m] << 32) | (uint32_t)nd[(m + 2) & 3];
}

__device__ __forceinline__ uint64_t slot_of(unsigned long long key, uint64_t mask) {
  return (key * 0x9E3779B97F4A7C15ull >> 17) & mask;
}

__global__ void k_skin_insert(int64_t n_sides, const int32_t* __restrict__ conn, unsigned long long* keys,
                              uint32_t* cnt, uint64_t mask, int* err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_sides) return;
  const unsigned long long key = side_key(conn, i / 6, (int)(i % 6));
  uint64_t slot = slot_of(key, mask);
  for (uint64_t it = 0; it <= mask; ++it) {
    const unsigned long long prev = atomicCAS(keys + slot, kEmpty, key);
    if (prev == kEmpty || prev == key) {
      atomicAdd(cnt + slot, 1u);
      return;
    }
    slot = (slot + 1) & mask;
  }
  atomicAdd(err, 1);
}

__global__ void k_skin_mark(int64_t n_sides, const int32_t* __restrict__ conn, const unsigned long long* keys,
                            const uint32_t* cnt, uint64_t mask, uint8_t* flags, int* err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_sides) return;
  const unsigned long long key = side_key(conn, i / 6, (int)(i % 6));
  uint64_t slot = slot_of(key, mask);
  for (uint64_t it = 0; it <= mask; ++it) {
    const unsigned long long k = keys[slot];
    if (k == key) {
      flags[i] = cnt[slot] == 1u ? 1 : 0;
      return;
    }
    if (k == kEmpty) break;
    slot = (slot + 1) & mask;
  }
  flags[i] = 0;
  atomicAdd(err, 1);
}

// ---- per-face kernels -----------------------------------------------------------
struct FaceArgs {
  int64_t n;
  const int32_t* felem;
  const uint8_t* fside;
  const double* dynp;  // [n][4] or null
  const int32_t* conn;
  const double* x;
  // nodal fields (LID order)
  const double* q;
  int ncomp;
  const double* dvol;
  double* grad;
  const double* rho;
  const double* u;  // velocity (open) or cont_velocity_bc (inflow)
  const double* p;
  const double* pbc;
  const double* gpdx;
  double pts;  // projTimeScale
  int shift_grad, lhs_shift, shift_mdot;
  // system
  const int64_t* rowptr;
  const uint8_t* slots;
  double* values;
  double* rhs;
  double* area_out;  // [n][4][3] or null
  int64_t cap_face;
  double* cap_lhs;
  double* cap_rhs;
};

__device__ __forceinline__ void load_face(const FaceArgs& a, int64_t f, int64_t& e, int& s, int32_t nd[8],
                                          double x[8][3]) {
  e = __ldg(a.felem + f);
  s = __ldg(a.fside + f);
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    nd[n] = __ldg(a.conn + 8 * e + n);
#pragma unroll
    for (int d = 0; d < 3; ++d) x[n][d] = __ldg(a.x + 3 * (int64_t)nd[n] + d);
  }
}

__device__ __forceinline__ void side_areas(int s, const double x[8][3], double ar[4][3]) {
  double p[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d) p[k][d] = x[c_side[s][k]][d];
  quad_areas(p, ar);
}

__global__ void __launch_bounds__(kFaceThreads) k_face_area(FaceArgs a) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.n) return;
  int64_t e;
  int s;
  int32_t nd[8];
  double x[8][3], ar[4][3];
  load_face(a, f, e, s, nd, x);
  side_areas(s, x, ar);
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d) a.area_out[(f * 4 + k) * 3 + d] = ar[k][d];
}

template <int NC>
__global__ void __launch_bounds__(kFaceThreads) k_grad_boundary(FaceArgs a, bool shifted) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.n) return;
  int64_t e;
  int s;
  int32_t nd[8];
  double x[8][3], ar[4][3];
  load_face(a, f, e, s, nd, x);
  side_areas(s, x, ar);
  double qf[4][NC];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int c = 0; c < NC; ++c) qf[k][c] = __ldg(a.q + (int64_t)nd[c_side[s][k]] * NC + c);
#pragma unroll
  for (int ip = 0; ip < 4; ++ip) {
    const int64_t nn = nd[c_side[s][ip]];
    const double inv = 1.0 / __ldg(a.dvol + nn);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      double qip = 0.0;
#pragma unroll
      for (int ic = 0; ic < 4; ++ic) qip += face_w(ip, ic, shifted) * qf[ic][c];
#pragma unroll
      for (int j = 0; j < 3; ++j) atomicAdd(a.grad + (nn * NC + c) * 3 + j, qip * ar[ip][j] * inv);
    }
  }
}

// scatter of one face row (element-local row r) into the system, or capture
template <int OUT>
__device__ __forceinline__ void put_row(const FaceArgs& a, int64_t e, const int32_t nd[8], int r, const double v[8],
                                        double rs, bool has_lhs) {
  if (OUT == 2) {
    if (has_lhs)
#pragma unroll
      for (int c = 0; c < 8; ++c) a.cap_lhs[r * 8 + c] += v[c];
    a.cap_rhs[r] += rs;
    return;
  }
  const int64_t row = nd[r];
  if (has_lhs) {
    const int64_t base = __ldg(a.rowptr + row);
    const uint2 o2 = __ldg(reinterpret_cast<const uint2*>(a.slots + 64 * e + 8 * r));
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const uint32_t word = c < 4 ? o2.x : o2.y;
      const int off = (word >> (8 * (c & 3))) & 0xff;
      atomicAdd(a.values + base + off, v[c]);
    }
  }
  atomicAdd(a.rhs + row, rs);
}

template <int OUT>
__global__ void __launch_bounds__(kFaceThreads) k_cont_inflow(FaceArgs a) {
  const int64_t f = OUT == 2 ? a.cap_face : (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (OUT == 2 ? threadIdx.x != 0 : f >= a.n) return;
  int64_t e;
  int s;
  int32_t nd[8];
  double x[8][3], ar[4][3];
  load_face(a, f, e, s, nd, x);
  side_areas(s, x, ar);
  double rho[4], ub[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int64_t n = nd[c_side[s][k]];
    rho[k] = __ldg(a.rho + n);
#pragma unroll
    for (int d = 0; d < 3; ++d) ub[k][d] = __ldg(a.u + 3 * n + d);
  }
  const double zero[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int ip = 0; ip < 4; ++ip) {
    double w[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int ic = 0; ic < 4; ++ic) {
      const double r = face_w(ip, ic, a.shift_mdot != 0) * rho[ic];
#pragma unroll
      for (int j = 0; j < 3; ++j) w[j] += r * ub[ic][j];
    }
    const double mdot = w[0] * ar[ip][0] + w[1] * ar[ip][1] + w[2] * ar[ip][2];
    put_row<OUT>(a, e, nd, c_side[s][ip], zero, -mdot / a.pts, false);
  }
}

template <int OUT>
__global__ void __launch_bounds__(kFaceThreads) k_cont_open(FaceArgs a) {
  const int64_t f = OUT == 2 ? a.cap_face : (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (OUT == 2 ? threadIdx.x != 0 : f >= a.n) return;
  int64_t e;
  int s;
  int32_t nd[8];
  double x[8][3], ar[4][3];
  load_face(a, f, e, s, nd, x);
  side_areas(s, x, ar);
  double pe[8];
#pragma unroll
  for (int n = 0; n < 8; ++n) pe[n] = __ldg(a.p + nd[n]);
  double rho[4], pbc[4], uf[4][3], gf[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int64_t n = nd[c_side[s][k]];
    rho[k] = __ldg(a.rho + n);
    pbc[k] = __ldg(a.pbc + n);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      uf[k][d] = __ldg(a.u + 3 * n + d);
      gf[k][d] = __ldg(a.gpdx + 3 * n + d);
    }
  }
  const bool smdot = a.shift_mdot != 0;
#pragma unroll 1
  for (int ip = 0; ip < 4; ++ip) {
    const double A[3] = {ar[ip][0], ar[ip][1], ar[ip][2]};
    const double aMag = sqrt(A[0] * A[0] + A[1] * A[1] + A[2] * A[2]);
    double pt[3], gA[8], gA_lhs[8];
    face_ip_point(s, ip, a.shift_grad != 0, pt);
    dndx_dot(x, pt, A, gA);
    if (a.lhs_shift != a.shift_grad) {
      face_ip_point(s, ip, a.lhs_shift != 0, pt);
      dndx_dot(x, pt, A, gA_lhs);
    } else {
#pragma unroll
      for (int n = 0; n < 8; ++n) gA_lhs[n] = gA[n];
    }
    double invL = 0.0;
#pragma unroll
    for (int ic = 0; ic < 4; ++ic) invL += gA[c_side[s][ic]];
    invL /= aMag;
    double pBip = 0.0, pbcBip = a.dynp ? -__ldg(a.dynp + 4 * f + ip) : 0.0, ru[3] = {0, 0, 0}, gp[3] = {0, 0, 0};
#pragma unroll
    for (int ic = 0; ic < 4; ++ic) {
      const double r = face_w(ip, ic, smdot);
      pBip += r * pe[c_side[s][ic]];
      pbcBip += r * pbc[ic];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        ru[j] += r * rho[ic] * uf[ic][j];
        gp[j] += r * gf[ic][j];
      }
    }
    double dpA = 0.0;  // (dp/dx)_ip . A
#pragma unroll
    for (int n = 0; n < 8; ++n) dpA += gA[n] * pe[n];
    double mdot = kPenaltyFac * a.pts * invL * (pBip - pbcBip) * aMag;
    // + (rho u - tau (dp/dx - Gp)) . A, with dp/dx . A formed through G
    mdot += (ru[0] + a.pts * gp[0]) * A[0] + (ru[1] + a.pts * gp[1]) * A[1] + (ru[2] + a.pts * gp[2]) * A[2];
    mdot -= a.pts * dpA;
    double v[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) v[n] = -gA_lhs[n];
#pragma unroll
    for (int ic = 0; ic < 4; ++ic) v[c_side[s][ic]] += face_w(ip, ic, smdot) * kPenaltyFac * invL * aMag;
    put_row<OUT>(a, e, nd, c_side[s][ip], v, -mdot / a.pts, true);
  }
}

unsigned grid_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

FaceArgs face_args(nalu_ctx* ctx, const FaceSet& fs) {
  FaceArgs a{};
  a.n = fs.n;
  a.felem = fs.elem.p;
  a.fside = fs.side.p;
  a.dynp = fs.dynp.n ? fs.dynp.p : nullptr;
  a.conn = ctx->d_conn.p;
  a.x = ctx->fields[NALU_FIELD_COORDINATES].d.p;
  a.cap_face = -1;
  return a;
}

int check_set(nalu_ctx* ctx, int set) {
  if (set < 0 || set >= NALU_MAX_FACE_SETS) return set_error(ctx, NALU_ERR_ARG, "face set index");
  if (!ctx->face_sets[set].defined) return set_error(ctx, NALU_ERR_STATE, "face set not defined");
  return NALU_OK;
}

}  // namespace

void FaceSet::clear() {
  elem.free();
  side.free();
  dynp.free();
  h_elem.clear();
  h_side.clear();
  n = 0;
  defined = false;
}

}  // namespace nalu_gb300

using namespace nalu_gb300;

extern "C" {

int nalu_faceset_define(nalu_ctx* ctx, int set, int64_t n, const int64_t* elem, const int32_t* side) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || set < 0 || set >= NALU_MAX_FACE_SETS || n < 0 || (n > 0 && (!elem || !side)))
    return set_error(ctx, NALU_ERR_ARG, "face set args");
  if (!ctx->fields[NALU_FIELD_COORDINATES].set) return set_error(ctx, NALU_ERR_STATE, "no mesh");
  std::vector<int32_t> he((size_t)n);
  std::vector<uint8_t> hs((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    if (elem[i] < 0 || elem[i] >= ctx->n_elems || side[i] < 0 || side[i] > 5)
      return set_error(ctx, NALU_ERR_ARG, "face " + std::to_string(i) + ": element or side ordinal out of range");
    he[i] = (int32_t)elem[i];
    hs[i] = (uint8_t)side[i];
  }
  cudaSetDevice(ctx->device);
  FaceSet& fs = ctx->face_sets[set];
  fs.clear();
  if (n > 0) {
    NALU_CUDA(ctx, fs.elem.alloc(n));
    NALU_CUDA(ctx, fs.side.alloc(n));
    NALU_CUDA(ctx, cudaMemcpyAsync(fs.elem.p, he.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, ctx->stream));
    NALU_CUDA(ctx, cudaMemcpyAsync(fs.side.p, hs.data(), n, cudaMemcpyHostToDevice, ctx->stream));
    NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  fs.h_elem.swap(he);
  fs.h_side.swap(hs);
  fs.n = n;
  fs.defined = true;
  return NALU_OK;
}

int nalu_faceset_skin(nalu_ctx* ctx, int set, int64_t* n_faces) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || set < 0 || set >= NALU_MAX_FACE_SETS) return set_error(ctx, NALU_ERR_ARG, "face set args");
  if (!ctx->fields[NALU_FIELD_COORDINATES].set) return set_error(ctx, NALU_ERR_STATE, "no mesh");
  cudaSetDevice(ctx->device);
  const int64_t n_sides = 6 * ctx->n_elems;
  uint64_t cap = 1024;
  while (cap < 2 * (uint64_t)n_sides) cap <<= 1;
  DBuf<unsigned long long> keys;
  DBuf<uint32_t> cnt;
  DBuf<uint8_t> flags;
  DBuf<int> err;
  NALU_CUDA(ctx, keys.alloc((int64_t)cap));
  NALU_CUDA(ctx, cnt.alloc((int64_t)cap));
  NALU_CUDA(ctx, flags.alloc(n_sides));
  NALU_CUDA(ctx, err.alloc(1));
  NALU_CUDA(ctx, cudaMemsetAsync(keys.p, 0xff, sizeof(unsigned long long) * cap, ctx->stream));
  NALU_CUDA(ctx, cudaMemsetAsync(cnt.p, 0, sizeof(uint32_t) * cap, ctx->stream));
  NALU_CUDA(ctx, cudaMemsetAsync(err.p, 0, sizeof(int), ctx->stream));
  k_skin_insert<<<grid_for(n_sides, 256), 256, 0, ctx->stream>>>(n_sides, ctx->d_conn.p, keys.p, cnt.p, cap - 1,
                                                                 err.p);
  k_skin_mark<<<grid_for(n_sides, 256), 256, 0, ctx->stream>>>(n_sides, ctx->d_conn.p, keys.p, cnt.p, cap - 1,
                                                               flags.p, err.p);
  ctx->launches += 2;
  NALU_CUDA(ctx, cudaGetLastError());
  std::vector<uint8_t> hf((size_t)n_sides);
  int herr = 0;
  NALU_CUDA(ctx, cudaMemcpyAsync(hf.data(), flags.p, n_sides, cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (herr) return set_error(ctx, NALU_ERR_CUDA, "face hash table overflow");
  std::vector<int64_t> fe;
  std::vector<int32_t> fsd;
  for (int64_t i = 0; i < n_sides; ++i)
    if (hf[i]) {
      fe.push_back(i / 6);
      fsd.push_back((int32_t)(i % 6));
    }
  if (n_faces) *n_faces = (int64_t)fe.size();
  return nalu_faceset_define(ctx, set, (int64_t)fe.size(), fe.data(), fsd.data());
}

int nalu_faceset_size(nalu_ctx* ctx, int set, int64_t* n_faces) {
  if (!ctx || !n_faces) return NALU_ERR_ARG;
  int rc = check_set(ctx, set);
  if (rc) return rc;
  *n_faces = ctx->face_sets[set].n;
  return NALU_OK;
}

int nalu_faceset_get(nalu_ctx* ctx, int set, int64_t* elem, int32_t* side) {
  if (!ctx) return NALU_ERR_ARG;
  int rc = check_set(ctx, set);
  if (rc) return rc;
  const FaceSet& fs = ctx->face_sets[set];
  for (int64_t i = 0; i < fs.n; ++i) {
    if (elem) elem[i] = fs.h_elem[i];
    if (side) side[i] = fs.h_side[i];
  }
  return NALU_OK;
}

int nalu_faceset_dynamic_pressure(nalu_ctx* ctx, int set, const double* dynp) {
  if (!ctx) return NALU_ERR_ARG;
  int rc = check_set(ctx, set);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  FaceSet& fs = ctx->face_sets[set];
  fs.dynp.free();
  if (!dynp || fs.n == 0) return NALU_OK;
  NALU_CUDA(ctx, fs.dynp.alloc(4 * fs.n));
  NALU_CUDA(ctx, cudaMemcpyAsync(fs.dynp.p, dynp, sizeof(double) * 4 * fs.n, cudaMemcpyHostToDevice, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

int nalu_faceset_exposed_area(nalu_ctx* ctx, int set, double* area) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || !area) return NALU_ERR_ARG;
  int rc = check_set(ctx, set);
  if (rc) return rc;
  const FaceSet& fs = ctx->face_sets[set];
  if (fs.n == 0) return NALU_OK;
  cudaSetDevice(ctx->device);
  DBuf<double> d;
  NALU_CUDA(ctx, d.alloc(12 * fs.n));
  FaceArgs a = face_args(ctx, fs);
  a.area_out = d.p;
  k_face_area<<<grid_for(fs.n, kFaceThreads), kFaceThreads, 0, ctx->stream>>>(a);
  ctx->launches++;
  NALU_CUDA(ctx, cudaGetLastError());
  NALU_CUDA(ctx, cudaMemcpyAsync(area, d.p, sizeof(double) * 12 * fs.n, cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

int nalu_nodal_gradient_boundary(nalu_ctx* ctx, int set, int src_field, int dst_field, int shifted) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx) return NALU_ERR_ARG;
  int rc = check_set(ctx, set);
  if (rc) return rc;
  if (src_field < 0 || src_field >= NALU_FIELD_COUNT || dst_field < 0 || dst_field >= NALU_FIELD_COUNT ||
      src_field == NALU_FIELD_MDOT_SCS || dst_field == NALU_FIELD_MDOT_SCS || src_field == dst_field)
    return set_error(ctx, NALU_ERR_ARG, "gradient fields");
  const int sc = field_comps(src_field), dc = field_comps(dst_field);
  if (!((sc == 1 && dc == 3) || (sc == 3 && dc == 9)))
    return set_error(ctx, NALU_ERR_ARG, "gradient of a scalar needs a 3-vector field, of a vector a 9-component one");
  if (!ctx->fields[src_field].set) return set_error(ctx, NALU_ERR_STATE, "gradient source field not set");
  if (!ctx->fields[NALU_FIELD_DUAL_VOLUME].set)
    return set_error(ctx, NALU_ERR_STATE, "dual_nodal_volume not computed (nalu_compute_dual_volume)");
  if (!ctx->fields[dst_field].set || ctx->fields[dst_field].comps != dc)
    return set_error(ctx, NALU_ERR_STATE, "gradient field not computed (nalu_compute_nodal_gradient first)");
  const FaceSet& fs = ctx->face_sets[set];
  if (fs.n == 0) return NALU_OK;
  cudaSetDevice(ctx->device);
  FaceArgs a = face_args(ctx, fs);
  a.q = ctx->fields[src_field].d.p;
  a.dvol = ctx->fields[NALU_FIELD_DUAL_VOLUME].d.p;
  a.grad = ctx->fields[dst_field].d.p;
  if (sc == 1) k_grad_boundary<1><<<grid_for(fs.n, kFaceThreads), kFaceThreads, 0, ctx->stream>>>(a, shifted != 0);
  else k_grad_boundary<3><<<grid_for(fs.n, kFaceThreads), kFaceThreads, 0, ctx->stream>>>(a, shifted != 0);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "nodal gradient boundary");
}

static int face_kernel_setup(nalu_ctx* ctx, int set, int kernel, const nalu_assemble_opts* o, FaceArgs& a) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || !o) return NALU_ERR_ARG;
  int rc = check_set(ctx, set);
  if (rc) return rc;
  if (kernel != NALU_FACE_CONTINUITY_INFLOW && kernel != NALU_FACE_CONTINUITY_OPEN)
    return set_error(ctx, NALU_ERR_ARG, "unknown face kernel");
  if (!(o->proj_time_scale != 0.0)) return set_error(ctx, NALU_ERR_ARG, "proj_time_scale must be non-zero");
  auto need = [&](int f, const char* name) -> int {
    if (!ctx->fields[f].set) return set_error(ctx, NALU_ERR_STATE, std::string("field not set: ") + name);
    return NALU_OK;
  };
  if ((rc = need(NALU_FIELD_DENSITY, "density"))) return rc;
  a = face_args(ctx, ctx->face_sets[set]);
  a.rho = ctx->fields[NALU_FIELD_DENSITY].d.p;
  a.pts = o->proj_time_scale;
  a.shift_mdot = o->shift_mdot != 0;
  if (kernel == NALU_FACE_CONTINUITY_INFLOW) {
    if ((rc = need(NALU_FIELD_VELOCITY_BC, "cont_velocity_bc"))) return rc;
    a.u = ctx->fields[NALU_FIELD_VELOCITY_BC].d.p;
  } else {
    if ((rc = need(NALU_FIELD_VELOCITY, "velocity"))) return rc;
    if ((rc = need(NALU_FIELD_PRESSURE, "pressure"))) return rc;
    if ((rc = need(NALU_FIELD_PRESSURE_BC, "pressure_bc"))) return rc;
    if ((rc = need(NALU_FIELD_DPDX, "dpdx"))) return rc;
    a.u = ctx->fields[NALU_FIELD_VELOCITY].d.p;
    a.p = ctx->fields[NALU_FIELD_PRESSURE].d.p;
    a.pbc = ctx->fields[NALU_FIELD_PRESSURE_BC].d.p;
    a.gpdx = ctx->fields[NALU_FIELD_DPDX].d.p;
    a.shift_grad = o->shift_poisson != 0;
    a.lhs_shift = (o->shift_poisson != 0 || o->reduced_sens != 0);
  }
  return NALU_OK;
}

int nalu_assemble_faces(nalu_ctx* ctx, int set, int kernel, const nalu_assemble_opts* opts) {
  FaceArgs a{};
  int rc = face_kernel_setup(ctx, set, kernel, opts, a);
  if (rc) return rc;
  if (ctx->num_dof != 1) return set_error(ctx, NALU_ERR_STATE, "face kernels need a numDof 1 graph");
  if (a.n == 0) return NALU_OK;
  cudaSetDevice(ctx->device);
  a.rowptr = ctx->d_rowptr.p;
  a.slots = ctx->d_slots.p;
  a.values = ctx->d_values.p;
  a.rhs = ctx->d_rhs.p;
  if (kernel == NALU_FACE_CONTINUITY_INFLOW)
    k_cont_inflow<0><<<grid_for(a.n, kFaceThreads), kFaceThreads, 0, ctx->stream>>>(a);
  else
    k_cont_open<0><<<grid_for(a.n, kFaceThreads), kFaceThreads, 0, ctx->stream>>>(a);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "face assembly");
}

int nalu_capture_face(nalu_ctx* ctx, int set, int kernel, const nalu_assemble_opts* opts, int64_t face, double* lhs,
                      double* rhs) {
  FaceArgs a{};
  if (!lhs || !rhs) return set_error(ctx, NALU_ERR_ARG, "capture args");
  int rc = face_kernel_setup(ctx, set, kernel, opts, a);
  if (rc) return rc;
  if (face < 0 || face >= a.n) return set_error(ctx, NALU_ERR_ARG, "face out of range");
  cudaSetDevice(ctx->device);
  DBuf<double> dl, dr;
  NALU_CUDA(ctx, dl.alloc(64));
  NALU_CUDA(ctx, dr.alloc(8));
  NALU_CUDA(ctx, cudaMemsetAsync(dl.p, 0, sizeof(double) * 64, ctx->stream));
  NALU_CUDA(ctx, cudaMemsetAsync(dr.p, 0, sizeof(double) * 8, ctx->stream));
  a.cap_face = face;
  a.cap_lhs = dl.p;
  a.cap_rhs = dr.p;
  if (kernel == NALU_FACE_CONTINUITY_INFLOW) k_cont_inflow<2><<<1, 32, 0, ctx->stream>>>(a);
  else k_cont_open<2><<<1, 32, 0, ctx->stream>>>(a);
  ctx->launches++;
  NALU_CUDA(ctx, cudaGetLastError());
  NALU_CUDA(ctx, cudaMemcpyAsync(lhs, dl.p, sizeof(double) * 64, cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(rhs, dr.p, sizeof(double) * 8, cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

}  // extern "C"
