// assemble.cu -- sm_103a kernels of the Hex8 CVFEM assembly path.
//
// Replaces AssembleElemSolverAlgorithm::execute (src/AssembleElemSolverAlgorithm.C:75-100):
// gather (fill_pre_req_data, src/ScratchViews.C:408-483), master-element
// views (ScratchViews.h:476-551), Kernel::execute and LinearSystem::sumInto
// (src/TpetraLinearSystem.C:1458-1522) fused into one kernel per element
// batch.  One thread owns one element; its 8x8 element matrix lives in a
// thread-private column of shared memory ([entry][thread], conflict free),
// and is scattered into the CRS values through a per-element slot table
// (byte offsets of each element column inside the node's CRS row).
#include <cuda_runtime.h>

#include <cstdint>

#include "hex8_elem.h"
#include "internal.h"

namespace nalu_gb300 {

constexpr int kAsmBlock = 64;

enum OutMode { OUT_ATOMIC = 0, OUT_COLOURED = 1, OUT_CAPTURE = 2 };

struct AsmArgs {
  const int32_t* __restrict__ conn;   // [E][8] LIDs
  const double* __restrict__ x;       // [n][3]
  const double* __restrict__ f_a;     // q (scalar diff) or pressure (continuity)
  const double* __restrict__ f_b;     // diff coeff (scalar diff) or density
  const double* __restrict__ f_u;     // velocity [n][3]
  const double* __restrict__ f_gp;    // dpdx [n][3]
  double tau, inv_tau;
  const int64_t* __restrict__ rowptr;
  const uint8_t* __restrict__ slots;  // [E][64]
  double* __restrict__ values;
  double* __restrict__ rhs;
  const int32_t* __restrict__ elems;  // element list (colour group) or null
  int64_t count;
  int32_t* flags;
  double* cap_lhs;
  double* cap_rhs;
  int64_t cap_elem;
};

struct SmemAcc {
  double (*s)[kAsmBlock];
  int t;
  __device__ __forceinline__ void set(int r, int c, double v) { s[r * 8 + c][t] = v; }
  __device__ __forceinline__ void add(int r, int c, double v) { s[r * 8 + c][t] += v; }
  __device__ __forceinline__ double get(int r, int c) const { return s[r * 8 + c][t]; }
};

__device__ __forceinline__ void load_conn(const int32_t* __restrict__ conn, int64_t e, int nd[8]) {
  const int4* c4 = reinterpret_cast<const int4*>(conn + 8 * e);
  const int4 a = __ldg(c4), b = __ldg(c4 + 1);
  nd[0] = a.x; nd[1] = a.y; nd[2] = a.z; nd[3] = a.w;
  nd[4] = b.x; nd[5] = b.y; nd[6] = b.z; nd[7] = b.w;
}

__device__ __forceinline__ void gather3(const double* __restrict__ f, const int nd[8], double v[8][3]) {
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const double* p = f + 3 * (int64_t)nd[n];
    v[n][0] = __ldg(p);
    v[n][1] = __ldg(p + 1);
    v[n][2] = __ldg(p + 2);
  }
}
__device__ __forceinline__ void gather1(const double* __restrict__ f, const int nd[8], double v[8]) {
#pragma unroll
  for (int n = 0; n < 8; ++n) v[n] = __ldg(f + nd[n]);
}

// KIND 0: ScalarDiff, 1: ContinuityAdv.  MODE: continuity grad-op mode (see
// hex8_elem.h).  SHIFT: scalar-diff shifted grad op.  SMDOT: shifted mdot
// shape functions.
template <int KIND, int MODE, bool SHIFT, bool SMDOT, int OUT>
__global__ void __launch_bounds__(kAsmBlock) k_assemble_scalar(AsmArgs a) {
  __shared__ double s_lhs[64][kAsmBlock];
  const int t = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * kAsmBlock + t;
  if (i >= a.count) return;
  const int64_t e = (OUT == OUT_CAPTURE) ? a.cap_elem : (a.elems ? (int64_t)a.elems[i] : i);
  int nd[8];
  load_conn(a.conn, e, nd);
  double x[8][3];
  gather3(a.x, nd, x);
  SmemAcc acc{s_lhs, t};
  double rhs[8];
  double pv[8];
  double mindet;
  bool rhs_from_lhs;
  if (KIND == 0) {
    double k[8];
    gather1(a.f_b, nd, k);
    mindet = scalar_diff_lhs<SHIFT>(x, k, acc);
    gather1(a.f_a, nd, pv);
#pragma unroll
    for (int r = 0; r < 8; ++r) rhs[r] = 0.0;
    rhs_from_lhs = true;
  } else {
    double w[8][3];
    {
      double u[8][3], g[8][3], rho[8];
      gather3(a.f_u, nd, u);
      gather3(a.f_gp, nd, g);
      gather1(a.f_b, nd, rho);
#pragma unroll
      for (int n = 0; n < 8; ++n)
#pragma unroll
        for (int d = 0; d < 3; ++d) w[n][d] = rho[n] * u[n][d] + a.tau * g[n][d];
    }
    gather1(a.f_a, nd, pv);
    mindet = continuity_elem<MODE, SMDOT>(x, w, a.inv_tau, pv, acc, rhs);
    rhs_from_lhs = (MODE != 1);
  }
  if (!(mindet > 1.0e-50)) atomicAdd(a.flags + FLAG_NEG_JAC, 1);

  if (OUT == OUT_CAPTURE) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      double s = rhs[r];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const double v = acc.get(r, c);
        a.cap_lhs[r * 8 + c] = v;
        if (rhs_from_lhs) s -= v * pv[c];
      }
      a.cap_rhs[r] = s;
    }
    return;
  }
  const uint8_t* sl = a.slots + 64 * e;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int64_t base = __ldg(a.rowptr + nd[r]);
    const uint2 o2 = __ldg(reinterpret_cast<const uint2*>(sl + 8 * r));
    double s = rhs[r];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const uint32_t word = c < 4 ? o2.x : o2.y;
      const int off = (word >> (8 * (c & 3))) & 0xff;
      const double v = acc.get(r, c);
      if (rhs_from_lhs) s -= v * pv[c];
      double* dst = a.values + base + off;
      if (OUT == OUT_ATOMIC) atomicAdd(dst, v);
      else *dst += v;
    }
    if (OUT == OUT_ATOMIC) atomicAdd(a.rhs + nd[r], s);
    else a.rhs[nd[r]] += s;
  }
}

// ComputeMdotElemAlgorithm: writes the element field mass_flow_rate_scs
template <bool SMDOT, bool SPOIS>
__global__ void __launch_bounds__(128) k_mdot(AsmArgs a, double* __restrict__ mdot) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.count) return;
  int nd[8];
  load_conn(a.conn, e, nd);
  double x[8][3], w[8][3], pv[8];
  gather3(a.x, nd, x);
  {
    double u[8][3], g[8][3], rho[8];
    gather3(a.f_u, nd, u);
    gather3(a.f_gp, nd, g);
    gather1(a.f_b, nd, rho);
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int d = 0; d < 3; ++d) w[n][d] = rho[n] * u[n][d] + a.tau * g[n][d];
  }
  gather1(a.f_a, nd, pv);
  double m[12];
  const double mindet = mdot_elem<SMDOT, SPOIS>(x, w, pv, a.tau, m);
  if (!(mindet > 1.0e-50)) atomicAdd(a.flags + FLAG_NEG_JAC, 1);
#pragma unroll
  for (int ip = 0; ip < 12; ++ip) mdot[12 * e + ip] = m[ip];
}

// ---------------------------------------------------------------------------
// graph helpers
// ---------------------------------------------------------------------------

// slot table: offset of element node c inside the node-graph row of node r
__global__ void k_slot_table(const int32_t* __restrict__ conn, const int64_t* __restrict__ nrowptr,
                             const int32_t* __restrict__ ncolind, uint8_t* __restrict__ slots, int64_t n_elems,
                             int32_t* flags) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  int nd[8];
  load_conn(conn, e, nd);
  for (int r = 0; r < 8; ++r) {
    const int64_t rb = nrowptr[nd[r]], re = nrowptr[nd[r] + 1];
    for (int c = 0; c < 8; ++c) {
      const int32_t key = nd[c];
      int64_t lo = rb, hi = re;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (ncolind[mid] < key) lo = mid + 1;
        else hi = mid;
      }
      int off = 0;
      if (lo >= re || ncolind[lo] != key) atomicAdd(flags + FLAG_GRAPH_MISS, 1);
      else if (lo - rb > 255) atomicAdd(flags + FLAG_CAPACITY, 1);
      else off = (int)(lo - rb);
      slots[64 * e + 8 * r + c] = (uint8_t)off;
    }
  }
}

// dof-level CRS from the node graph (fill_in_extra_dof_rows_per_node layout):
// row (a,d) lists, for every neighbour b in ascending order, columns nd*b+0..nd-1
__global__ void k_expand_rowptr(const int64_t* __restrict__ nrowptr, int64_t* __restrict__ rowptr,
                                int64_t n_nodes, int nd) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a > n_nodes) return;
  if (a == n_nodes) {
    rowptr[n_nodes * nd] = (int64_t)nd * nd * nrowptr[n_nodes];
    return;
  }
  const int64_t len = nrowptr[a + 1] - nrowptr[a];
  for (int d = 0; d < nd; ++d) rowptr[a * nd + d] = (int64_t)nd * nd * nrowptr[a] + (int64_t)d * nd * len;
}
__global__ void k_expand_colind(const int64_t* __restrict__ nrowptr, const int32_t* __restrict__ ncolind,
                                int32_t* __restrict__ colind, int64_t n_nodes, int nd) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.y + threadIdx.y;
  if (a >= n_nodes) return;
  const int64_t nb = nrowptr[a], len = nrowptr[a + 1] - nb;
  const int64_t base = (int64_t)nd * nd * nb;
  for (int64_t j = threadIdx.x; j < len * nd; j += blockDim.x) {
    const int32_t col = nd * ncolind[nb + j / nd] + (int32_t)(j % nd);
    for (int d = 0; d < nd; ++d) colind[base + (int64_t)d * nd * len + j] = col;
  }
}

// sumInto of caller-provided element matrices (host API path), atomics
__global__ void k_sum_into(const int32_t* __restrict__ conn, const int64_t* __restrict__ rowptr,
                           const uint8_t* __restrict__ slots, const int64_t* __restrict__ elems,
                           const double* __restrict__ lhs, const double* __restrict__ rhs, double* values,
                           double* sysrhs, int64_t n, int nd, int64_t n_elems, int32_t* flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t e = elems[i];
  if (e < 0 || e >= n_elems) {
    atomicAdd(flags + FLAG_GRAPH_MISS, 1);
    return;
  }
  int nodes[8];
  load_conn(conn, e, nodes);
  const int ne = 8 * nd;
  const double* L = lhs + (int64_t)ne * ne * i;
  const double* R = rhs + (int64_t)ne * i;
  for (int r = 0; r < 8; ++r)
    for (int di = 0; di < nd; ++di) {
      const int64_t row = (int64_t)nodes[r] * nd + di;
      const int64_t base = rowptr[row];
      for (int c = 0; c < 8; ++c) {
        const int off = slots[64 * e + 8 * r + c];
        for (int dj = 0; dj < nd; ++dj) atomicAdd(values + base + (int64_t)nd * off + dj, L[(r * nd + di) * ne + c * nd + dj]);
      }
      atomicAdd(sysrhs + row, R[r * nd + di]);
    }
}

// Dirichlet (mode 0: identity row, rhs = val), reset (mode 1: zero row and rhs),
// diag (mode 2: diag += val[0], rhs += val[1])
__global__ void k_bc_rows(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind, double* values,
                          double* rhs, const int32_t* __restrict__ rows, const double* __restrict__ vals, int64_t n,
                          int mode) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.y + threadIdx.y;
  if (k >= n) return;
  const int32_t r = rows[k];
  const int64_t b = rowptr[r], e = rowptr[r + 1];
  for (int64_t j = b + threadIdx.x; j < e; j += blockDim.x) {
    if (mode == 0) values[j] = (colind[j] == r) ? 1.0 : 0.0;
    else if (mode == 1) values[j] = 0.0;
    else if (colind[j] == r) values[j] += vals[2 * k];
  }
  if (threadIdx.x == 0) {
    if (mode == 0) rhs[r] = vals[k];
    else if (mode == 1) rhs[r] = 0.0;
    else rhs[r] += vals[2 * k + 1];
  }
}

__global__ void k_permute(const double* __restrict__ src, double* __restrict__ dst, const int32_t* __restrict__ lid,
                          int comps, int64_t n, int to_lid) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t l = lid[i];
  for (int c = 0; c < comps; ++c) {
    if (to_lid) dst[l * comps + c] = src[i * comps + c];
    else dst[i * comps + c] = src[l * comps + c];
  }
}

__global__ void k_fill(double* p, int64_t n, double v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// FP64 FMA throughput probe: independent FMA chains per thread
__global__ void __launch_bounds__(256) k_fp64_probe(double* out, int iters, double a, double b) {
  double v0 = threadIdx.x * 1e-9, v1 = v0 + 1, v2 = v0 + 2, v3 = v0 + 3, v4 = v0 + 4, v5 = v0 + 5, v6 = v0 + 6,
         v7 = v0 + 7;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      v0 = fma(v0, a, b); v1 = fma(v1, a, b); v2 = fma(v2, a, b); v3 = fma(v3, a, b);
      v4 = fma(v4, a, b); v5 = fma(v5, a, b); v6 = fma(v6, a, b); v7 = fma(v7, a, b);
    }
  }
  const double s = v0 + v1 + v2 + v3 + v4 + v5 + v6 + v7;
  if (s == 123.456) out[0] = s;  // keep the chains live
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
namespace {

inline int64_t blocks_for(int64_t n, int b) { return (n + b - 1) / b; }

AsmArgs base_args(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o) {
  AsmArgs a{};
  a.conn = ctx->d_conn.p;
  a.x = ctx->fields[NALU_FIELD_COORDINATES].d.p;
  if (kernel == NALU_KERNEL_SCALAR_DIFF) {
    a.f_a = ctx->fields[NALU_FIELD_SCALAR_Q].d.p;
    a.f_b = ctx->fields[NALU_FIELD_DIFF_COEFF].d.p;
  } else {
    a.f_a = ctx->fields[NALU_FIELD_PRESSURE].d.p;
    a.f_b = ctx->fields[NALU_FIELD_DENSITY].d.p;
    a.f_u = ctx->fields[NALU_FIELD_VELOCITY].d.p;
    a.f_gp = ctx->fields[NALU_FIELD_DPDX].d.p;
  }
  a.tau = o.proj_time_scale;
  a.inv_tau = 1.0 / o.proj_time_scale;
  a.rowptr = ctx->d_rowptr.p;
  a.slots = ctx->d_slots.p;
  a.values = ctx->d_values.p;
  a.rhs = ctx->d_rhs.p;
  a.flags = ctx->d_flags.p;
  return a;
}

template <int KIND, int MODE, bool SHIFT, bool SMDOT>
void launch_scalar_variant(nalu_ctx* ctx, AsmArgs a, int out) {
  const dim3 block(kAsmBlock);
  const dim3 grid((unsigned)blocks_for(a.count, kAsmBlock));
  if (a.count <= 0) return;
  if (out == OUT_ATOMIC) k_assemble_scalar<KIND, MODE, SHIFT, SMDOT, OUT_ATOMIC><<<grid, block, 0, ctx->stream>>>(a);
  else if (out == OUT_COLOURED) k_assemble_scalar<KIND, MODE, SHIFT, SMDOT, OUT_COLOURED><<<grid, block, 0, ctx->stream>>>(a);
  else k_assemble_scalar<KIND, MODE, SHIFT, SMDOT, OUT_CAPTURE><<<1, 1, 0, ctx->stream>>>(a);
  ctx->launches++;
}

// dispatch on the runtime options to a compiled variant
void launch_scalar(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, AsmArgs a, int out) {
  if (kernel == NALU_KERNEL_SCALAR_DIFF) {
    if (o.shifted_grad_op) launch_scalar_variant<0, 0, true, false>(ctx, a, out);
    else launch_scalar_variant<0, 0, false, false>(ctx, a, out);
    return;
  }
  const int mode = o.shift_poisson ? 2 : (o.reduced_sens ? 1 : 0);
  if (o.shift_mdot) {
    if (mode == 0) launch_scalar_variant<1, 0, false, true>(ctx, a, out);
    else if (mode == 1) launch_scalar_variant<1, 1, false, true>(ctx, a, out);
    else launch_scalar_variant<1, 2, false, true>(ctx, a, out);
  } else {
    if (mode == 0) launch_scalar_variant<1, 0, false, false>(ctx, a, out);
    else if (mode == 1) launch_scalar_variant<1, 1, false, false>(ctx, a, out);
    else launch_scalar_variant<1, 2, false, false>(ctx, a, out);
  }
}

}  // namespace

int launch_momentum(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int scatter, int64_t cap_elem,
                    double* cap_lhs, double* cap_rhs);

int launch_assemble(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int scatter) {
  if (kernel >= NALU_KERNEL_CONTINUITY_MASS) return launch_mass(ctx, kernel, o, scatter, -1, nullptr, nullptr);
  if (kernel >= NALU_KERNEL_MOMENTUM_ADV_DIFF) return launch_momentum(ctx, kernel, o, scatter, -1, nullptr, nullptr);
  if (o.arith == NALU_ARITH_DF64) return launch_assemble_df(ctx, kernel, o, scatter);
  AsmArgs a = base_args(ctx, kernel, o);
  if (scatter == NALU_SCATTER_COLOURED) {
    const int nc = (int)ctx->colour_offsets.size() - 1;
    for (int c = 0; c < nc; ++c) {
      AsmArgs ac = a;
      ac.elems = ctx->d_colour_elems.p + ctx->colour_offsets[c];
      ac.count = ctx->colour_offsets[c + 1] - ctx->colour_offsets[c];
      launch_scalar(ctx, kernel, o, ac, OUT_COLOURED);
    }
  } else {
    a.count = ctx->n_elems;
    launch_scalar(ctx, kernel, o, a, OUT_ATOMIC);
  }
  return cuda_check(ctx, cudaGetLastError(), "assemble launch");
}

int launch_capture(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int64_t elem, double* d_lhs,
                   double* d_rhs) {
  if (kernel >= NALU_KERNEL_CONTINUITY_MASS) return launch_mass(ctx, kernel, o, 0, elem, d_lhs, d_rhs);
  if (kernel >= NALU_KERNEL_MOMENTUM_ADV_DIFF) return launch_momentum(ctx, kernel, o, 0, elem, d_lhs, d_rhs);
  if (o.arith == NALU_ARITH_DF64) return launch_capture_df(ctx, kernel, o, elem, d_lhs, d_rhs);
  AsmArgs a = base_args(ctx, kernel, o);
  a.count = 1;
  a.cap_elem = elem;
  a.cap_lhs = d_lhs;
  a.cap_rhs = d_rhs;
  launch_scalar(ctx, kernel, o, a, OUT_CAPTURE);
  return cuda_check(ctx, cudaGetLastError(), "capture launch");
}

int launch_mdot(nalu_ctx* ctx, const nalu_assemble_opts& o) {
  if (o.arith == NALU_ARITH_DF64) return launch_mdot_df(ctx, o);
  AsmArgs a = base_args(ctx, NALU_KERNEL_CONTINUITY_ADV, o);
  a.f_u = ctx->fields[NALU_FIELD_VELOCITY_RTM].d.p;
  a.count = ctx->n_elems;
  double* out = ctx->fields[NALU_FIELD_MDOT_SCS].d.p;
  const dim3 grid((unsigned)blocks_for(a.count, 128));
  if (o.shift_mdot) {
    if (o.shift_poisson) k_mdot<true, true><<<grid, 128, 0, ctx->stream>>>(a, out);
    else k_mdot<true, false><<<grid, 128, 0, ctx->stream>>>(a, out);
  } else {
    if (o.shift_poisson) k_mdot<false, true><<<grid, 128, 0, ctx->stream>>>(a, out);
    else k_mdot<false, false><<<grid, 128, 0, ctx->stream>>>(a, out);
  }
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "mdot launch");
}

int launch_slot_table(nalu_ctx* ctx) {
  k_slot_table<<<(unsigned)blocks_for(ctx->n_elems, 128), 128, 0, ctx->stream>>>(
      ctx->d_conn.p, ctx->d_nrowptr.p, ctx->d_ncolind.p, ctx->d_slots.p, ctx->n_elems, ctx->d_flags.p);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "slot table launch");
}

int launch_expand_graph(nalu_ctx* ctx) {
  const int nd = ctx->num_dof;
  k_expand_rowptr<<<(unsigned)blocks_for(ctx->n_nodes + 1, 256), 256, 0, ctx->stream>>>(
      ctx->d_nrowptr.p, ctx->d_rowptr.p, ctx->n_nodes, nd);
  const dim3 blk(32, 8);
  k_expand_colind<<<(unsigned)blocks_for(ctx->n_nodes, 8), blk, 0, ctx->stream>>>(
      ctx->d_nrowptr.p, ctx->d_ncolind.p, ctx->d_colind.p, ctx->n_nodes, nd);
  ctx->launches += 2;
  return cuda_check(ctx, cudaGetLastError(), "expand graph launch");
}

int launch_sum_into(nalu_ctx* ctx, int64_t n, const int64_t* d_elems, const double* d_lhs, const double* d_rhs) {
  k_sum_into<<<(unsigned)blocks_for(n, 64), 64, 0, ctx->stream>>>(ctx->d_conn.p, ctx->d_rowptr.p, ctx->d_slots.p,
                                                                  d_elems, d_lhs, d_rhs, ctx->d_values.p,
                                                                  ctx->d_rhs.p, n, ctx->num_dof, ctx->n_elems,
                                                                  ctx->d_flags.p);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "sum_into launch");
}

int launch_bc_rows(nalu_ctx* ctx, int64_t n, const int32_t* d_rows, const double* d_vals, int mode) {
  const dim3 blk(32, 8);
  k_bc_rows<<<(unsigned)blocks_for(n, 8), blk, 0, ctx->stream>>>(ctx->d_rowptr.p, ctx->d_colind.p,
                                                                 ctx->d_values.p, ctx->d_rhs.p, d_rows, d_vals, n,
                                                                 mode);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "bc rows launch");
}

int launch_permute_in(nalu_ctx* ctx, const double* src, double* dst, int comps, int64_t n) {
  k_permute<<<(unsigned)blocks_for(n, 256), 256, 0, ctx->stream>>>(src, dst, ctx->d_lid.p, comps, n, 1);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "permute launch");
}
int launch_permute_in_on(nalu_ctx* ctx, cudaStream_t st, const double* src, double* dst, int comps, int64_t n) {
  k_permute<<<(unsigned)blocks_for(n, 256), 256, 0, st>>>(src, dst, ctx->d_lid.p, comps, n, 1);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "permute launch");
}
int launch_permute_out(nalu_ctx* ctx, const double* src, double* dst, int comps, int64_t n) {
  k_permute<<<(unsigned)blocks_for(n, 256), 256, 0, ctx->stream>>>(src, dst, ctx->d_lid.p, comps, n, 0);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "permute launch");
}
int launch_fill(nalu_ctx* ctx, double* p, int64_t n, double v) {
  if (n <= 0) return NALU_OK;
  k_fill<<<(unsigned)blocks_for(n, 256), 256, 0, ctx->stream>>>(p, n, v);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "fill launch");
}

int probe_fp64(nalu_ctx* ctx, double* tflops) {
  DBuf<double> out;
  NALU_CUDA(ctx, out.alloc(1));
  const int blocks = ctx->sm_count * 8, threads = 256, iters = 2048;
  k_fp64_probe<<<blocks, threads, 0, ctx->stream>>>(out.p, 16, 0.999999, 1e-7);  // warm-up
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, ctx->stream);
  k_fp64_probe<<<blocks, threads, 0, ctx->stream>>>(out.p, iters, 0.999999, 1e-7);
  cudaEventRecord(e1, ctx->stream);
  ctx->launches += 2;
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  out.free();
  NALU_CUDA(ctx, err);
  const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return NALU_OK;
}

}  // namespace nalu_gb300
