// assemble_df.cu -- the scalar assembly kernels (ScalarDiffElemKernel,
// ContinuityAdvElemKernel) with the element math in double-float (df64) on
// the FP32 pipes (hex8_elem_df.h).  FP64 stays where precision is set by the
// inputs and outputs: coordinate differences, the -lhs.p residual term, the
// conversion of element-matrix entries back to FP64 and the CRS scatter.
//
// A per-node pre-pass splits the nodal inputs once (w = rho u + tau Gpdx for
// continuity, the diffusion coefficient for ScalarDiff) into df64, so the
// element kernel gathers 8-byte df64 values instead of converting 8x per node.
#include <cuda_runtime.h>

#include <cstdint>

#include "assemble_df.cuh"
#include "assemble_ip.cuh"

namespace nalu_gb300 {

NALU_DF_VARIANTS(NALU_DF_EXTERN)
NALU_IP_VARIANTS(NALU_IP_EXTERN, 8)
NALU_IP_VARIANTS(NALU_IP_EXTERN, 16)

// (the splits and the double-float arithmetic use the FP32 and integer pipes:
// GB300's FP64 rate made the FP64 form of this pass FP64-bound, 74 us at 128^3)
// An input outside the pairs' range (inf, NaN, |x| >= 2^127) raises
// FLAG_NONFINITE: the element kernels' widening back to FP64 would turn it
// into a large finite value.
__global__ void k_prepass_k_df(const double* __restrict__ k, df64* __restrict__ out, int64_t n, int32_t* flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double kv = __ldg(k + i);
  out[i] = df_split_input(kv);
  if (!df_split_in_range(kv)) atomicAdd(flags + FLAG_NONFINITE, 1);
}

__global__ void k_prepass_w_df(const double* __restrict__ u, const double* __restrict__ gp,
                               const double* __restrict__ rho, df64 tau, df64* __restrict__ out, int64_t n,
                               int32_t* flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double rv = __ldg(rho + i);
  const df64 r = df_split_input(rv);
  bool ok = df_split_in_range(rv);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double uv = __ldg(u + 3 * i + d), gv = __ldg(gp + 3 * i + d);
    ok = ok && df_split_in_range(uv) && df_split_in_range(gv);
    out[3 * i + d] = df_nodal_w(r, uv, tau, gv);
  }
  if (!ok) atomicAdd(flags + FLAG_NONFINITE, 1);
}

// ComputeMdot in df64: one thread per element, the twelve SCS mass flow rates
template <bool SMDOT, bool SPOIS>
__global__ void __launch_bounds__(kAsmBlockDF, NALU_DF_MINB) k_mdot_df(int64_t n_elems, const int32_t* __restrict__ conn,
                                                                    const double* __restrict__ x,
                                                                    const df64* __restrict__ w,
                                                                    const double* __restrict__ p, df64 tau,
                                                                    double* __restrict__ mdot, int32_t* flags) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  int nd[8];
  {
    const int4* c4 = reinterpret_cast<const int4*>(conn + 8 * e);
    const int4 p0 = __ldg(c4), p1 = __ldg(c4 + 1);
    nd[0] = p0.x; nd[1] = p0.y; nd[2] = p0.z; nd[3] = p0.w;
    nd[4] = p1.x; nd[5] = p1.y; nd[6] = p1.z; nd[7] = p1.w;
  }
  double xe[8][3];
  df64 we[8][3], pe[8];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      xe[n][d] = __ldg(x + 3 * (int64_t)nd[n] + d);
      we[n][d] = w[3 * (int64_t)nd[n] + d];
    }
    pe[n] = df_split_bits(__ldg(p + nd[n]));
  }
  const double mindet = mdot_elem_df<SMDOT, SPOIS>(xe, we, pe, tau, mdot + 12 * e);
  if (!(mindet > 1.0e-50)) atomicAdd(flags + FLAG_NEG_JAC, 1);
}

int launch_mdot_df(nalu_ctx* ctx, const nalu_assemble_opts& o) {
  const int64_t n = ctx->n_nodes, E = ctx->n_elems;
  if (ctx->d_node_df.n < 3 * n) NALU_CUDA(ctx, ctx->d_node_df.alloc(3 * n));
  df64* w = reinterpret_cast<df64*>(ctx->d_node_df.p);
  k_prepass_w_df<<<nblk_df(n, 256), 256, 0, ctx->stream>>>(ctx->fields[NALU_FIELD_VELOCITY_RTM].d.p,
                                                        ctx->fields[NALU_FIELD_DPDX].d.p,
                                                        ctx->fields[NALU_FIELD_DENSITY].d.p,
                                                        df_split_input(o.proj_time_scale), w, n, ctx->d_flags.p);
  const unsigned grid = nblk_df(E, kAsmBlockDF);
  const double* x = ctx->fields[NALU_FIELD_COORDINATES].d.p;
  const double* p = ctx->fields[NALU_FIELD_PRESSURE].d.p;
  double* out = ctx->fields[NALU_FIELD_MDOT_SCS].d.p;
  const df64 tau = df_from_double(o.proj_time_scale);
  if (o.shift_mdot) {
    if (o.shift_poisson) k_mdot_df<true, true><<<grid, kAsmBlockDF, 0, ctx->stream>>>(E, ctx->d_conn.p, x, w, p, tau, out, ctx->d_flags.p);
    else k_mdot_df<true, false><<<grid, kAsmBlockDF, 0, ctx->stream>>>(E, ctx->d_conn.p, x, w, p, tau, out, ctx->d_flags.p);
  } else {
    if (o.shift_poisson) k_mdot_df<false, true><<<grid, kAsmBlockDF, 0, ctx->stream>>>(E, ctx->d_conn.p, x, w, p, tau, out, ctx->d_flags.p);
    else k_mdot_df<false, false><<<grid, kAsmBlockDF, 0, ctx->stream>>>(E, ctx->d_conn.p, x, w, p, tau, out, ctx->d_flags.p);
  }
  ctx->launches += 2;
  return cuda_check(ctx, cudaGetLastError(), "df64 mdot launch");
}

namespace {

template <int EPB>
void launch_ip(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, const AsmArgsDF& a, int out) {
  if (kernel == NALU_KERNEL_SCALAR_DIFF) {
    if (o.shifted_grad_op) launch_ip_variant<EPB, 0, 0, true, false>(ctx, a, out);
    else launch_ip_variant<EPB, 0, 0, false, false>(ctx, a, out);
    return;
  }
  const int mode = o.shift_poisson ? 2 : (o.reduced_sens ? 1 : 0);
  if (o.shift_mdot) {
    if (mode == 0) launch_ip_variant<EPB, 1, 0, false, true>(ctx, a, out);
    else if (mode == 1) launch_ip_variant<EPB, 1, 1, false, true>(ctx, a, out);
    else launch_ip_variant<EPB, 1, 2, false, true>(ctx, a, out);
  } else {
    if (mode == 0) launch_ip_variant<EPB, 1, 0, false, false>(ctx, a, out);
    else if (mode == 1) launch_ip_variant<EPB, 1, 1, false, false>(ctx, a, out);
    else launch_ip_variant<EPB, 1, 2, false, false>(ctx, a, out);
  }
}

// schedule: NALU_SCHEDULE_ELEMENT, _IP8 or _IP16 (resolved by the caller)
void launch_df(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, const AsmArgsDF& a, int out, int schedule) {
  if (schedule == NALU_SCHEDULE_IP8) return launch_ip<8>(ctx, kernel, o, a, out);
  if (schedule == NALU_SCHEDULE_IP16) return launch_ip<16>(ctx, kernel, o, a, out);
  if (kernel == NALU_KERNEL_SCALAR_DIFF) {
    if (o.shifted_grad_op) launch_df_variant<0, 0, true, false>(ctx, a, out);
    else launch_df_variant<0, 0, false, false>(ctx, a, out);
    return;
  }
  const int mode = o.shift_poisson ? 2 : (o.reduced_sens ? 1 : 0);
  if (o.shift_mdot) {
    if (mode == 0) launch_df_variant<1, 0, false, true>(ctx, a, out);
    else if (mode == 1) launch_df_variant<1, 1, false, true>(ctx, a, out);
    else launch_df_variant<1, 2, false, true>(ctx, a, out);
  } else {
    if (mode == 0) launch_df_variant<1, 0, false, false>(ctx, a, out);
    else if (mode == 1) launch_df_variant<1, 1, false, false>(ctx, a, out);
    else launch_df_variant<1, 2, false, false>(ctx, a, out);
  }
}

// the schedule a call runs: the option if set, else the context's tuned
// choice for the kernel, else one thread per SCS ip with 8 elements per block
int resolve_schedule(const nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o) {
  if (o.schedule >= NALU_SCHEDULE_ELEMENT && o.schedule <= NALU_SCHEDULE_IP16) return o.schedule;
  const int k = kernel == NALU_KERNEL_SCALAR_DIFF ? 0 : 1;
  return ctx->df_schedule[k] ? ctx->df_schedule[k] : NALU_SCHEDULE_IP8;
}

// split the nodal inputs into df64 (scratch owned by the context)
int prepass(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, AsmArgsDF& a) {
  const int64_t n = ctx->n_nodes;
  const int64_t need = kernel == NALU_KERNEL_SCALAR_DIFF ? n : 3 * n;
  if (ctx->d_node_df.n < need) NALU_CUDA(ctx, ctx->d_node_df.alloc(need));
  df64* out = reinterpret_cast<df64*>(ctx->d_node_df.p);
  if (kernel == NALU_KERNEL_SCALAR_DIFF) {
    k_prepass_k_df<<<nblk_df(n, 256), 256, 0, ctx->stream>>>(ctx->fields[NALU_FIELD_DIFF_COEFF].d.p, out, n,
                                                          ctx->d_flags.p);
  } else {
    k_prepass_w_df<<<nblk_df(n, 256), 256, 0, ctx->stream>>>(ctx->fields[NALU_FIELD_VELOCITY].d.p,
                                                          ctx->fields[NALU_FIELD_DPDX].d.p,
                                                          ctx->fields[NALU_FIELD_DENSITY].d.p,
                                                          df_split_input(o.proj_time_scale), out, n, ctx->d_flags.p);
  }
  ctx->launches++;
  a.nodal = out;
  return cuda_check(ctx, cudaGetLastError(), "df64 prepass");
}

AsmArgsDF base_args_df(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o) {
  AsmArgsDF a{};
  a.conn = ctx->d_conn.p;
  a.x = ctx->fields[NALU_FIELD_COORDINATES].d.p;
  a.f_a = kernel == NALU_KERNEL_SCALAR_DIFF ? ctx->fields[NALU_FIELD_SCALAR_Q].d.p : ctx->fields[NALU_FIELD_PRESSURE].d.p;
  a.inv_tau = df_from_double(1.0 / o.proj_time_scale);
  a.rowptr = ctx->d_rowptr.p;
  a.slots = ctx->d_slots.p;
  a.values = ctx->d_values.p;
  a.rhs = ctx->d_rhs.p;
  a.flags = ctx->d_flags.p;
  return a;
}

}  // namespace

int launch_assemble_df(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int scatter) {
  AsmArgsDF a = base_args_df(ctx, kernel, o);
  int rc = prepass(ctx, kernel, o, a);
  if (rc) return rc;
  const int schedule = resolve_schedule(ctx, kernel, o);
  if (scatter == NALU_SCATTER_COLOURED) {
    const int nc = (int)ctx->colour_offsets.size() - 1;
    for (int c = 0; c < nc; ++c) {
      AsmArgsDF ac = a;
      ac.elems = ctx->d_colour_elems.p + ctx->colour_offsets[c];
      ac.count = ctx->colour_offsets[c + 1] - ctx->colour_offsets[c];
      launch_df(ctx, kernel, o, ac, 1, schedule);
    }
  } else {
    a.count = ctx->n_elems;
    launch_df(ctx, kernel, o, a, 0, schedule);
  }
  return cuda_check(ctx, cudaGetLastError(), "df64 assemble launch");
}

int launch_capture_df(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int64_t elem, double* d_lhs,
                      double* d_rhs) {
  AsmArgsDF a = base_args_df(ctx, kernel, o);
  int rc = prepass(ctx, kernel, o, a);
  if (rc) return rc;
  a.count = 1;
  a.cap_elem = elem;
  a.cap_lhs = d_lhs;
  a.cap_rhs = d_rhs;
  launch_df(ctx, kernel, o, a, 2, resolve_schedule(ctx, kernel, o));
  return cuda_check(ctx, cudaGetLastError(), "df64 capture launch");
}

}  // namespace nalu_gb300
