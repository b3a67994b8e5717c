// cg_fast.cu -- Jacobi-preconditioned CG with three kernels per iteration on a
// sliced-ELL copy of the CRS matrix.
//
// Layout: SELL-32 (slices of 32 consecutive rows; entry k of every row of a
// slice stored contiguously, so one thread per row reads coalesced; rows
// shorter than the slice are padded with their own diagonal index and 0).
// The copy is made once per solve from the assembled CRS values (FP64 or
// FP32 for the mixed-precision inner solve).
//
// pcg_df (the FP64 solve) keeps x, r, p and q = A p as FP32 pairs (about 48
// significant bits) so that no iteration kernel issues an FP64 instruction per
// row; x and r are split on entry and joined back to FP64 on exit.
//
// Iteration k (rz_k = r_k . z_k, z_k = D^-1 r_k):
//   K0  beta = rz_k / rz_{k-1};  p = z + beta p
//   K1  q = A p (one multiply-add per stored entry);  partial sums of p . q
//   K2  alpha = rz_k / (p . q);  x += alpha p;  r -= alpha q;
//       z = D^-1 r;  partial sums of r.z and r.r
// Every block re-reduces the previous kernel's 1024 partials in the same
// order, so all blocks use bit-identical alpha/beta and no scalar kernel or
// host round trip sits between the kernels.  (Forming p inside the SpMV
// gather instead would double its FP64 multiply-adds; on GB300 the SpMV is
// then FP64-issue bound rather than HBM bound.)  The rz partial buffers
// alternate between even and odd iterations; a chunk of iterations is
// captured once into a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <type_traits>
#include <vector>

#include "internal.h"
#include "reduce.cuh"
#include "spmv_df.cuh"

namespace nalu_gb300 {

constexpr int kSlice = 32;
constexpr int kCgBlocks = 1024;
constexpr int kCgThreads = 256;

namespace {

using red::block_store;
using red::block_total;
using red::warp_sum_d;

// slice lengths (max row length in each slice of 32 rows)
__global__ void k_sell_len(int64_t n, const int64_t* __restrict__ rp, int32_t* __restrict__ slen, int64_t nslices) {
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (gw >= nslices) return;
  const int64_t row = gw * kSlice + lane;
  int len = row < n ? (int)(rp[row + 1] - rp[row]) : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) len = max(len, __shfl_xor_sync(0xffffffffu, len, o));
  if (lane == 0) slen[gw] = len;
}

template <class VT>
__device__ __forceinline__ VT sell_value(double v) {
  return (VT)v;
}
template <>
__device__ __forceinline__ float2 sell_value<float2>(double v) {
  return split_df(v);
}

template <class VT>
__global__ void k_sell_fill(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            const double* __restrict__ v, const int64_t* __restrict__ sptr,
                            const int32_t* __restrict__ slen, int32_t* __restrict__ scol, VT* __restrict__ sval) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t s = row / kSlice;
  const int lane = (int)(row % kSlice);
  if (row >= n) return;
  const int64_t b = rp[row], len = rp[row + 1] - b;
  const int sl = slen[s];
  const int64_t base = sptr[s] + lane;
  for (int k = 0; k < sl; ++k) {
    const bool real = k < len;
    scol[base + (int64_t)k * kSlice] = real ? ci[b + k] : (int32_t)row;
    sval[base + (int64_t)k * kSlice] = sell_value<VT>(real ? v[b + k] : 0.0);
  }
}

// 16-bit column offsets: one warp per slice; for entry k the base is the
// smallest column of the slice's 32 rows, and a slice whose columns at some k
// spread over more than 65535 is marked wide (it keeps the 32-bit indices)
__global__ void k_sell_c16(int64_t nslices, const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                           const int32_t* __restrict__ scol, uint16_t* __restrict__ col16,
                           int32_t* __restrict__ cbase, uint8_t* __restrict__ wide) {
  const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (s >= nslices) return;
  const int64_t b0 = sptr[s];
  const int len = slen[s];
  bool too_wide = false;
  for (int k = 0; k < len; ++k) {
    const int32_t c = scol[b0 + (int64_t)k * 32 + lane];
    int32_t lo = c, hi = c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((int64_t)hi - lo > 65535) too_wide = true;
    col16[b0 + (int64_t)k * 32 + lane] = (uint16_t)(c - lo);
    if (lane == 0) cbase[b0 / 32 + k] = lo;
  }
  if (lane == 0) wide[s] = too_wide ? 1 : 0;
}

// z = D^-1 r ; partials of r.z and r.r
template <class T>
__global__ void __launch_bounds__(kCgThreads) k_cg_init(int64_t n, const T* __restrict__ r, const T* __restrict__ dinv,
                                                        T* __restrict__ z, double* __restrict__ rz_part,
                                                        double* __restrict__ rr_part) {
  __shared__ double sh[33];
  T rz = 0, rr = 0;  // arithmetic in T (FP32 for the FP32-inner solve), block sums in FP64
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T ri = r[i];
    const T zi = dinv[i] * ri;
    z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  block_store((double)rz, rz_part + blockIdx.x, sh);
  block_store((double)rr, rr_part + blockIdx.x, sh);
}

// p = z + beta p with beta = rz_cur / rz_prev (beta = 0 on the first iteration)
template <class T>
__global__ void __launch_bounds__(kCgThreads) k_cg_pupdate(int64_t n, const T* __restrict__ z, T* __restrict__ p,
                                                           const double* __restrict__ rz_cur,
                                                           const double* __restrict__ rz_prev, int first) {
  __shared__ double sh[33];
  double beta = 0.0;
  if (!first) {
    const double a = block_total(rz_cur, kCgBlocks, sh);
    const double b = block_total(rz_prev, kCgBlocks, sh);
    beta = a / b;
  }
  const T b = (T)beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = first ? z[i] : z[i] + b * p[i];
}

// q = A p on the SELL-32 copy (one multiply-add per stored entry, in stored
// order); partials of p.q.  Column and value loads go out in predicated
// groups of eight ahead of their gathers (past the row's length: column of
// the group's first entry, value 0).
template <class T, class VT>
__global__ void __launch_bounds__(kCgThreads) k_cg_spmv(int64_t n, int64_t nrows_padded, const int64_t* __restrict__ sptr,
                                                        const int32_t* __restrict__ slen, const int32_t* __restrict__ scol,
                                                        const VT* __restrict__ sval, const T* __restrict__ p,
                                                        T* __restrict__ q, double* __restrict__ pq_part) {
  __shared__ double sh[33];
  T dot = 0;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < nrows_padded;
       row += (int64_t)gridDim.x * blockDim.x) {
    if (row >= n) continue;
    const int64_t s = row / kSlice;
    const int len = __ldg(slen + s);
    const int64_t base = __ldg(sptr + s) + (row % kSlice);
    T acc = 0;
    for (int k = 0; k < len; k += 8) {
      int32_t c[8];
      VT v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const bool in = k + u < len;
        const int64_t off = base + (int64_t)(in ? k + u : k) * kSlice;
        c[u] = __ldg(scol + off);
        v[u] = in ? __ldg(sval + off) : (VT)0;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) acc += (T)v[u] * __ldg(p + c[u]);
    }
    q[row] = acc;
    dot += p[row] * acc;
  }
  block_store((double)dot, pq_part + blockIdx.x, sh);
}

template <class T>
__global__ void __launch_bounds__(kCgThreads) k_cg_axpy(int64_t n, T* __restrict__ x, const T* __restrict__ p,
                                                        T* __restrict__ r, const T* __restrict__ q,
                                                        T* __restrict__ z, const T* __restrict__ dinv,
                                                        const double* __restrict__ rz_cur,
                                                        const double* __restrict__ pq_part,
                                                        double* __restrict__ rz_next, double* __restrict__ rr_part) {
  __shared__ double sh[33];
  const double rz = block_total(rz_cur, kCgBlocks, sh);
  const double pq = block_total(pq_part, kCgBlocks, sh);
  const T alpha = (T)(rz / pq);
  T rzn = 0, rr = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = x[i] + alpha * p[i];
    const T ri = r[i] - alpha * q[i];
    r[i] = ri;
    const T zi = dinv[i] * ri;
    z[i] = zi;
    rzn += ri * zi;
    rr += ri * ri;
  }
  block_store((double)rzn, rz_next + blockIdx.x, sh);
  block_store((double)rr, rr_part + blockIdx.x, sh);
}

template <class T, class VT>
void cg_iteration(nalu_ctx* ctx, int k, int first, int64_t n, int64_t npad, const int64_t* sptr, const int32_t* slen,
                  const int32_t* scol, const VT* sval, T* x, T* r, T* z, T* p, T* q, const T* dinv,
                  double* rzbuf[2], double* pq_part, double* rr_part) {
  const int cur = k & 1, prev = cur ^ 1;
  k_cg_pupdate<T><<<kCgBlocks, kCgThreads, 0, ctx->stream>>>(n, z, p, rzbuf[cur], rzbuf[prev], first);
  k_cg_spmv<T, VT><<<kCgBlocks, kCgThreads, 0, ctx->stream>>>(n, npad, sptr, slen, scol, sval, p, q, pq_part);
  k_cg_axpy<T><<<kCgBlocks, kCgThreads, 0, ctx->stream>>>(n, x, p, r, q, z, dinv, rzbuf[cur], pq_part, rzbuf[prev],
                                                          rr_part);
  ctx->launches += 3;
}

// ---- FP64 Jacobi-CG with the df64 SpMV and single-block scalar reductions ----
__global__ void k_convert_f(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// scalars: cs[CS_RZ] = r.z, cs[CS_ALPHA], cs[CS_BETA], cs[CS_RR] = r.r, cs[CS_PQ]
enum { CS_RZ = 0, CS_ALPHA = 1, CS_BETA = 2, CS_RR = 3, CS_PQ = 4 };

// Jacobi with the FP32-rounded inverse diagonal (the same one the iterations use)
__global__ void __launch_bounds__(kCgThreads) k_cgd_init(int64_t n, const double* __restrict__ r,
                                                         const float* __restrict__ dinvf, float2* __restrict__ r2,
                                                         float2* __restrict__ x2, double* __restrict__ part,
                                                         unsigned* __restrict__ cnt, double* __restrict__ cs) {
  __shared__ double sh[33];
  float zh = 0.0f, zl = 0.0f, rh = 0.0f, rl = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 rs = split_df(r[i]);
    r2[i] = rs;
    x2[i] = make_float2(0.0f, 0.0f);
    acc_sq_df(zh, zl, rs, dinvf[i]);
    acc_sq_df(rh, rl, rs, 1.0f);
  }
  const double v[2] = {join_df(make_float2(zh, zl)), join_df(make_float2(rh, rl))};
  double t[2];
  if (red::grid_reduce<2>(v, part, kCgBlocks, cnt, t, sh) && threadIdx.x == 0) {
    cs[CS_RZ] = t[0];
    cs[CS_RR] = t[1];
  }
}

// p = D^-1 r + beta p (FP32 pairs)
__global__ void __launch_bounds__(kCgThreads) k_cgd_pupdate(int64_t n, const float2* __restrict__ r2,
                                                            const float* __restrict__ dinvf,
                                                            float2* __restrict__ p, const double* __restrict__ cs,
                                                            int first) {
  const float2 beta = split_df(first ? 0.0 : cs[CS_BETA]);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 z = fma_df(r2[i], make_float2(dinvf[i], 0.0f), make_float2(0.0f, 0.0f));
    p[i] = first ? z : fma_df(beta, p[i], z);
  }
}

// resident blocks per SM the SpMV's register allocation must allow
#ifndef NALU_CG_SPMV_MINB
#define NALU_CG_SPMV_MINB 4  // 64 registers: 4 blocks of 256 (measured best: 5 spills, 1 takes 72)
#endif

// q = A p (FP32 pairs); alpha = r.z / p.q by the last block
__global__ void __launch_bounds__(kCgThreads, NALU_CG_SPMV_MINB) k_cgd_spmv(int64_t n, int64_t npad, const int64_t* __restrict__ sptr,
                                                         const int32_t* __restrict__ slen,
                                                         const int32_t* __restrict__ scol,
                                                         const uint16_t* __restrict__ col16,
                                                         const int32_t* __restrict__ cbase,
                                                         const uint8_t* __restrict__ wide,
                                                         const float2* __restrict__ sval,
                                                         const float2* __restrict__ p, float2* __restrict__ q2,
                                                         double* __restrict__ part, unsigned* __restrict__ cnt,
                                                         double* __restrict__ cs) {
  __shared__ double sh[33];
  float dh = 0.0f, dl = 0.0f;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < npad;
       row += (int64_t)gridDim.x * blockDim.x) {
    if (row >= n) continue;
    const int64_t s = row / kSlice;
    const int64_t b0 = __ldg(sptr + s);
    const float2 qi = __ldg(wide + s) ? sell_row_df2(b0 + (row % kSlice), __ldg(slen + s), scol, sval, p)
                                      : sell_row_df2_c16(b0 + (row % kSlice), __ldg(slen + s), col16,
                                                         cbase + b0 / kSlice, sval, p);
    q2[row] = qi;
    acc_mul_df(dh, dl, p[row], qi);
  }
  const double v[1] = {join_df(make_float2(dh, dl))};
  double t[1];
  if (red::grid_reduce<1>(v, part, kCgBlocks, cnt, t, sh) && threadIdx.x == 0) {
    cs[CS_PQ] = t[0];
    cs[CS_ALPHA] = cs[CS_RZ] / t[0];
  }
}

// x += alpha p; r -= alpha q; r.D^-1 r and r.r, all as FP32 pairs (no FP64
// instruction per row); beta = rz_new / rz by the last block
__global__ void __launch_bounds__(kCgThreads) k_cgd_axpy(int64_t n, float2* __restrict__ x2,
                                                         const float2* __restrict__ p, float2* __restrict__ r2,
                                                         const float2* __restrict__ q2,
                                                         const float* __restrict__ dinvf,
                                                         double* __restrict__ part, unsigned* __restrict__ cnt,
                                                         double* __restrict__ cs) {
  __shared__ double sh[33];
  const float2 alpha = split_df(cs[CS_ALPHA]);
  const float2 nalpha = make_float2(-alpha.x, -alpha.y);
  float zh = 0.0f, zl = 0.0f, rh = 0.0f, rl = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x2[i] = fma_df(alpha, p[i], x2[i]);
    const float2 rs = fma_df(nalpha, q2[i], r2[i]);
    r2[i] = rs;
    acc_sq_df(zh, zl, rs, dinvf[i]);
    acc_sq_df(rh, rl, rs, 1.0f);
  }
  const double v[2] = {join_df(make_float2(zh, zl)), join_df(make_float2(rh, rl))};
  double t[2];
  if (red::grid_reduce<2>(v, part, kCgBlocks, cnt, t, sh) && threadIdx.x == 0) {
    cs[CS_BETA] = t[0] / cs[CS_RZ];
    cs[CS_RZ] = t[0];
    cs[CS_RR] = t[1];
  }
}

// iterate and residual back to FP64
__global__ void k_cgd_finish(int64_t n, const float2* __restrict__ x2, const float2* __restrict__ r2,
                             double* __restrict__ x, double* __restrict__ r) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = join_df(x2[i]);
    r[i] = join_df(r2[i]);
  }
}

}  // namespace

// Build the SELL-32 copy of the context's matrix (values as VT).
template <class VT>
int sell_build(nalu_ctx* ctx, SellMatrix& S, const VT** vals_out) {
  const int64_t n = ctx->n_rows;
  const int64_t ns = (n + kSlice - 1) / kSlice;
  if (S.len.n < ns) NALU_CUDA(ctx, S.len.alloc(ns));
  if (S.ptr.n < ns + 1) NALU_CUDA(ctx, S.ptr.alloc(ns + 1));
  k_sell_len<<<(unsigned)((ns * 32 + 255) / 256), 256, 0, ctx->stream>>>(n, ctx->d_rowptr.p, S.len.p, ns);
  ctx->launches++;
  std::vector<int32_t> hl(ns);
  NALU_CUDA(ctx, cudaMemcpyAsync(hl.data(), S.len.p, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<int64_t> hp(ns + 1, 0);
  for (int64_t s = 0; s < ns; ++s) hp[s + 1] = hp[s] + (int64_t)hl[s] * kSlice;
  const int64_t total = hp[ns];
  NALU_CUDA(ctx, cudaMemcpyAsync(S.ptr.p, hp.data(), sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice, ctx->stream));
  if (S.col.n < total) NALU_CUDA(ctx, S.col.alloc(total));
  VT* vals = nullptr;
  if constexpr (std::is_same<VT, float2>::value) {
    if (S.val2.n < total) NALU_CUDA(ctx, S.val2.alloc(total));
    vals = reinterpret_cast<VT*>(S.val2.p);
  } else if constexpr (sizeof(VT) == 8) {
    if (S.vald.n < total) NALU_CUDA(ctx, S.vald.alloc(total));
    vals = reinterpret_cast<VT*>(S.vald.p);
  } else {
    if (S.valf.n < total) NALU_CUDA(ctx, S.valf.alloc(total));
    vals = reinterpret_cast<VT*>(S.valf.p);
  }
  k_sell_fill<VT><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(n, ctx->d_rowptr.p, ctx->d_colind.p,
                                                                        ctx->d_values.p, S.ptr.p, S.len.p, S.col.p,
                                                                        vals);
  ctx->launches++;
  S.nslices = ns;
  S.stored = total;
  S.c16_valid = false;
  *vals_out = vals;
  NALU_CUDA(ctx, cudaMemcpyAsync(S.ptr.p, hp.data(), sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return cuda_check(ctx, cudaGetLastError(), "sell build");
}

int sell_c16_ensure(nalu_ctx* ctx, SellMatrix& S) {
  if (S.c16_valid) return NALU_OK;
  if (S.col16.n < S.stored) NALU_CUDA(ctx, S.col16.alloc(S.stored));
  if (S.cbase.n < S.stored / kSlice + 1) NALU_CUDA(ctx, S.cbase.alloc(S.stored / kSlice + 1));
  if (S.wide.n < S.nslices) NALU_CUDA(ctx, S.wide.alloc(S.nslices));
  k_sell_c16<<<(unsigned)((S.nslices * 32 + 255) / 256), 256, 0, ctx->stream>>>(S.nslices, S.ptr.p, S.len.p, S.col.p,
                                                                                S.col16.p, S.cbase.p, S.wide.p);
  ctx->launches++;
  const int rc = cuda_check(ctx, cudaGetLastError(), "sell c16");
  if (rc == NALU_OK) S.c16_valid = true;
  return rc;
}

// Jacobi-CG on A x = r (x from 0), vectors of type T, matrix values VT.
// r holds the initial residual; on return x holds the solution increment.
template <class T, class VT>
int pcg_fast(nalu_ctx* ctx, const VT* sval, const SellMatrix& S, T* x, T* r, T* z, T* p0, T* p1, T* q,
             const T* dinv, double rtol, double r0norm, int max_it, int check_every, int* iters_out) {
  const int64_t n = ctx->n_rows;
  const int64_t npad = S.nslices * kSlice;
  DBuf<double>& part = ctx->sw.partial;
  if (part.n < 4 * kCgBlocks) NALU_CUDA(ctx, part.alloc(4 * kCgBlocks));
  double* rzbuf[2] = {part.p, part.p + kCgBlocks};
  double* pq_part = part.p + 2 * kCgBlocks;
  double* rr_part = part.p + 3 * kCgBlocks;
  NALU_CUDA(ctx, cudaMemsetAsync(x, 0, sizeof(T) * n, ctx->stream));
  k_cg_init<T><<<kCgBlocks, kCgThreads, 0, ctx->stream>>>(n, r, dinv, z, rzbuf[0], rr_part);
  ctx->launches++;
  // iteration 0 (p_0 = z_0) outside the graph
  cg_iteration<T, VT>(ctx, 0, 1, n, npad, S.ptr.p, S.len.p, S.col.p, sval, x, r, z, p0, q, dinv, rzbuf, pq_part,
                      rr_part);
  int chunk = check_every > 0 ? check_every : 50;
  chunk += chunk & 1;  // even: the buffer pattern repeats every two iterations
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "begin capture");
  for (int k = 1; k <= chunk; ++k)
    cg_iteration<T, VT>(ctx, k, 0, n, npad, S.ptr.p, S.len.p, S.col.p, sval, x, r, z, p0, q, dinv, rzbuf, pq_part,
                        rr_part);
  ce = cudaStreamEndCapture(ctx->stream, &graph);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "end capture");
  ce = cudaGraphInstantiate(&exec, graph, 0);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cuda_check(ctx, ce, "instantiate");
  }
  std::vector<double> hrr(kCgBlocks);
  int it = 1, rc = NALU_OK;
  const double stop = rtol * r0norm;
  auto converged = [&](bool* bad) {
    cudaMemcpyAsync(hrr.data(), rr_part, sizeof(double) * kCgBlocks, cudaMemcpyDeviceToHost, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      *bad = true;
      return false;
    }
    double s = 0.0;
    for (double v : hrr) s += v;
    *bad = !std::isfinite(s);
    return std::sqrt(s) <= stop;
  };
  bool bad = false;
  if (!converged(&bad) && !bad) {
    while (it < max_it) {
      cudaGraphLaunch(exec, ctx->stream);
      it += chunk;
      if (converged(&bad) || bad) break;
    }
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  *iters_out = it;
  if (bad) return set_error(ctx, NALU_ERR_NONFINITE, "CG breakdown (non-finite residual)");
  if (it >= max_it) return NALU_ERR_NOT_CONVERGED;
  return rc;
}

// grid of one full wave of `kernel`: SMs x resident blocks, capped at kCgBlocks
unsigned wave_grid(nalu_ctx* ctx, const void* kernel, int threads) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  return (unsigned)std::min(kCgBlocks, per_sm * std::max(1, ctx->sm_count));
}

// FP64 Jacobi-CG on A x = r (x from 0) with the df64 SpMV on S.val2;
// r holds the initial residual; on return x holds the solution increment.
int pcg_df(nalu_ctx* ctx, const SellMatrix& S, double* x, double* r, double* z, double* q, const double* dinv,
           double rtol, double r0norm, int max_it, int check_every, int* iters_out, float* iter_ms) {
  const int64_t n = ctx->n_rows;
  const int64_t npad = S.nslices * kSlice;
  SolverWork& w = ctx->sw;
  if (w.partial.n < 2 * kCgBlocks) NALU_CUDA(ctx, w.partial.alloc(2 * kCgBlocks));
  if (w.p2.n < n) NALU_CUDA(ctx, w.p2.alloc(n));
  if (w.cscal.n < 8) NALU_CUDA(ctx, w.cscal.alloc(8));
  if (w.ccount.n < 1) NALU_CUDA(ctx, w.ccount.alloc(1));
  if (w.x2.n < n) NALU_CUDA(ctx, w.x2.alloc(n));
  if (w.r2.n < n) NALU_CUDA(ctx, w.r2.alloc(n));
  if (w.q2.n < n) NALU_CUDA(ctx, w.q2.alloc(n));
  double* part = w.partial.p;
  unsigned* cnt = w.ccount.p;
  double* cs = w.cscal.p;
  float2* p = w.p2.p;
  float2* x2 = w.x2.p;
  float2* r2 = w.r2.p;
  float2* q2 = w.q2.p;
  cudaStream_t st = ctx->stream;
  NALU_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(unsigned), st));
  NALU_CUDA(ctx, cudaMemsetAsync(cs, 0, sizeof(double) * 8, st));
  if (w.fdinv.n < n) NALU_CUDA(ctx, w.fdinv.alloc(n));
  int rc = sell_c16_ensure(ctx, const_cast<SellMatrix&>(S));
  if (rc) return rc;
  float* dinvf = w.fdinv.p;
  k_convert_f<<<kCgBlocks, kCgThreads, 0, st>>>(n, dinv, dinvf);
  k_cgd_init<<<kCgBlocks, kCgThreads, 0, st>>>(n, r, dinvf, r2, x2, part, cnt, cs);
  ctx->launches++;
  // one full wave per kernel: SMs x resident blocks (at most the partial-sum capacity)
  const unsigned g_pu = wave_grid(ctx, (const void*)k_cgd_pupdate, kCgThreads);
  const unsigned g_sp = wave_grid(ctx, (const void*)k_cgd_spmv, kCgThreads);
  const unsigned g_ax = wave_grid(ctx, (const void*)k_cgd_axpy, kCgThreads);
  auto iteration = [&](int first) {
    k_cgd_pupdate<<<g_pu, kCgThreads, 0, st>>>(n, r2, dinvf, p, cs, first);
    k_cgd_spmv<<<g_sp, kCgThreads, 0, st>>>(n, npad, S.ptr.p, S.len.p, S.col.p, S.col16.p, S.cbase.p, S.wide.p,
                                            S.val2.p, p, q2, part, cnt, cs);
    k_cgd_axpy<<<g_ax, kCgThreads, 0, st>>>(n, x2, p, r2, q2, dinvf, part, cnt, cs);
    ctx->launches += 3;
  };
  ctx->launches++;
  iteration(1);
  const int chunk = check_every > 0 ? check_every : 50;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "begin capture");
  for (int k = 0; k < chunk; ++k) iteration(0);
  ce = cudaStreamEndCapture(st, &graph);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "end capture");
  ce = cudaGraphInstantiate(&exec, graph, 0);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cuda_check(ctx, ce, "instantiate");
  }
  const double stop = rtol * r0norm;
  double rr = 0.0;
  int it = 1;
  bool bad = false, conv = false;
  cudaEvent_t t_ev[2] = {nullptr, nullptr};
  if (iter_ms) {
    cudaEventCreate(&t_ev[0]);
    cudaEventCreate(&t_ev[1]);
    cudaEventRecord(t_ev[0], st);
  }
  for (;;) {
    NALU_CUDA(ctx, cudaMemcpyAsync(&rr, cs + CS_RR, sizeof(double), cudaMemcpyDeviceToHost, st));
    NALU_CUDA(ctx, cudaStreamSynchronize(st));
    if (!std::isfinite(rr)) {
      bad = true;
      break;
    }
    if (std::sqrt(rr) <= stop) {
      conv = true;
      break;
    }
    if (it >= max_it) break;
    cudaGraphLaunch(exec, st);
    it += chunk;
  }
  if (iter_ms) {
    cudaEventRecord(t_ev[1], st);
    cudaEventSynchronize(t_ev[1]);
    cudaEventElapsedTime(iter_ms, t_ev[0], t_ev[1]);
    cudaEventDestroy(t_ev[0]);
    cudaEventDestroy(t_ev[1]);
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  k_cgd_finish<<<kCgBlocks, kCgThreads, 0, st>>>(n, x2, r2, x, r);
  ctx->launches++;
  NALU_CUDA(ctx, cudaGetLastError());
  *iters_out = it;
  if (bad) return set_error(ctx, NALU_ERR_NONFINITE, "CG breakdown (non-finite residual)");
  return conv ? NALU_OK : NALU_ERR_NOT_CONVERGED;
}

template int sell_build<double>(nalu_ctx*, SellMatrix&, const double**);
template int sell_build<float2>(nalu_ctx*, SellMatrix&, const float2**);
template int sell_build<float>(nalu_ctx*, SellMatrix&, const float**);
template int pcg_fast<double, double>(nalu_ctx*, const double*, const SellMatrix&, double*, double*, double*, double*,
                                      double*, double*, const double*, double, double, int, int, int*);
template int pcg_fast<float, float>(nalu_ctx*, const float*, const SellMatrix&, float*, float*, float*, float*,
                                    float*, float*, const float*, double, double, int, int, int*);

}  // namespace nalu_gb300
