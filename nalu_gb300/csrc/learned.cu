// learned.cu -- learned 27-point preconditioner for scalar (continuity /
// heat) systems, its training, and flexible CG with it.
//
// Model.  A per-node MLP f: R^108 -> R (108 -> 64 -> 64 -> 64 -> 1, GELU in
// its tanh form) reads four features per slot s of the node's 27-point
// neighbourhood (slot = 9(dz+1) + 3(dy+1) + (dx+1) of the element-local
// offset between the two nodes):
//   f[s]      residual r_j / rms_i        (rms_i: RMS of r over the 27 slots)
//   f[27+s]   a_ij / a_ii
//   f[54+s]   1 if the neighbour exists
//   f[81+s]   a_jj / a_ii
// and the correction is z_i = (r_i + rms_i f) / a_ii.  Used as it stands the
// map is non-linear in r, which stalls CG-type methods.  The solve therefore
// uses its linear form: evaluated on the 27 unit-impulse residuals (r = e_s,
// rms = 1/sqrt 27) it yields a stencil c_is = f(sqrt27 e_s, static_i)/sqrt27,
// and the preconditioner is the symmetric part of D^-1 (I + C) on the
// sparsity of A, made positive definite by a symmetric Gershgorin scaling of
// its off-diagonals.  Training fits exactly that linear form.
//
// Kernels.
//   slot map        one thread per (element, local node pair), atomicMin
//   stencil         one warp per node: FP32 static part of layer 1, then the
//                   27 impulse rows (padded to 32) through layers 2-3 with
//                   mma.sync m16n8k16 BF16 -> FP32, activations kept in
//                   registers between layers (the accumulator fragment of two
//                   n-tiles is the A fragment of the next layer's k-tile)
//   SELL values     one thread per row, symmetrised
//   FCG             four kernels per iteration, partial sums re-reduced in a
//                   fixed order by every block (deterministic)
//   training        by default the fused BF16 tensor-core step of train_tc.cu;
//                   here the FP32 path: tiled SGEMM with bias/GELU epilogues,
//                   reductions in fixed order, Adam; one step is one CUDA graph
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>
#include <utility>
#include <vector>

#include "df64.h"
#include "internal.h"
#include "learned_mlp.cuh"
#include "reduce.cuh"
#include "spmv_df.cuh"

namespace nalu_gb300 {


constexpr int kFcgBlocks = 1024;
constexpr int kFcgThreads = 256;
constexpr int kSlice = 32;

namespace {


// ---------------------------------------------------------------------------
// slot map
// ---------------------------------------------------------------------------
__constant__ int8_t c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                      {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

__global__ void k_fill_i32(int64_t n, int32_t* __restrict__ p, int32_t v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void k_nbr_elem(int64_t n_elems, const int32_t* __restrict__ conn, int32_t* __restrict__ nbr) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_elems * 64) return;
  const int64_t e = t >> 6;
  const int a = (int)((t >> 3) & 7), b = (int)(t & 7);
  const int32_t i = conn[8 * e + a], j = conn[8 * e + b];
  const int code = 9 * (c_corner[b][2] - c_corner[a][2] + 1) + 3 * (c_corner[b][1] - c_corner[a][1] + 1) +
                   (c_corner[b][0] - c_corner[a][0] + 1);
  atomicMin(&nbr[(int64_t)i * 27 + code], j);
}

__global__ void k_nbr_fix(int64_t n, int32_t* __restrict__ nbr) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && nbr[i] == INT_MAX) nbr[i] = -1;
}

// static features of the 27 slots of row i, by the whole warp: st[s],
// st[27+s], st[54+s] for s = lane < 27.  The row's entries are read once,
// one per lane (in chunks of 32), and broadcast by shuffles; the lane of
// slot s keeps the value whose column is its neighbour (columns are unique
// within a row).
__device__ __forceinline__ void slot_static_warp(int64_t i, int lane, const int32_t* __restrict__ nbr,
                                                 const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                                 const double* __restrict__ v, const double* __restrict__ dinv,
                                                 float* st) {
  const int32_t j = lane < 27 ? nbr[i * 27 + lane] : -1;
  const int64_t r0 = rp[i], len = rp[i + 1] - r0;
  double aij = 0.0;
  for (int64_t b = 0; b < len; b += 32) {
    const int64_t k = b + lane;
    const int32_t c = k < len ? ci[r0 + k] : -2;
    const double val = k < len ? v[r0 + k] : 0.0;
    const int m = (int)(len - b < 32 ? len - b : 32);
    for (int q = 0; q < m; ++q) {
      const int32_t cq = __shfl_sync(0xffffffffu, c, q);
      const double vq = __shfl_sync(0xffffffffu, val, q);
      if (cq == j) aij = vq;
    }
  }
  if (lane < 27) {
    float fa = 0.0f, fm = 0.0f, fd = 0.0f;
    if (j >= 0) {
      const double di = dinv[i];
      fa = (float)(aij * di);
      fm = 1.0f;
      fd = (float)(di / dinv[j]);
    }
    st[lane] = fa;
    st[27 + lane] = fm;
    st[54 + lane] = fd;
  }
}

// Harvest: one warp per sample row.  r is the residual-like vector (q0 = A p0),
// e the error-like vector (p0).
__global__ void k_harvest(int64_t count, const int64_t* __restrict__ rows, const double* __restrict__ r,
                          const double* __restrict__ e, const int32_t* __restrict__ nbr,
                          const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                          const double* __restrict__ v, const double* __restrict__ dinv,
                          const uint8_t* __restrict__ idmask, float* __restrict__ st, float* __restrict__ rf,
                          float* __restrict__ tg, uint8_t* __restrict__ valid) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= count) return;
  const int64_t i = rows[w];
  double rj = 0.0;
  if (lane < 27) {
    const int32_t j = nbr[i * 27 + lane];
    rj = j >= 0 ? r[j] : 0.0;
  }
  slot_static_warp(i, lane, nbr, rp, ci, v, dinv, st + w * 81);  // the whole warp (w is warp-uniform)
  double ss = rj * rj;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  const double sig = sqrt(ss / 27.0);
  const bool ok = sig > 0.0 && !idmask[i];
  if (lane < 27) rf[w * 27 + lane] = ok ? (float)(rj / sig) : 0.0f;
  if (lane == 0) {
    tg[w] = ok ? (float)(e[i] / (dinv[i] * sig)) : 0.0f;
    valid[w] = ok ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// stencil kernel (inference, BF16 tensor cores)
// ---------------------------------------------------------------------------
constexpr int kStThreads = 128;
constexpr int kStWarps = kStThreads / 32;
constexpr int kStWarpFloats = 148;  // 81 static features (+3 pad) + 64 layer-1 values
constexpr size_t kStSmem = sizeof(float) * (81 * 64 + 27 * 64 + 4 * 64 + 8) + sizeof(uint16_t) * 2 * 64 * kWStride +
                           sizeof(float) * kStWarps * kStWarpFloats;

__global__ void __launch_bounds__(kStThreads) k_mlp_stencil(int64_t row0, int64_t row1, const float* __restrict__ P,
                                                            const uint16_t* __restrict__ wbf,
                                                            const int32_t* __restrict__ nbr,
                                                            const int64_t* __restrict__ rp,
                                                            const int32_t* __restrict__ ci,
                                                            const double* __restrict__ v,
                                                            const double* __restrict__ dinv,
                                                            const uint8_t* __restrict__ idmask,
                                                            float* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* w1s = reinterpret_cast<float*>(smem);  // [81][64] static part of W1, k-major
  float* w1r = w1s + 81 * 64;                   // [27][64] sqrt27 * W1[:, s]
  float* bb = w1r + 27 * 64;                    // b1 | b2 | b3 | w4 | b4
  uint32_t* w2 = reinterpret_cast<uint32_t*>(bb + 4 * 64 + 8);
  uint32_t* w3 = w2 + 64 * (kWStride / 2);
  float* wsp = reinterpret_cast<float*>(w3 + 64 * (kWStride / 2));
  const int tid = threadIdx.x;
  for (int idx = tid; idx < 81 * 64; idx += kStThreads) {
    const int k = idx >> 6, o = idx & 63;
    w1s[idx] = P[OFF_W1 + o * 108 + 27 + k];
  }
  for (int idx = tid; idx < 27 * 64; idx += kStThreads) {
    const int s = idx >> 6, o = idx & 63;
    w1r[idx] = kSqrt27 * P[OFF_W1 + o * 108 + s];
  }
  for (int idx = tid; idx < 64; idx += kStThreads) {
    bb[idx] = P[OFF_B1 + idx];
    bb[64 + idx] = P[OFF_B2 + idx];
    bb[128 + idx] = P[OFF_B3 + idx];
    bb[192 + idx] = P[OFF_W4 + idx];
  }
  if (tid == 0) bb[256] = P[OFF_B4];
  const uint32_t* wsrc = reinterpret_cast<const uint32_t*>(wbf);
  for (int idx = tid; idx < 64 * kWStride; idx += kStThreads) w2[idx] = wsrc[idx];  // w2 and w3 are contiguous
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  float* st = wsp + warp * kStWarpFloats;
  float* hs = st + 84;
  const float b4 = bb[256];
  for (int64_t i = row0 + (int64_t)blockIdx.x * kStWarps + warp; i < row1; i += (int64_t)gridDim.x * kStWarps) {
    if (idmask[i]) {  // warp-uniform
      if (lane < 27) out[i * 27 + lane] = 0.0f;
      continue;
    }
    slot_static_warp(i, lane, nbr, rp, ci, v, dinv, st);
    __syncwarp();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int o = lane + 32 * h;
      float acc = bb[o];
      for (int k = 0; k < 81; ++k) acc = fmaf(w1s[k * 64 + o], st[k], acc);
      hs[o] = acc;
    }
    __syncwarp();
    // layer 1 for the 32 impulse rows (slots 0..26, rows 27..31 zero)
    uint32_t a[2][4][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const int s0 = 16 * mt + g, s1 = s0 + 8;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const int c0 = 16 * kk + 2 * t;
        float x[8];
        const int cols[4] = {c0, c0 + 1, c0 + 8, c0 + 9};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          x[q] = s0 < 27 ? gelu_fast(hs[cols[q]] + w1r[s0 * 64 + cols[q]]) : 0.0f;
          x[4 + q] = s1 < 27 ? gelu_fast(hs[cols[q]] + w1r[s1 * 64 + cols[q]]) : 0.0f;
        }
        a[mt][kk][0] = pack_bf16(x[0], x[1]);
        a[mt][kk][1] = pack_bf16(x[4], x[5]);
        a[mt][kk][2] = pack_bf16(x[2], x[3]);
        a[mt][kk][3] = pack_bf16(x[6], x[7]);
      }
    }
    float acc[2][8][4];
    mlp_layer(acc, a, w2, bb + 64, g, t);
    gelu_pack(acc, a);
    mlp_layer(acc, a, w3, bb + 128, g, t);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      float o0 = 0.0f, o1 = 0.0f;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float wa = bb[192 + 8 * j + 2 * t], wb = bb[192 + 8 * j + 2 * t + 1];
        o0 = fmaf(gelu_fast(acc[mt][j][0]), wa, fmaf(gelu_fast(acc[mt][j][1]), wb, o0));
        o1 = fmaf(gelu_fast(acc[mt][j][2]), wa, fmaf(gelu_fast(acc[mt][j][3]), wb, o1));
      }
      o0 += __shfl_xor_sync(0xffffffffu, o0, 1);
      o0 += __shfl_xor_sync(0xffffffffu, o0, 2);
      o1 += __shfl_xor_sync(0xffffffffu, o1, 1);
      o1 += __shfl_xor_sync(0xffffffffu, o1, 2);
      const int s0 = 16 * mt + g, s1 = s0 + 8;
      if (t == 0 && s0 < 27) out[i * 27 + s0] = st[27 + s0] * (o0 + b4) * (1.0f / kSqrt27);
      if (t == 1 && s1 < 27) out[i * 27 + s1] = st[27 + s1] * (o1 + b4) * (1.0f / kSqrt27);
    }
    __syncwarp();
  }
}

// FP32 master W2/W3 -> BF16 with the padded row stride
__global__ void k_prep_wbf(const float* __restrict__ P, uint16_t* __restrict__ wbf) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 2 * 64 * kWStride) return;
  const int layer = idx / (64 * kWStride), rem = idx % (64 * kWStride);
  const int o = rem / kWStride, k = rem % kWStride;
  const float w = k < 64 ? P[(layer ? OFF_W3 : OFF_W2) + o * 64 + k] : 0.0f;
  const __nv_bfloat16 h = __float2bfloat16_rn(w);
  wbf[idx] = *reinterpret_cast<const uint16_t*>(&h);
}

// Preconditioner values on A's SELL-32 pattern: the symmetric part of
// D^-1 (I + C).  Identity rows keep 1 on the diagonal and nothing else;
// columns of identity rows are dropped.
__global__ void k_precond_sell(int64_t row0, int64_t row1, const int64_t* __restrict__ rp, const int64_t* __restrict__ sptr,
                               const int32_t* __restrict__ slen, const int32_t* __restrict__ scol,
                               const int32_t* __restrict__ nbr, const float* __restrict__ c,
                               const double* __restrict__ dinv, const uint8_t* __restrict__ idmask,
                               float* __restrict__ w) {
  const int64_t row = row0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= row1) return;
  const int64_t s = row / kSlice;
  const int64_t base = sptr[s] + row % kSlice;
  const int len = slen[s];
  const int64_t real = rp[row + 1] - rp[row];
  const bool idr = idmask[row] != 0;
  const float di = (float)dinv[row];
  for (int k = 0; k < len; ++k) {
    const int32_t col = scol[base + (int64_t)k * kSlice];
    float val = 0.0f;
    if (k < real) {
      if (col == row) {
        val = idr ? 1.0f : di * (1.0f + c[row * 27 + 13]);
      } else if (!idr && !idmask[col]) {
        int sa = -1, sb = -1;
        for (int q = 0; q < 27 && sa < 0; ++q)
          if (nbr[row * 27 + q] == col) sa = q;
        if (sa >= 0 && nbr[(int64_t)col * 27 + 26 - sa] == row) {
          sb = 26 - sa;  // consistently oriented elements: the opposite slot
        } else {
          for (int q = 0; q < 27 && sb < 0; ++q)
            if (nbr[(int64_t)col * 27 + q] == row) sb = q;
        }
        if (sa >= 0 && sb >= 0) val = 0.5f * (c[row * 27 + sa] * di + c[(int64_t)col * 27 + sb] * (float)dinv[col]);
      }
    }
    w[base + (int64_t)k * kSlice] = val;
  }
}

// SPD safeguard (Gershgorin on D^1/2 M D^1/2): with d = a_ii, row i's
// scaled diagonal is d_i M_ii (floored at 1/4) and its scaled off-diagonal mass
// sum_j |M_ij| sqrt(d_i d_j).  s_i = min(1, theta diag / offdiag); every
// off-diagonal is then multiplied by min(s_i, s_j), which keeps M symmetric
// and makes every scaled row diagonally dominant, hence M positive definite.
// A row with a non-positive diagonal falls back to its Jacobi entry.
constexpr float kSpdTheta = 0.95f;
constexpr float kSpdDiagFloor = 0.25f;

__global__ void k_precond_rowscale(int64_t row0, int64_t row1, const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                                   const int32_t* __restrict__ scol, float* __restrict__ w,
                                   const double* __restrict__ dinv, float* __restrict__ srow) {
  const int64_t row = row0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= row1) return;
  const int64_t base = sptr[row / kSlice] + row % kSlice;
  const int len = slen[row / kSlice];
  const float di = (float)dinv[row];
  float diag = 0.0f, off = 0.0f;
  int64_t dpos = -1;
  for (int k = 0; k < len; ++k) {
    const int64_t e = base + (int64_t)k * kSlice;
    const int32_t col = scol[e];
    const float val = w[e];
    if (col == row) {
      if (dpos < 0) {  // padding repeats the diagonal index with value 0
        diag = val / di;
        dpos = e;
      }
    } else {
      off += fabsf(val) * rsqrtf(di * (float)dinv[col]);
    }
  }
  // the scaled diagonal (M_ii a_ii, 1 for Jacobi) is kept at or above
  // kSpdDiagFloor, so Gershgorin bounds the smallest eigenvalue of
  // D^1/2 M D^1/2 below by (1 - theta) kSpdDiagFloor
  float sc = 1.0f;
  if (!(diag > 0.0f)) {
    sc = 0.0f;
    if (dpos >= 0) w[dpos] = di;
  } else {
    if (diag < kSpdDiagFloor) {
      diag = kSpdDiagFloor;
      if (dpos >= 0) w[dpos] = kSpdDiagFloor * di;
    }
    if (off > kSpdTheta * diag) sc = kSpdTheta * diag / off;
  }
  srow[row] = sc;
}

__global__ void k_precond_apply_scale(int64_t row0, int64_t row1, const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                                      const int32_t* __restrict__ scol, float* __restrict__ w,
                                      const float* __restrict__ srow) {
  const int64_t row = row0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= row1) return;
  const int64_t base = sptr[row / kSlice] + row % kSlice;
  const int len = slen[row / kSlice];
  const float si = srow[row];
  for (int k = 0; k < len; ++k) {
    const int64_t e = base + (int64_t)k * kSlice;
    const int32_t col = scol[e];
    if (col != row) w[e] *= fminf(si, srow[col]);
  }
}

// ---------------------------------------------------------------------------
// flexible CG (Notay's FCG(1)) with the learned preconditioner
//   z = M r;  beta = -(z . q_old) / (p_old . q_old);  p = z + beta p
//   q = A p;  alpha = (p . r) / (p . q);  x += alpha p;  r -= alpha q
// ---------------------------------------------------------------------------
// FP32 -> BF16, round to nearest even (finite values; the SPD scaling keeps
// the stencil finite)
__global__ void k_to_bf16(int64_t n, const float* __restrict__ w, uint16_t* __restrict__ w16) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t u = __float_as_uint(w[i]);
  w16[i] = (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
}

__device__ __forceinline__ float bf16_f(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

// one word per SELL entry for the stencil apply: BF16 value (high half) and
// the 16-bit column offset (low half)
__global__ void k_pack_prec(int64_t n, const uint16_t* __restrict__ w16, const uint16_t* __restrict__ col16,
                            uint32_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = ((uint32_t)w16[i] << 16) | (uint32_t)col16[i];
}

// gathers in flight per group in the packed stencil apply
#ifndef NALU_PREC_GROUP
#define NALU_PREC_GROUP 8  // measured at 128^3: 8 -> 1012 ms, 16 -> 1036, 24 -> 1229
#endif

// z_row from the packed words (non-wide slices)
__device__ __forceinline__ float prec_row_packed(int64_t base, int len, const uint32_t* __restrict__ wp,
                                                 const int32_t* __restrict__ cbase,
                                                 const float2* __restrict__ r2) {
  constexpr int G = NALU_PREC_GROUP;
  float acc = 0.0f;
  for (int k = 0; k < len; k += G) {
    uint32_t v[G];
    int32_t c[G];
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const bool in = k + u < len;
      v[u] = in ? __ldg(wp + base + (int64_t)(k + u) * kSlice) : 0u;
      c[u] = in ? __ldg(cbase + k + u) + (int32_t)(v[u] & 0xffffu) : -1;
    }
    float b[G];
#pragma unroll
    for (int u = 0; u < G; ++u) b[u] = c[u] >= 0 ? __ldg(r2 + c[u]).x : 0.0f;
#pragma unroll
    for (int u = 0; u < G; ++u) acc = fmaf(__uint_as_float(v[u] & 0xffff0000u), b[u], acc);
  }
  return acc;
}

// z_row = sum_k w[base + 32 k] r[col_k] in FP32 (w as BF16), col_k from the 32-bit
// indices (WIDE) or the 16-bit offsets from the slice's entry bases
template <bool WIDE>
__device__ __forceinline__ float prec_row(int64_t base, int len, const SellMatrix::View& S,
                                          const int32_t* __restrict__ cbase, const uint16_t* __restrict__ w,
                                          const float2* __restrict__ r2) {
  float acc = 0.0f;
  for (int k = 0; k < len; k += 8) {  // loads of a group issued before the gathers
    int32_t c[8];
    float a[8], b[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool in = k + u < len;
      const int64_t e = base + (int64_t)(k + u) * kSlice;
      c[u] = in ? (WIDE ? __ldg(S.col + e) : __ldg(cbase + k + u) + (int32_t)__ldg(S.col16 + e)) : -1;
      a[u] = in ? bf16_f(__ldg(w + e)) : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) b[u] = c[u] >= 0 ? __ldg(r2 + c[u]).x : 0.0f;
#pragma unroll
    for (int u = 0; u < 8; ++u) acc = fmaf(a[u], b[u], acc);
  }
  return acc;
}

// z = M r (FP32 stencil values, FP32 residual); beta = -(z . q_old) / (p . q)_old by the last block
__global__ void __launch_bounds__(kFcgThreads) k_fcg_prec(int64_t n, int64_t npad, SellMatrix::View S,
                                                          const uint16_t* __restrict__ w,
                                                          const uint32_t* __restrict__ wp, const float2* __restrict__ r2,
                                                          const float2* __restrict__ q2, float* __restrict__ zf,
                                                          double* __restrict__ part, unsigned* __restrict__ cnt,
                                                          double* __restrict__ fs, int first) {
  __shared__ double sh[33];
  float dh = 0.0f, dl = 0.0f;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < npad;
       row += (int64_t)gridDim.x * blockDim.x) {
    if (row >= n) continue;
    const int64_t s = row / kSlice;
    const int len = __ldg(S.len + s);
    const int64_t b0 = __ldg(S.ptr + s);
    const int64_t base = b0 + (row % kSlice);
    const float acc = __ldg(S.wide + s) ? prec_row<true>(base, len, S, nullptr, w, r2)
                                        : prec_row_packed(base, len, wp, S.cbase + b0 / kSlice, r2);
    zf[row] = acc;
    acc_mul_df(dh, dl, make_float2(acc, 0.0f), q2[row]);
  }
  const double v[1] = {join_df(make_float2(dh, dl))};
  double t[1];
  if (red::grid_reduce<1>(v, part, kFcgBlocks, cnt, t, sh) && threadIdx.x == 0)
    fs[FS_BETA] = first ? 0.0 : -t[0] / fs[FS_PQ];
}

__global__ void __launch_bounds__(kFcgThreads) k_fcg_pupdate(int64_t n, const float* __restrict__ zf,
                                                             float2* __restrict__ p, const double* __restrict__ fs,
                                                             int first) {
  const float2 beta = split_df(first ? 0.0 : fs[FS_BETA]);  // FP32-pair update, no FP64 instruction
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 zi = make_float2(zf[i], 0.0f);
    p[i] = first ? zi : fma_df(beta, p[i], zi);
  }
}

// q = A p (df64); alpha = (p . r) / (p . q) by the last block, which also
// counts non-positive steps (the preconditioner is then not positive definite)
__global__ void __launch_bounds__(kFcgThreads) k_fcg_spmv(int64_t n, int64_t npad, SellMatrix::View S,
                                                          const float2* __restrict__ sval,
                                                          const float2* __restrict__ p, const float2* __restrict__ r2,
                                                          float2* __restrict__ q2, double* __restrict__ part,
                                                          unsigned* __restrict__ cnt, double* __restrict__ fs,
                                                          int* __restrict__ nonpos) {
  __shared__ double sh[33];
  float qh = 0.0f, ql = 0.0f, rh = 0.0f, rl = 0.0f;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < npad;
       row += (int64_t)gridDim.x * blockDim.x) {
    if (row >= n) continue;
    const int64_t s = row / kSlice;
    const int64_t b0 = __ldg(S.ptr + s);
    const int len = __ldg(S.len + s);
    const float2 qi = __ldg(S.wide + s)
                          ? sell_row_df2(b0 + (row % kSlice), len, S.col, sval, p)
                          : sell_row_df2_c16(b0 + (row % kSlice), len, S.col16, S.cbase + b0 / kSlice, sval, p);
    q2[row] = qi;
    const float2 pi = p[row];
    acc_mul_df(qh, ql, pi, qi);
    acc_mul_df(rh, rl, pi, r2[row]);
  }
  const double v[2] = {join_df(make_float2(qh, ql)), join_df(make_float2(rh, rl))};
  double t[2];
  if (red::grid_reduce<2>(v, part, kFcgBlocks, cnt, t, sh) && threadIdx.x == 0) {
    // fs[4] > 0: a stop threshold on r.r past which the iterate is frozen
    // (chunks of steps run between convergence checks); 0 in the learned FCG
    const bool frozen = fs[4] > 0.0 && fs[FS_RR] <= fs[4];
    const double alpha = frozen ? 0.0 : t[1] / t[0];
    if (!frozen) fs[FS_PQ] = t[0];
    fs[FS_ALPHA] = alpha;
    if (!frozen && !(alpha > 0.0)) *nonpos += 1;
  }
}

// x += alpha p; r -= alpha q; r.r -- all as FP32 pairs
__global__ void __launch_bounds__(kFcgThreads) k_fcg_axpy(int64_t n, float2* __restrict__ x2,
                                                          const float2* __restrict__ p, float2* __restrict__ r2,
                                                          const float2* __restrict__ q2, double* __restrict__ part,
                                                          unsigned* __restrict__ cnt, double* __restrict__ fs) {
  __shared__ double sh[33];
  const float2 alpha = split_df(fs[FS_ALPHA]);
  const float2 nalpha = make_float2(-alpha.x, -alpha.y);
  float rh = 0.0f, rl = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x2[i] = fma_df(alpha, p[i], x2[i]);
    const float2 ri = fma_df(nalpha, q2[i], r2[i]);
    r2[i] = ri;
    acc_sq_df(rh, rl, ri, 1.0f);
  }
  const double v[1] = {join_df(make_float2(rh, rl))};
  double t[1];
  if (red::grid_reduce<1>(v, part, kFcgBlocks, cnt, t, sh) && threadIdx.x == 0) fs[FS_RR] = t[0];
}

// FP64 <-> FP32-pair vectors at the ends of the solve
__global__ void k_fcg_split(int64_t n, const double* __restrict__ r, float2* __restrict__ r2,
                            float2* __restrict__ x2, float2* __restrict__ q2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    r2[i] = split_df(r[i]);
    x2[i] = make_float2(0.0f, 0.0f);
    q2[i] = make_float2(0.0f, 0.0f);
  }
}
__global__ void k_fcg_join(int64_t n, const float2* __restrict__ x2, const float2* __restrict__ r2,
                           double* __restrict__ x, double* __restrict__ r) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = join_df(x2[i]);
    r[i] = join_df(r2[i]);
  }
}

// flexible CG with an external preconditioner: beta = -(z . q_old) / (p . q)_old
// from the preconditioned residual z (FP32) by the last block
__global__ void __launch_bounds__(kFcgThreads) k_fcg_beta(int64_t n, const float* __restrict__ zf,
                                                          const float2* __restrict__ q2, double* __restrict__ part,
                                                          unsigned* __restrict__ cnt, double* __restrict__ fs,
                                                          int first) {
  __shared__ double sh[33];
  float dh = 0.0f, dl = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc_mul_df(dh, dl, make_float2(zf[i], 0.0f), q2[i]);
  const double v[1] = {join_df(make_float2(dh, dl))};
  double t[1];
  if (red::grid_reduce<1>(v, part, kFcgBlocks, cnt, t, sh) && threadIdx.x == 0)
    fs[FS_BETA] = first ? 0.0 : -t[0] / fs[FS_PQ];
}
// the high words of the FP32-pair residual: the preconditioner's FP32 input
__global__ void k_fcg_hi(int64_t n, const float2* __restrict__ r2, float* __restrict__ rf) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    rf[i] = r2[i].x;
}
// steps that moved the iterate: counted while r.r is above the stop threshold
// (fs[4] threshold, fs[5] count, fs[6] 1 while counting)
__global__ void k_fcg_count(double* __restrict__ fs) {
  if (fs[6] != 0.0) {
    fs[5] += 1.0;
    if (fs[FS_RR] <= fs[4]) fs[6] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// training (FP32)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float gelu_f(float x) {
  const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
  return 0.5f * x * (1.0f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad_f(float x) {
  const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
  const float th = tanhf(u);
  return 0.5f * (1.0f + th) + 0.5f * x * (1.0f - th * th) * 0.7978845608028654f * (1.0f + 3.0f * 0.044715f * x * x);
}

// C(m,n) = sum_k A(m,k) B(k,n) with strided operands and an epilogue:
//   0: C = acc + bias[n]         1: Z = acc + bias[n], C = gelu(Z)
//   2: C = acc * gelu'(GZ(m,n))  (GZ indexed like C)
struct Gemm {
  int M, N, K;
  const float* A;
  int64_t am, ak;
  const float* B;
  int64_t bk, bn;
  float* C;
  int64_t cm, cn;
  const float* bias;
  int epi;
  float* Z;
  const float* GZ;
};

__global__ void __launch_bounds__(256) k_sgemm(Gemm g) {
  __shared__ float As[16][17], Bs[16][17];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m = blockIdx.y * 16 + ty, n0 = blockIdx.x * 16, n = n0 + tx;
  float acc = 0.0f;
  for (int k0 = 0; k0 < g.K; k0 += 16) {
    const int ka = k0 + tx, kb = k0 + ty;
    As[ty][tx] = (m < g.M && ka < g.K) ? g.A[m * g.am + ka * g.ak] : 0.0f;
    Bs[ty][tx] = (kb < g.K && n < g.N) ? g.B[kb * g.bk + n * g.bn] : 0.0f;
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) acc = fmaf(As[ty][kk], Bs[kk][tx], acc);
    __syncthreads();
  }
  if (m >= g.M || n >= g.N) return;
  const int64_t ci = m * g.cm + n * g.cn;
  if (g.epi == 0) {
    g.C[ci] = acc + (g.bias ? g.bias[n] : 0.0f);
  } else if (g.epi == 1) {
    const float zz = acc + (g.bias ? g.bias[n] : 0.0f);
    g.Z[ci] = zz;
    g.C[ci] = gelu_f(zz);
  } else {
    g.C[ci] = acc * gelu_grad_f(g.GZ[ci]);
  }
}

// out[c] = sum_r X[r*ld + c] (one block per column, fixed-order tree), scaled
__global__ void k_colsum(int R, int ld, const float* __restrict__ X, float* __restrict__ out, float scale) {
  __shared__ float sh[256];
  const int c = blockIdx.x;
  float s = 0.0f;
  for (int r = threadIdx.x; r < R; r += blockDim.x) s += X[(int64_t)r * ld + c];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = scale * sh[0];
}

// batch gather from an index list: idx[step * B + b] (step from *stepp when given)
__global__ void k_tr_gather(int B, const int32_t* __restrict__ idx, const int* __restrict__ stepp, int step,
                            const float* __restrict__ st, const float* __restrict__ rf, const float* __restrict__ tg,
                            float* __restrict__ stb, float* __restrict__ rfb, float* __restrict__ tgb) {
  const int s = stepp ? *stepp : step;
  const int b = blockIdx.x;
  const int64_t src = idx[(int64_t)s * B + b];
  for (int k = threadIdx.x; k < 81; k += blockDim.x) stb[b * 81 + k] = st[src * 81 + k];
  for (int k = threadIdx.x; k < 27; k += blockDim.x) rfb[b * 27 + k] = rf[src * 27 + k];
  if (threadIdx.x == 0) tgb[b] = tg[src];
}

// Z1[(b,s), o] = HS[b][o] + sqrt27 W1[o][s];  H1 = gelu(Z1)
__global__ void k_tr_z1(int B, const float* __restrict__ HS, const float* __restrict__ P, float* __restrict__ Z1,
                        float* __restrict__ H1) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)B * 27 * 64) return;
  const int o = (int)(idx & 63);
  const int64_t r = idx >> 6;
  const int b = (int)(r / 27), s = (int)(r % 27);
  const float z = HS[b * 64 + o] + kSqrt27 * P[OFF_W1 + o * 108 + s];
  Z1[idx] = z;
  H1[idx] = gelu_f(z);
}

// output layer, stencil-form prediction, loss and dO; one thread per sample
__global__ void __launch_bounds__(1024) k_tr_loss(int B, int nvalid, const float* __restrict__ H3, const float* __restrict__ P,
                          const float* __restrict__ stb, const float* __restrict__ rfb, const float* __restrict__ tgb,
                          float* __restrict__ dO, float* __restrict__ loss_out, const int* __restrict__ stepp) {
  __shared__ float sh[1024];
  const int b = threadIdx.x;
  float l = 0.0f;
  if (b < B) {
    float pred = rfb[b * 27 + 13];
    for (int s = 0; s < 27; ++s) {
      const float* h = H3 + ((int64_t)b * 27 + s) * 64;
      float o = P[OFF_B4];
      for (int k = 0; k < 64; ++k) o = fmaf(P[OFF_W4 + k], h[k], o);
      pred = fmaf(stb[b * 81 + 27 + s] * o * (1.0f / kSqrt27), rfb[b * 27 + s], pred);
    }
    const bool ok = b < nvalid;
    const float diff = ok ? pred - tgb[b] : 0.0f;
    l = diff * diff;
    const float gs = 2.0f * diff / (float)nvalid;
    for (int s = 0; s < 27; ++s) dO[b * 27 + s] = gs * rfb[b * 27 + s] * stb[b * 81 + 27 + s] * (1.0f / kSqrt27);
  }
  sh[threadIdx.x] = l;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_out[stepp ? *stepp : 0] = sh[0] / (float)nvalid;
}

// dZ3 = dO w4^T * gelu'(Z3)
__global__ void k_tr_dz3(int64_t R, const float* __restrict__ dO, const float* __restrict__ P,
                         const float* __restrict__ Z3, float* __restrict__ dZ3) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= R * 64) return;
  dZ3[idx] = dO[idx >> 6] * P[OFF_W4 + (idx & 63)] * gelu_grad_f(Z3[idx]);
}

// dW1[o][s] = sqrt27 sum_b dZ1[(b,s),o]
__global__ void k_tr_w1r(int B, const float* __restrict__ dZ1, float* __restrict__ G) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 27 * 64) return;
  const int s = idx / 64, o = idx % 64;
  float acc = 0.0f;
  for (int b = 0; b < B; ++b) acc += dZ1[((int64_t)b * 27 + s) * 64 + o];
  G[OFF_W1 + o * 108 + s] = kSqrt27 * acc;
}

// dHS[b][o] = sum_s dZ1[(b,s),o]
__global__ void k_tr_dhs(int B, const float* __restrict__ dZ1, float* __restrict__ dHS) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * 64) return;
  const int b = idx / 64, o = idx % 64;
  float acc = 0.0f;
  for (int s = 0; s < 27; ++s) acc += dZ1[((int64_t)b * 27 + s) * 64 + o];
  dHS[idx] = acc;
}

__global__ void k_adam(const float* __restrict__ G, float* __restrict__ P, float* __restrict__ m,
                       float* __restrict__ v, const int* __restrict__ stepp, float lr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kNP) return;
  const float t = (float)(*stepp + 1);
  const float g = G[i];
  const float mi = 0.9f * m[i] + 0.1f * g;
  const float vi = 0.999f * v[i] + 0.001f * g * g;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.0f - powf(0.9f, t));
  const float vh = vi / (1.0f - powf(0.999f, t));
  P[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
}

__global__ void k_step_inc(int* stepp) { *stepp += 1; }

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

int ensure_learned_buffers(nalu_ctx* ctx) {
  LearnedState& L = ctx->learned;
  if (L.params.n < kNP) NALU_CUDA(ctx, L.params.alloc(kNP));
  if (L.grad.n < kNP) NALU_CUDA(ctx, L.grad.alloc(kNP));
  if (L.adam_m.n < kNP) NALU_CUDA(ctx, L.adam_m.alloc(kNP));
  if (L.adam_v.n < kNP) NALU_CUDA(ctx, L.adam_v.alloc(kNP));
  if (L.wbf.n < 2 * 64 * kWStride) NALU_CUDA(ctx, L.wbf.alloc(2 * 64 * kWStride));
  return NALU_OK;
}

int check_scalar(nalu_ctx* ctx) {
  if (ctx->num_dof != 1) return set_error(ctx, NALU_ERR_STATE, "the learned preconditioner needs a scalar system");
  return NALU_OK;
}

int build_slot_map(nalu_ctx* ctx) {
  LearnedState& L = ctx->learned;
  const int64_t n = ctx->n_nodes;
  if (L.nbr_nodes == n && L.nbr.n >= n * 27) return NALU_OK;
  if (L.nbr.n < n * 27) NALU_CUDA(ctx, L.nbr.alloc(n * 27));
  const int64_t tot = n * 27;
  k_fill_i32<<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(tot, L.nbr.p, INT_MAX);
  const int64_t pairs = ctx->n_elems * 64;
  k_nbr_elem<<<(unsigned)((pairs + 255) / 256), 256, 0, ctx->stream>>>(ctx->n_elems, ctx->d_conn.p, L.nbr.p);
  k_nbr_fix<<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(tot, L.nbr.p);
  ctx->launches += 3;
  L.nbr_nodes = n;
  return cuda_check(ctx, cudaGetLastError(), "slot map");
}

// the stencil of rows [row0, row1) (all rows by default)
int launch_stencil(nalu_ctx* ctx, int64_t row0 = 0, int64_t row1 = -1) {
  LearnedState& L = ctx->learned;
  const int64_t n = ctx->n_rows;
  if (row1 < 0) row1 = n;
  if (L.stencil.n < n * 27) NALU_CUDA(ctx, L.stencil.alloc(n * 27));
  k_prep_wbf<<<(2 * 64 * kWStride + 255) / 256, 256, 0, ctx->stream>>>(L.params.p, L.wbf.p);
  NALU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_stencil, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStSmem));
  int per_sm = 0;
  NALU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mlp_stencil, kStThreads, kStSmem));
  const int64_t need = (row1 - row0 + kStWarps - 1) / kStWarps;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)std::max(1, per_sm) * ctx->sm_count));
  k_mlp_stencil<<<grid, kStThreads, kStSmem, ctx->stream>>>(row0, row1, L.params.p, L.wbf.p, L.nbr.p, ctx->d_rowptr.p,
                                                           ctx->d_colind.p, ctx->d_values.p, ctx->sw.dinv.p,
                                                           ctx->d_bcmask.p, L.stencil.p);
  ctx->launches += 2;
  return cuda_check(ctx, cudaGetLastError(), "learned stencil");
}

void gemm(nalu_ctx* ctx, const Gemm& g) {
  dim3 grid((g.N + 15) / 16, (g.M + 15) / 16);
  k_sgemm<<<grid, 256, 0, ctx->stream>>>(g);
  ctx->launches++;
}
Gemm mk(int M, int N, int K, const float* A, int64_t am, int64_t ak, const float* B, int64_t bk, int64_t bn, float* C,
        int64_t cm, int64_t cn, const float* bias = nullptr, int epi = 0, float* Z = nullptr,
        const float* GZ = nullptr) {
  return Gemm{M, N, K, A, am, ak, B, bk, bn, C, cm, cn, bias, epi, Z, GZ};
}

// Training workspace for batches of B samples
struct TrainWork {
  int B = 0;
  DBuf<float> stb, rfb, tgb, hs, z1, h1, z2, h2, z3, h3, dO, d3, d2, d1, dhs, loss;
  int alloc(nalu_ctx* ctx, int b, int64_t loss_slots) {
    B = b;
    const int64_t R = (int64_t)b * 27;
    for (auto& pr : {std::make_pair(&stb, (int64_t)b * 81), std::make_pair(&rfb, R), std::make_pair(&tgb, (int64_t)b),
                     std::make_pair(&hs, (int64_t)b * 64), std::make_pair(&z1, R * 64), std::make_pair(&h1, R * 64),
                     std::make_pair(&z2, R * 64), std::make_pair(&h2, R * 64), std::make_pair(&z3, R * 64),
                     std::make_pair(&h3, R * 64), std::make_pair(&dO, R), std::make_pair(&d3, R * 64),
                     std::make_pair(&d2, R * 64), std::make_pair(&d1, R * 64), std::make_pair(&dhs, (int64_t)b * 64),
                     std::make_pair(&loss, loss_slots)})
      NALU_CUDA(ctx, pr.first->alloc(pr.second));
    return NALU_OK;
  }
};

// forward pass of one gathered batch; loss of the batch into loss[*stepp or 0]; dO
void forward(nalu_ctx* ctx, TrainWork& w, const float* P, int nvalid, const int* stepp) {
  const int B = w.B;
  const int R = B * 27;
  gemm(ctx, mk(B, 64, 81, w.stb.p, 81, 1, P + OFF_W1 + 27, 1, 108, w.hs.p, 64, 1, P + OFF_B1));
  k_tr_z1<<<(unsigned)(((int64_t)R * 64 + 255) / 256), 256, 0, ctx->stream>>>(B, w.hs.p, P, w.z1.p, w.h1.p);
  gemm(ctx, mk(R, 64, 64, w.h1.p, 64, 1, P + OFF_W2, 1, 64, w.h2.p, 64, 1, P + OFF_B2, 1, w.z2.p));
  gemm(ctx, mk(R, 64, 64, w.h2.p, 64, 1, P + OFF_W3, 1, 64, w.h3.p, 64, 1, P + OFF_B3, 1, w.z3.p));
  k_tr_loss<<<1, 1024, 0, ctx->stream>>>(B, nvalid, w.h3.p, P, w.stb.p, w.rfb.p, w.tgb.p, w.dO.p, w.loss.p, stepp);
  ctx->launches += 2;
}

// gradient of the batch loss into G (overwrites)
void backward(nalu_ctx* ctx, TrainWork& w, const float* P, float* G) {
  const int B = w.B;
  const int R = B * 27;
  // output layer
  gemm(ctx, mk(1, 64, R, w.dO.p, 0, 1, w.h3.p, 64, 1, G + OFF_W4, 0, 1));
  k_colsum<<<1, 256, 0, ctx->stream>>>(R, 1, w.dO.p, G + OFF_B4, 1.0f);
  k_tr_dz3<<<(unsigned)(((int64_t)R * 64 + 255) / 256), 256, 0, ctx->stream>>>(R, w.dO.p, P, w.z3.p, w.d3.p);
  // layer 3
  gemm(ctx, mk(64, 64, R, w.d3.p, 1, 64, w.h2.p, 64, 1, G + OFF_W3, 64, 1));
  k_colsum<<<64, 256, 0, ctx->stream>>>(R, 64, w.d3.p, G + OFF_B3, 1.0f);
  gemm(ctx, mk(R, 64, 64, w.d3.p, 64, 1, P + OFF_W3, 64, 1, w.d2.p, 64, 1, nullptr, 2, nullptr, w.z2.p));
  // layer 2
  gemm(ctx, mk(64, 64, R, w.d2.p, 1, 64, w.h1.p, 64, 1, G + OFF_W2, 64, 1));
  k_colsum<<<64, 256, 0, ctx->stream>>>(R, 64, w.d2.p, G + OFF_B2, 1.0f);
  gemm(ctx, mk(R, 64, 64, w.d2.p, 64, 1, P + OFF_W2, 64, 1, w.d1.p, 64, 1, nullptr, 2, nullptr, w.z1.p));
  // layer 1: impulse columns, then the static part through HS
  k_tr_w1r<<<(27 * 64 + 255) / 256, 256, 0, ctx->stream>>>(B, w.d1.p, G);
  k_tr_dhs<<<(B * 64 + 255) / 256, 256, 0, ctx->stream>>>(B, w.d1.p, w.dhs.p);
  gemm(ctx, mk(64, 81, B, w.dhs.p, 1, 64, w.stb.p, 81, 1, G + OFF_W1 + 27, 108, 1));
  k_colsum<<<64, 256, 0, ctx->stream>>>(B, 64, w.dhs.p, G + OFF_B1, 1.0f);
  ctx->launches += 7;
}

}  // namespace

int learned_prepare_rows(nalu_ctx* ctx, int64_t row0, int64_t row1) {
  int rc = check_scalar(ctx);
  if (rc) return rc;
  LearnedState& L = ctx->learned;
  if (!L.has_weights) return set_error(ctx, NALU_ERR_STATE, "learned preconditioner has no weights");
  const int64_t n = ctx->n_rows;
  if (row0 < 0 || row1 > n || row0 >= row1) return set_error(ctx, NALU_ERR_ARG, "learned set-up: bad row range");
  if ((rc = build_slot_map(ctx))) return rc;
  if ((rc = launch_stencil(ctx, row0, row1))) return rc;
  const SellMatrix& S = ctx->sw.sell;
  if (L.wsell.n < S.stored) NALU_CUDA(ctx, L.wsell.alloc(S.stored));
  if (L.srow.n < n) NALU_CUDA(ctx, L.srow.alloc(n));
  const unsigned g = (unsigned)((row1 - row0 + 255) / 256);
  k_precond_sell<<<g, 256, 0, ctx->stream>>>(row0, row1, ctx->d_rowptr.p, S.ptr.p, S.len.p, S.col.p, L.nbr.p,
                                             L.stencil.p, ctx->sw.dinv.p, ctx->d_bcmask.p, L.wsell.p);
  k_precond_rowscale<<<g, 256, 0, ctx->stream>>>(row0, row1, S.ptr.p, S.len.p, S.col.p, L.wsell.p, ctx->sw.dinv.p,
                                                 L.srow.p);
  k_precond_apply_scale<<<g, 256, 0, ctx->stream>>>(row0, row1, S.ptr.p, S.len.p, S.col.p, L.wsell.p, L.srow.p);
  ctx->launches += 3;
  return cuda_check(ctx, cudaGetLastError(), "learned preconditioner values");
}

int learned_prepare(nalu_ctx* ctx) {
  const int64_t n = ctx->n_rows;
  int rc = learned_prepare_rows(ctx, 0, n);
  if (rc) return rc;
  LearnedState& L = ctx->learned;
  const SellMatrix& S = ctx->sw.sell;
  if (L.wsell16.n < S.stored) NALU_CUDA(ctx, L.wsell16.alloc(S.stored));
  k_to_bf16<<<(unsigned)((S.stored + 255) / 256), 256, 0, ctx->stream>>>(S.stored, L.wsell.p, L.wsell16.p);
  ctx->launches++;
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return cuda_check(ctx, cudaGetLastError(), "learned preconditioner values");
}

int fcg_learned(nalu_ctx* ctx, double* x, double* r, double rtol, double r0norm, int max_it, int check_every,
                int stall_window, int* iters_out, int* stalled, float* iter_ms) {
  const int64_t n = ctx->n_rows;
  SolverWork& s = ctx->sw;
  const SellMatrix& S = s.sell;
  const int64_t npad = S.nslices * kSlice;
  *stalled = 0;
  if (s.partial.n < 2 * kFcgBlocks) NALU_CUDA(ctx, s.partial.alloc(2 * kFcgBlocks));
  if (s.p2.n < n) NALU_CUDA(ctx, s.p2.alloc(n));
  if (s.cscal.n < 8) NALU_CUDA(ctx, s.cscal.alloc(8));
  if (s.ccount.n < 1) NALU_CUDA(ctx, s.ccount.alloc(1));
  if (s.x2.n < n) NALU_CUDA(ctx, s.x2.alloc(n));
  if (s.r2.n < n) NALU_CUDA(ctx, s.r2.alloc(n));
  if (s.q2.n < n) NALU_CUDA(ctx, s.q2.alloc(n));
  if (s.zf.n < n) NALU_CUDA(ctx, s.zf.alloc(n));
  int rc = sell_c16_ensure(ctx, s.sell);
  if (rc) return rc;
  const SellMatrix::View SV = S.view();
  double* part = s.partial.p;
  unsigned* cnt = s.ccount.p;
  double* fs = s.cscal.p;
  float* zf = s.zf.p;
  float2 *p = s.p2.p, *x2 = s.x2.p, *r2 = s.r2.p, *q2 = s.q2.p;
  DBuf<int> nonpos;
  NALU_CUDA(ctx, nonpos.alloc(1));
  cudaStream_t st = ctx->stream;
  NALU_CUDA(ctx, cudaMemsetAsync(nonpos.p, 0, sizeof(int), st));
  NALU_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(unsigned), st));
  NALU_CUDA(ctx, cudaMemsetAsync(fs, 0, sizeof(double) * 8, st));
  k_fcg_split<<<kFcgBlocks, kFcgThreads, 0, st>>>(n, r, r2, x2, q2);
  ctx->launches++;
  const uint16_t* w = ctx->learned.wsell16.p;
  LearnedState& L = ctx->learned;
  if (L.wpack.n < S.stored) NALU_CUDA(ctx, L.wpack.alloc(S.stored));
  k_pack_prec<<<(unsigned)((S.stored + 255) / 256), 256, 0, st>>>(S.stored, L.wsell16.p, S.col16.p, L.wpack.p);
  ctx->launches++;
  const uint32_t* wp = L.wpack.p;
  const unsigned g_pc = wave_grid(ctx, (const void*)k_fcg_prec, kFcgThreads);
  const unsigned g_pu = wave_grid(ctx, (const void*)k_fcg_pupdate, kFcgThreads);
  const unsigned g_sp = wave_grid(ctx, (const void*)k_fcg_spmv, kFcgThreads);
  const unsigned g_ax = wave_grid(ctx, (const void*)k_fcg_axpy, kFcgThreads);
  auto iteration = [&](int first) {
    k_fcg_prec<<<g_pc, kFcgThreads, 0, st>>>(n, npad, SV, w, wp, r2, q2, zf, part, cnt, fs, first);
    k_fcg_pupdate<<<g_pu, kFcgThreads, 0, st>>>(n, zf, p, fs, first);
    k_fcg_spmv<<<g_sp, kFcgThreads, 0, st>>>(n, npad, SV, S.val2.p, p, r2, q2, part, cnt, fs, nonpos.p);
    k_fcg_axpy<<<g_ax, kFcgThreads, 0, st>>>(n, x2, p, r2, q2, part, cnt, fs);
    ctx->launches += 4;
  };
  iteration(1);
  const int chunk = std::max(1, check_every > 0 ? std::min(check_every, 10) : 10);
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
  double last = INFINITY, best = INFINITY;
  int it = 1, best_it = 0, hnonpos = 0;
  bool bad = false, conv = false;
  cudaEvent_t t_ev[2] = {nullptr, nullptr};
  if (iter_ms) {
    cudaEventCreate(&t_ev[0]);
    cudaEventCreate(&t_ev[1]);
    cudaEventRecord(t_ev[0], st);
  }
  for (;;) {
    double rr = 0.0;
    cudaMemcpyAsync(&rr, fs + FS_RR, sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&hnonpos, nonpos.p, sizeof(int), cudaMemcpyDeviceToHost, st);
    const double res = cudaStreamSynchronize(st) == cudaSuccess ? std::sqrt(rr) : (double)NAN;
    last = res;
    if (!std::isfinite(res) || hnonpos > 0) {
      bad = true;  // breakdown: non-finite values or an indefinite preconditioner
      break;
    }
    if (res <= stop) {
      conv = true;
      break;
    }
    if (res < 0.999 * best) {
      best = res;
      best_it = it;
    } else if (it - best_it > std::max(stall_window, 10 * best_it)) {
      // CG residual norms rise and fall in humps whose length grows with the
      // iteration count (measured beyond the age of the current minimum), so
      // the window is at least ten times the iterations the current minimum
      // took to reach
      *stalled = 1;
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
  k_fcg_join<<<kFcgBlocks, kFcgThreads, 0, st>>>(n, x2, r2, x, r);
  ctx->launches++;
  NALU_CUDA(ctx, cudaGetLastError());
  *iters_out = it;
  if (bad) *stalled = 1;  // a breakdown is handed to the fallback like a stall
  if (*stalled && !(last < r0norm)) {
    // no progress at all: hand the fallback a zero increment, not a diverged one
    NALU_CUDA(ctx, cudaMemsetAsync(x, 0, sizeof(double) * n, st));
  }
  if (bad) return NALU_ERR_NOT_CONVERGED;
  return conv ? NALU_OK : NALU_ERR_NOT_CONVERGED;
}

// Flexible CG (FCG(1)) on FP32-pair vectors with the df64 SELL-32 SpMV, as the
// learned FCG, preconditioned by prec(rf, zf): kernels on the context stream
// that compute zf ~ A^-1 rf from the FP32 residual rf (captured into the
// iteration's CUDA graph).  x (FP64) receives the correction from zero, r (FP64)
// the updated residual; the stop rule is ||r|| <= rtol r0norm, checked every
// check_every (at most 10) steps; *iters_out counts the steps taken before it
// was met, exactly (counted on the device).
int fcg_df_external(nalu_ctx* ctx, double* x, double* r, double rtol, double r0norm, int max_it, int check_every,
                    const std::function<void(const float*, float*)>& prec, int* iters_out) {
  const int64_t n = ctx->n_rows;
  SolverWork& s = ctx->sw;
  const SellMatrix& S = s.sell;
  const int64_t npad = S.nslices * kSlice;
  *iters_out = 0;
  if (s.partial.n < 2 * kFcgBlocks) NALU_CUDA(ctx, s.partial.alloc(2 * kFcgBlocks));
  if (s.p2.n < n) NALU_CUDA(ctx, s.p2.alloc(n));
  if (s.cscal.n < 8) NALU_CUDA(ctx, s.cscal.alloc(8));
  if (s.ccount.n < 1) NALU_CUDA(ctx, s.ccount.alloc(1));
  if (s.x2.n < n) NALU_CUDA(ctx, s.x2.alloc(n));
  if (s.r2.n < n) NALU_CUDA(ctx, s.r2.alloc(n));
  if (s.q2.n < n) NALU_CUDA(ctx, s.q2.alloc(n));
  if (s.zf.n < n) NALU_CUDA(ctx, s.zf.alloc(n));
  if (s.fr.n < n) NALU_CUDA(ctx, s.fr.alloc(n));
  int rc = sell_c16_ensure(ctx, s.sell);
  if (rc) return rc;
  const SellMatrix::View SV = S.view();
  double* part = s.partial.p;
  unsigned* cnt = s.ccount.p;
  double* fs = s.cscal.p;
  float* zf = s.zf.p;
  float* rf = s.fr.p;
  float2 *p = s.p2.p, *x2 = s.x2.p, *r2 = s.r2.p, *q2 = s.q2.p;
  DBuf<int> nonpos;
  NALU_CUDA(ctx, nonpos.alloc(1));
  cudaStream_t st = ctx->stream;
  const double stop = rtol * r0norm;
  {
    const double init[8] = {0.0, 0.0, 0.0, r0norm * r0norm, stop * stop, 0.0, 1.0, 0.0};
    NALU_CUDA(ctx, cudaMemsetAsync(nonpos.p, 0, sizeof(int), st));
    NALU_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(unsigned), st));
    NALU_CUDA(ctx, cudaMemcpyAsync(fs, init, sizeof(init), cudaMemcpyHostToDevice, st));
    NALU_CUDA(ctx, cudaStreamSynchronize(st));
  }
  k_fcg_split<<<kFcgBlocks, kFcgThreads, 0, st>>>(n, r, r2, x2, q2);
  ctx->launches++;
  const unsigned g_b = wave_grid(ctx, (const void*)k_fcg_beta, kFcgThreads);
  const unsigned g_pu = wave_grid(ctx, (const void*)k_fcg_pupdate, kFcgThreads);
  const unsigned g_sp = wave_grid(ctx, (const void*)k_fcg_spmv, kFcgThreads);
  const unsigned g_ax = wave_grid(ctx, (const void*)k_fcg_axpy, kFcgThreads);
  auto iteration = [&](int first) {
    k_fcg_hi<<<kFcgBlocks, kFcgThreads, 0, st>>>(n, r2, rf);
    prec(rf, zf);
    k_fcg_beta<<<g_b, kFcgThreads, 0, st>>>(n, zf, q2, part, cnt, fs, first);
    k_fcg_pupdate<<<g_pu, kFcgThreads, 0, st>>>(n, zf, p, fs, first);
    k_fcg_spmv<<<g_sp, kFcgThreads, 0, st>>>(n, npad, SV, S.val2.p, p, r2, q2, part, cnt, fs, nonpos.p);
    k_fcg_axpy<<<g_ax, kFcgThreads, 0, st>>>(n, x2, p, r2, q2, part, cnt, fs);
    k_fcg_count<<<1, 1, 0, st>>>(fs);
    ctx->launches += 6;
  };
  iteration(1);
  const int chunk = std::max(1, check_every > 0 ? std::min(check_every, 10) : 10);
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
  int it = 1, hnonpos = 0;
  bool conv = false;
  for (;;) {
    double h[8] = {};
    cudaMemcpyAsync(h, fs, sizeof(h), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&hnonpos, nonpos.p, sizeof(int), cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      rc = cuda_check(ctx, e, "flexible CG");
      break;
    }
    const double res = std::sqrt(h[FS_RR]);
    *iters_out = (int)h[5];
    if (std::isfinite(res) && res <= stop) {
      conv = true;
      break;
    }
    if (!std::isfinite(res) || hnonpos > 0) {
      rc = set_error(ctx, NALU_ERR_NONFINITE, "flexible CG breakdown (non-finite or non-positive step)");
      break;
    }
    if (it >= max_it) break;
    cudaGraphLaunch(exec, st);
    it += chunk;
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  k_fcg_join<<<kFcgBlocks, kFcgThreads, 0, st>>>(n, x2, r2, x, r);
  ctx->launches++;
  NALU_CUDA(ctx, cudaGetLastError());
  if (rc) return rc;
  return conv ? NALU_OK : NALU_ERR_NOT_CONVERGED;
}

}  // namespace nalu_gb300

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace nalu_gb300;

extern "C" {

int nalu_learned_init(nalu_ctx* ctx, uint64_t seed) {
  if (!ctx) return NALU_ERR_ARG;
  cudaSetDevice(ctx->device);
  int rc = ensure_learned_buffers(ctx);
  if (rc) return rc;
  std::vector<float> P(kNP, 0.0f);
  uint64_t s = seed;
  auto fill = [&](int off, int count, int fan_in) {
    const double b = 1.0 / std::sqrt((double)fan_in);
    for (int i = 0; i < count; ++i) P[off + i] = (float)((2.0 * uniform01(s) - 1.0) * b);
  };
  fill(OFF_W1, 64 * 108, 108);
  fill(OFF_B1, 64, 108);
  fill(OFF_W2, 64 * 64, 64);
  fill(OFF_B2, 64, 64);
  fill(OFF_W3, 64 * 64, 64);
  fill(OFF_B3, 64, 64);  // w4 and b4 stay 0: the untrained preconditioner is Jacobi
  return nalu_learned_set_weights(ctx, P.data(), kNP);
}

int nalu_learned_set_weights(nalu_ctx* ctx, const float* params, int64_t n) {
  if (!ctx || !params) return NALU_ERR_ARG;
  if (n != kNP) return set_error(ctx, NALU_ERR_ARG, "expected NALU_LEARNED_PARAMS parameters");
  cudaSetDevice(ctx->device);
  int rc = ensure_learned_buffers(ctx);
  if (rc) return rc;
  NALU_CUDA(ctx, cudaMemcpyAsync(ctx->learned.params.p, params, sizeof(float) * kNP, cudaMemcpyHostToDevice,
                                 ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->learned.has_weights = true;
  return NALU_OK;
}

int nalu_learned_get_weights(nalu_ctx* ctx, float* params, int64_t n) {
  if (!ctx || !params) return NALU_ERR_ARG;
  if (n != kNP) return set_error(ctx, NALU_ERR_ARG, "expected NALU_LEARNED_PARAMS parameters");
  if (!ctx->learned.has_weights) return set_error(ctx, NALU_ERR_STATE, "no weights");
  cudaSetDevice(ctx->device);
  NALU_CUDA(ctx, cudaMemcpyAsync(params, ctx->learned.params.p, sizeof(float) * kNP, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

int nalu_learned_harvest(nalu_ctx* ctx, int n_rhs, uint64_t seed, int64_t n_samples, float* static_feats,
                         float* resid_feats, float* targets, int64_t* rows_out, int64_t* n_out) {
  if (!ctx || n_rhs < 1 || n_samples < 1 || !static_feats || !resid_feats || !targets || !n_out)
    return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no linear system");
  int rc = check_scalar(ctx);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  const int64_t n = ctx->n_rows;
  if ((rc = compute_dinv(ctx)) || (rc = build_slot_map(ctx))) return rc;
  DBuf<double> b, p0, q0;
  DBuf<int64_t> rows;
  DBuf<float> st, rf, tg;
  DBuf<uint8_t> valid;
  const int64_t per = (n_samples + n_rhs - 1) / n_rhs;
  NALU_CUDA(ctx, b.alloc(n));
  NALU_CUDA(ctx, p0.alloc(n));
  NALU_CUDA(ctx, q0.alloc(n));
  NALU_CUDA(ctx, rows.alloc(per));
  NALU_CUDA(ctx, st.alloc(per * 81));
  NALU_CUDA(ctx, rf.alloc(per * 27));
  NALU_CUDA(ctx, tg.alloc(per));
  NALU_CUDA(ctx, valid.alloc(per));
  uint64_t s = seed;
  std::vector<double> hb(n), hd(n);
  std::vector<int64_t> hrows(per);
  std::vector<uint8_t> hvalid(per);
  NALU_CUDA(ctx, cudaMemcpyAsync(hd.data(), ctx->sw.dinv.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  int64_t got = 0;
  for (int k = 0; k < n_rhs && got < n_samples; ++k) {
    // b ~ N(0,1) (Box-Muller on splitmix64 uniforms); p0 = D^-1 b; q0 = A p0
    for (int64_t i = 0; i < n; i += 2) {
      const double u1 = std::max(uniform01(s), 1e-300), u2 = uniform01(s);
      const double rad = std::sqrt(-2.0 * std::log(u1));
      hb[i] = rad * std::cos(6.283185307179586 * u2);
      if (i + 1 < n) hb[i + 1] = rad * std::sin(6.283185307179586 * u2);
    }
    for (int64_t i = 0; i < n; ++i) hb[i] *= hd[i];
    NALU_CUDA(ctx, cudaMemcpyAsync(p0.p, hb.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = spmv_fp64(ctx, p0.p, q0.p))) return rc;
    const int64_t want = std::min(per, n_samples - got);
    for (int64_t j = 0; j < want; ++j) hrows[j] = (int64_t)(uniform01(s) * (double)n) % n;
    NALU_CUDA(ctx, cudaMemcpyAsync(rows.p, hrows.data(), sizeof(int64_t) * want, cudaMemcpyHostToDevice, ctx->stream));
    k_harvest<<<(unsigned)((want * 32 + 255) / 256), 256, 0, ctx->stream>>>(
        want, rows.p, q0.p, p0.p, ctx->learned.nbr.p, ctx->d_rowptr.p, ctx->d_colind.p, ctx->d_values.p,
        ctx->sw.dinv.p, ctx->d_bcmask.p, st.p, rf.p, tg.p, valid.p);
    ctx->launches++;
    std::vector<float> hst(want * 81), hrf(want * 27), htg(want);
    NALU_CUDA(ctx, cudaMemcpyAsync(hst.data(), st.p, sizeof(float) * want * 81, cudaMemcpyDeviceToHost, ctx->stream));
    NALU_CUDA(ctx, cudaMemcpyAsync(hrf.data(), rf.p, sizeof(float) * want * 27, cudaMemcpyDeviceToHost, ctx->stream));
    NALU_CUDA(ctx, cudaMemcpyAsync(htg.data(), tg.p, sizeof(float) * want, cudaMemcpyDeviceToHost, ctx->stream));
    NALU_CUDA(ctx, cudaMemcpyAsync(hvalid.data(), valid.p, want, cudaMemcpyDeviceToHost, ctx->stream));
    NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t j = 0; j < want; ++j) {
      if (!hvalid[j]) continue;
      std::memcpy(static_feats + got * 81, &hst[j * 81], sizeof(float) * 81);
      std::memcpy(resid_feats + got * 27, &hrf[j * 27], sizeof(float) * 27);
      targets[got] = htg[j];
      if (rows_out) rows_out[got] = hrows[j];
      ++got;
    }
  }
  *n_out = got;
  return cuda_check(ctx, cudaGetLastError(), "harvest");
}

void nalu_train_opts_default(nalu_train_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->epochs = 40;
  o->batch = 256;
  o->lr = 1e-3;
  o->val_fraction = 0.1;
  o->seed = 1;
}

int nalu_learned_gradient(nalu_ctx* ctx, const float* static_feats, const float* resid_feats, const float* targets,
                          int64_t n, float* grad, double* loss) {
  if (!ctx || !static_feats || !resid_feats || !targets || !grad || n < 1) return NALU_ERR_ARG;
  if (n > 1024) return set_error(ctx, NALU_ERR_ARG, "at most 1024 samples per gradient");
  if (!ctx->learned.has_weights) return set_error(ctx, NALU_ERR_STATE, "no weights");
  cudaSetDevice(ctx->device);
  const int B = (int)n;
  TrainWork w;
  int rc = w.alloc(ctx, B, 1);
  if (rc) return rc;
  DBuf<int32_t> idx;
  NALU_CUDA(ctx, idx.alloc(B));
  std::vector<int32_t> hidx(B);
  std::iota(hidx.begin(), hidx.end(), 0);
  NALU_CUDA(ctx, cudaMemcpyAsync(idx.p, hidx.data(), sizeof(int32_t) * B, cudaMemcpyHostToDevice, ctx->stream));
  DBuf<float> st, rf, tg;
  NALU_CUDA(ctx, st.alloc(n * 81));
  NALU_CUDA(ctx, rf.alloc(n * 27));
  NALU_CUDA(ctx, tg.alloc(n));
  NALU_CUDA(ctx, cudaMemcpyAsync(st.p, static_feats, sizeof(float) * n * 81, cudaMemcpyHostToDevice, ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(rf.p, resid_feats, sizeof(float) * n * 27, cudaMemcpyHostToDevice, ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(tg.p, targets, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
  k_tr_gather<<<B, 128, 0, ctx->stream>>>(B, idx.p, nullptr, 0, st.p, rf.p, tg.p, w.stb.p, w.rfb.p, w.tgb.p);
  ctx->launches++;
  const float* P = ctx->learned.params.p;
  forward(ctx, w, P, B, nullptr);
  backward(ctx, w, P, ctx->learned.grad.p);
  float l = 0.0f;
  NALU_CUDA(ctx, cudaMemcpyAsync(grad, ctx->learned.grad.p, sizeof(float) * kNP, cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(&l, w.loss.p, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (loss) *loss = l;
  return cuda_check(ctx, cudaGetLastError(), "gradient");
}

int nalu_learned_gradient_bf16(nalu_ctx* ctx, const float* static_feats, const float* resid_feats,
                               const float* targets, int64_t n, float* grad, double* loss) {
  if (!ctx || !static_feats || !resid_feats || !targets || !grad || n < 1 || n > INT_MAX / 81) return NALU_ERR_ARG;
  if (!ctx->learned.has_weights) return set_error(ctx, NALU_ERR_STATE, "no weights");
  cudaSetDevice(ctx->device);
  DBuf<int32_t> idx;
  DBuf<float> st, rf, tg, g, l;
  NALU_CUDA(ctx, idx.alloc(n));
  NALU_CUDA(ctx, st.alloc(n * 81));
  NALU_CUDA(ctx, rf.alloc(n * 27));
  NALU_CUDA(ctx, tg.alloc(n));
  NALU_CUDA(ctx, g.alloc(kNP));
  NALU_CUDA(ctx, l.alloc(1));
  std::vector<int32_t> hidx(n);
  std::iota(hidx.begin(), hidx.end(), 0);
  cudaStream_t s0 = ctx->stream;
  NALU_CUDA(ctx, cudaMemcpyAsync(idx.p, hidx.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s0));
  NALU_CUDA(ctx, cudaMemcpyAsync(st.p, static_feats, sizeof(float) * n * 81, cudaMemcpyHostToDevice, s0));
  NALU_CUDA(ctx, cudaMemcpyAsync(rf.p, resid_feats, sizeof(float) * n * 27, cudaMemcpyHostToDevice, s0));
  NALU_CUDA(ctx, cudaMemcpyAsync(tg.p, targets, sizeof(float) * n, cudaMemcpyHostToDevice, s0));
  int rc = gradient_tc(ctx, st.p, rf.p, tg.p, idx.p, (int)n, g.p, l.p);
  if (rc) return rc;
  float lv = 0.0f;
  NALU_CUDA(ctx, cudaMemcpyAsync(grad, g.p, sizeof(float) * kNP, cudaMemcpyDeviceToHost, s0));
  NALU_CUDA(ctx, cudaMemcpyAsync(&lv, l.p, sizeof(float), cudaMemcpyDeviceToHost, s0));
  NALU_CUDA(ctx, cudaStreamSynchronize(s0));
  if (loss) *loss = lv;
  return NALU_OK;
}

int nalu_learned_train(nalu_ctx* ctx, const float* static_feats, const float* resid_feats, const float* targets,
                       int64_t n, const nalu_train_opts* opts, float* history) {
  if (!ctx || !static_feats || !resid_feats || !targets || !opts || n < 2) return NALU_ERR_ARG;
  const int B = opts->batch;
  if (B < 1 || B > 1024 || opts->epochs < 1 || !(opts->lr > 0.0)) return set_error(ctx, NALU_ERR_ARG, "train opts");
  if (!ctx->learned.has_weights) return set_error(ctx, NALU_ERR_STATE, "no weights (nalu_learned_init)");
  cudaSetDevice(ctx->device);
  int rc = ensure_learned_buffers(ctx);
  if (rc) return rc;
  // shuffle once: the first n_val samples are held out
  uint64_t s = opts->seed;
  std::vector<int32_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  for (int64_t i = n - 1; i > 0; --i) std::swap(order[i], order[(int64_t)(uniform01(s) * (double)(i + 1)) % (i + 1)]);
  const int64_t n_val = std::min<int64_t>(n - 1, (int64_t)(opts->val_fraction * (double)n));
  const int64_t n_tr = n - n_val;
  const int steps_per_epoch = (int)(n_tr / B);
  if (steps_per_epoch < 1) return set_error(ctx, NALU_ERR_ARG, "fewer training samples than one batch");
  const int64_t total_steps = (int64_t)steps_per_epoch * opts->epochs;
  std::vector<int32_t> idx((size_t)total_steps * B);
  std::vector<int32_t> tr(order.begin() + n_val, order.end());
  for (int e = 0; e < opts->epochs; ++e) {
    for (int64_t i = n_tr - 1; i > 0; --i) std::swap(tr[i], tr[(int64_t)(uniform01(s) * (double)(i + 1)) % (i + 1)]);
    std::copy(tr.begin(), tr.begin() + (int64_t)steps_per_epoch * B, idx.begin() + (int64_t)e * steps_per_epoch * B);
  }
  const int val_batches = (int)((n_val + B - 1) / B);
  std::vector<int32_t> vidx((size_t)std::max(1, val_batches) * B, order.empty() ? 0 : order[0]);
  for (int64_t i = 0; i < n_val; ++i) vidx[i] = order[i];
  const bool tc = opts->precision == NALU_TRAIN_BF16;
  if (!tc && opts->precision != NALU_TRAIN_FP32) return set_error(ctx, NALU_ERR_ARG, "train opts: precision");
  DBuf<float> st, rf, tg;
  DBuf<int32_t> d_idx, d_vidx, d_step;
  NALU_CUDA(ctx, st.alloc(n * 81));
  NALU_CUDA(ctx, rf.alloc(n * 27));
  NALU_CUDA(ctx, tg.alloc(n));
  NALU_CUDA(ctx, d_idx.alloc((int64_t)idx.size()));
  NALU_CUDA(ctx, d_vidx.alloc((int64_t)vidx.size()));
  NALU_CUDA(ctx, d_step.alloc(1));
  cudaStream_t st0 = ctx->stream;
  NALU_CUDA(ctx, cudaMemcpyAsync(st.p, static_feats, sizeof(float) * n * 81, cudaMemcpyHostToDevice, st0));
  NALU_CUDA(ctx, cudaMemcpyAsync(rf.p, resid_feats, sizeof(float) * n * 27, cudaMemcpyHostToDevice, st0));
  NALU_CUDA(ctx, cudaMemcpyAsync(tg.p, targets, sizeof(float) * n, cudaMemcpyHostToDevice, st0));
  NALU_CUDA(ctx, cudaMemcpyAsync(d_idx.p, idx.data(), sizeof(int32_t) * idx.size(), cudaMemcpyHostToDevice, st0));
  NALU_CUDA(ctx, cudaMemcpyAsync(d_vidx.p, vidx.data(), sizeof(int32_t) * vidx.size(), cudaMemcpyHostToDevice, st0));
  NALU_CUDA(ctx, cudaMemsetAsync(d_step.p, 0, sizeof(int), st0));
  LearnedState& L = ctx->learned;
  NALU_CUDA(ctx, cudaMemsetAsync(L.adam_m.p, 0, sizeof(float) * kNP, st0));
  NALU_CUDA(ctx, cudaMemsetAsync(L.adam_v.p, 0, sizeof(float) * kNP, st0));
  if (tc) {
    TrainData d{st.p, rf.p, tg.p, d_idx.p, d_vidx.p, B, steps_per_epoch, opts->epochs, n_val, (float)opts->lr};
    return train_tc(ctx, d, history);
  }
  TrainWork w;
  if ((rc = w.alloc(ctx, B, total_steps))) return rc;
  TrainWork wv;
  if ((rc = wv.alloc(ctx, B, 1))) return rc;
  // one Adam step as a graph: gather, forward, backward, update, step++
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(st0, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "begin capture");
  k_tr_gather<<<B, 128, 0, st0>>>(B, d_idx.p, d_step.p, 0, st.p, rf.p, tg.p, w.stb.p, w.rfb.p, w.tgb.p);
  forward(ctx, w, L.params.p, B, d_step.p);
  backward(ctx, w, L.params.p, L.grad.p);
  k_adam<<<(kNP + 255) / 256, 256, 0, st0>>>(L.grad.p, L.params.p, L.adam_m.p, L.adam_v.p, d_step.p,
                                              (float)opts->lr);
  k_step_inc<<<1, 1, 0, st0>>>(d_step.p);
  ctx->launches += 3;
  ce = cudaStreamEndCapture(st0, &graph);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "end capture");
  ce = cudaGraphInstantiate(&exec, graph, 0);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cuda_check(ctx, ce, "instantiate");
  }
  std::vector<float> hl((size_t)total_steps);
  for (int e = 0; e < opts->epochs; ++e) {
    for (int k = 0; k < steps_per_epoch; ++k) cudaGraphLaunch(exec, st0);
    if (history) {
      double vs = 0.0;
      for (int vb = 0; vb < val_batches; ++vb) {
        const int nvalid = (int)std::min<int64_t>(B, n_val - (int64_t)vb * B);
        k_tr_gather<<<B, 128, 0, st0>>>(B, d_vidx.p, nullptr, vb, st.p, rf.p, tg.p, wv.stb.p, wv.rfb.p, wv.tgb.p);
        forward(ctx, wv, L.params.p, nvalid, nullptr);
        float l = 0.0f;
        NALU_CUDA(ctx, cudaMemcpyAsync(&l, wv.loss.p, sizeof(float), cudaMemcpyDeviceToHost, st0));
        NALU_CUDA(ctx, cudaStreamSynchronize(st0));
        vs += (double)l * nvalid;
      }
      history[2 * e + 1] = n_val > 0 ? (float)(vs / (double)n_val) : 0.0f;
    }
  }
  NALU_CUDA(ctx, cudaMemcpyAsync(hl.data(), w.loss.p, sizeof(float) * total_steps, cudaMemcpyDeviceToHost, st0));
  NALU_CUDA(ctx, cudaStreamSynchronize(st0));
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  if (history)
    for (int e = 0; e < opts->epochs; ++e) {
      double m = 0.0;
      for (int k = 0; k < steps_per_epoch; ++k) m += hl[(size_t)e * steps_per_epoch + k];
      history[2 * e] = (float)(m / steps_per_epoch);
    }
  return cuda_check(ctx, cudaGetLastError(), "train");
}

int nalu_learned_stencil(nalu_ctx* ctx, float* stencil) {
  if (!ctx || !stencil) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no linear system");
  int rc = check_scalar(ctx);
  if (rc) return rc;
  if (!ctx->learned.has_weights) return set_error(ctx, NALU_ERR_STATE, "no weights");
  cudaSetDevice(ctx->device);
  if ((rc = compute_dinv(ctx)) || (rc = build_slot_map(ctx)) || (rc = launch_stencil(ctx))) return rc;
  NALU_CUDA(ctx, cudaMemcpyAsync(stencil, ctx->learned.stencil.p, sizeof(float) * ctx->n_rows * 27,
                                 cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

}  // extern "C"
