// krylov.cu -- sm_103a Krylov solvers for the assembled CRS system.
//
// Replaces TpetraLinearSolver::solve (src/LinearSolver.C:183-232), i.e.
// Belos CG/GMRES with an Ifpack2 Jacobi (RELAXATION, one sweep) or Chebyshev
// preconditioner (src/LinearSolverConfig.C:71-97).  Stopping rule: the true
// FP64 residual ||b - A x||_2 / ||b||_2 <= tol, verified after the iteration
// has converged on its recursive residual.
//
// All scalars stay on the device; a chunk of `check_every` iterations is
// captured once into a CUDA graph and replayed, with one 8-byte read-back per
// chunk.  Reductions are deterministic (fixed grid, per-block partials,
// single-block finish).  Rows that are identity rows (Dirichlet and pinned
// rows of applyDirichletBCs / resetRows + sumInto) start from x = b there, so
// their residual is zero and CG runs on the complementary block, which is
// symmetric for the continuity and diffusion operators.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstdint>
#include <mutex>
#include <vector>

#include "internal.h"

namespace nalu_gb300 {

constexpr int kRedBlocks = 1024;   // fixed grid for deterministic reductions
constexpr int kRedThreads = 256;
constexpr int kMaxRestart = 1000;  // Krylov basis size bound of GMRES(m)

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <class T>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// accumulator of a row: FP32 when matrix and vector are FP32 (the inner
// solve of the FP32-inner / FP64-refinement scheme), FP64 otherwise
template <class VT, class XT> struct RowAcc { using type = double; };
template <> struct RowAcc<float, float> { using type = float; };

// y = A x, TPR threads per row; optional partial of dot(x_own, y)
template <class VT, class XT, int TPR, bool DOT>
__global__ void __launch_bounds__(256) k_spmv(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                              const VT* __restrict__ v, const XT* __restrict__ x, XT* __restrict__ y,
                                              double* __restrict__ partial) {
  __shared__ double sh[32];
  const int sub = threadIdx.x % TPR;
  const int64_t rows_per_block = blockDim.x / TPR;
  double dot = 0.0;
  // the loop bound is uniform across the warp (all lanes reach the shuffles)
  using Acc = typename RowAcc<VT, XT>::type;
  for (int64_t base = (int64_t)blockIdx.x * rows_per_block; base < n; base += (int64_t)gridDim.x * rows_per_block) {
    const int64_t row = base + threadIdx.x / TPR;
    const bool valid = row < n;
    Acc s = 0;
    if (valid) {
      const int64_t b = __ldg(rp + row), e = __ldg(rp + row + 1);
      for (int64_t j = b + sub; j < e; j += TPR) s += (Acc)__ldg(v + j) * (Acc)__ldg(x + __ldg(ci + j));
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, TPR);
    if (valid && sub == 0) {
      y[row] = (XT)s;
      if (DOT) dot += (double)s * (double)x[row];
    }
  }
  if (DOT) {
    const double t = block_sum<double>(dot, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

// y = A x on the FP32 3x3-block copy: TPB threads per node row, each
// summing the 3x3 products of its blocks (value k = 3 r + c of block b at
// bv[k * nblk + b]); 4.4 bytes per nonzero against 8 for FP32 CRS.
template <class XT, int TPB, bool DOT>
__global__ void __launch_bounds__(256) k_spmv_b3(int64_t nb, int64_t nblk, const int64_t* __restrict__ brp,
                                                 const int32_t* __restrict__ bcol, const float* __restrict__ bv,
                                                 const XT* __restrict__ x, XT* __restrict__ y,
                                                 double* __restrict__ partial) {
  __shared__ double sh[32];
  using Acc = typename RowAcc<float, XT>::type;
  const int sub = threadIdx.x % TPB;
  const int64_t nodes_per_block = blockDim.x / TPB;
  double dot = 0.0;
  // the loop bound is uniform across the warp (all lanes reach the shuffles)
  for (int64_t base = (int64_t)blockIdx.x * nodes_per_block; base < nb; base += (int64_t)gridDim.x * nodes_per_block) {
    const int64_t node = base + threadIdx.x / TPB;
    const bool valid = node < nb;
    Acc s0 = 0, s1 = 0, s2 = 0;
    if (valid) {
      const int64_t e = __ldg(brp + node + 1);
      for (int64_t b = __ldg(brp + node) + sub; b < e; b += TPB) {
        const int64_t c3 = 3 * (int64_t)__ldg(bcol + b);
        const Acc x0 = (Acc)__ldg(x + c3), x1 = (Acc)__ldg(x + c3 + 1), x2 = (Acc)__ldg(x + c3 + 2);
        float a[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) a[k] = __ldg(bv + k * nblk + b);
        s0 += (Acc)a[0] * x0 + (Acc)a[1] * x1 + (Acc)a[2] * x2;
        s1 += (Acc)a[3] * x0 + (Acc)a[4] * x1 + (Acc)a[5] * x2;
        s2 += (Acc)a[6] * x0 + (Acc)a[7] * x1 + (Acc)a[8] * x2;
      }
    }
#pragma unroll
    for (int o = TPB / 2; o > 0; o >>= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, o, TPB);
      s1 += __shfl_xor_sync(0xffffffffu, s1, o, TPB);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o, TPB);
    }
    if (valid && sub == 0) {
      y[3 * node] = (XT)s0;
      y[3 * node + 1] = (XT)s1;
      y[3 * node + 2] = (XT)s2;
      if (DOT) dot += (double)s0 * (double)x[3 * node] + (double)s1 * (double)x[3 * node + 1] +
                      (double)s2 * (double)x[3 * node + 2];
    }
  }
  if (DOT) {
    const double t = block_sum<double>(dot, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

// Structure of the 3x3-block copy, one warp per node (lanes over the
// node's column triples).  The CRS graph must have the 3-dof Tpetra form:
// the three rows of a node share one column pattern made of whole column
// triples (3 c, 3 c + 1, 3 c + 2).  A node that breaks it sets *bad;
// otherwise brp[node] = rp[3 node] / 9 and the block columns follow the
// first row's triples.
__global__ void k_b3_struct(int64_t nb, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            int64_t* __restrict__ brp, int32_t* __restrict__ bcol, int* __restrict__ bad) {
  const int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (node > nb) return;
  if (node == nb) {
    if (lane == 0) {
      const int64_t nnz = rp[3 * nb];
      if (nnz % 9) atomicOr(bad, 1);
      brp[nb] = nnz / 9;
    }
    return;
  }
  const int64_t r0 = rp[3 * node], len = rp[3 * node + 1] - r0;
  bool ok = len % 3 == 0 && r0 % 9 == 0 && rp[3 * node + 2] - rp[3 * node + 1] == len &&
            rp[3 * node + 3] - rp[3 * node + 2] == len;
  if (ok) {
    const int64_t b0 = r0 / 9;
    if (lane == 0) brp[node] = b0;
    for (int64_t t = lane; t < len / 3; t += 32) {
      const int64_t e = 3 * t;
      const int32_t c = ci[r0 + e];
      bool tok = c % 3 == 0 && ci[r0 + e + 1] == c + 1 && ci[r0 + e + 2] == c + 2;
      for (int r = 1; r < 3; ++r) {
        const int64_t rr = rp[3 * node + r] + e;
        tok = tok && ci[rr] == c && ci[rr + 1] == c + 1 && ci[rr + 2] == c + 2;
      }
      bcol[b0 + t] = c / 3;
      ok = ok && tok;
    }
  }
  if (!ok) atomicOr(bad, 1);
}

// FP32 block values from the FP64 CRS values, one warp per row (coalesced
// reads; each lane's entry goes to plane 3 (row % 3) + entry % 3).
__global__ void k_b3_values(int64_t n, int64_t nblk, const int64_t* __restrict__ rp, const double* __restrict__ v,
                            float* __restrict__ bv) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const int64_t r0 = rp[row], len = rp[row + 1] - r0, b0 = rp[row - row % 3] / 9;
  const int plane0 = 3 * (int)(row % 3);
  for (int64_t e = lane; e < len; e += 32) bv[(int64_t)(plane0 + (int)(e % 3)) * nblk + b0 + e / 3] = (float)v[r0 + e];
}

// r = b - A x (FP64), with partial of r.r
__global__ void __launch_bounds__(256) k_residual(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                                  const double* __restrict__ v, const double* __restrict__ x,
                                                  const double* __restrict__ b, double* __restrict__ r,
                                                  double* __restrict__ partial) {
  __shared__ double sh[32];
  constexpr int TPR = 8;
  const int sub = threadIdx.x % TPR;
  const int64_t rows_per_block = blockDim.x / TPR;
  double acc = 0.0;
  for (int64_t base = (int64_t)blockIdx.x * rows_per_block; base < n; base += (int64_t)gridDim.x * rows_per_block) {
    const int64_t row = base + threadIdx.x / TPR;
    const bool valid = row < n;
    double s = 0.0;
    if (valid) {
      const int64_t s0 = __ldg(rp + row), e = __ldg(rp + row + 1);
      for (int64_t j = s0 + sub; j < e; j += TPR) s += __ldg(v + j) * __ldg(x + __ldg(ci + j));
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, TPR);
    if (valid && sub == 0) {
      const double d = b[row] - s;
      r[row] = d;
      acc += d * d;
    }
  }
  const double t = block_sum<double>(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// finish a reduction of `nparts` partial arrays into scal[dst..]
// (one warp per part, lanes over the blocks in a fixed order)
__global__ void k_finish(const double* __restrict__ partial, int nblocks, int nparts, double* scal, int dst) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int p = wid; p < nparts; p += nw) {
    double s = 0.0;
    for (int i = lane; i < nblocks; i += 32) s += partial[p * nblocks + i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) scal[dst + p] = s;
  }
}

// scalar slots
enum { S_RZ = 0, S_PQ = 1, S_RZNEW = 2, S_RR = 3, S_ALPHA = 4, S_BETA = 5, S_BB = 6, S_TMP = 7, S_BAD = 8, S_STOP = 9 };

// True once r.r has reached the stop threshold scal[S_STOP] (0: none set).
// CG iterations run in chunks captured as one graph, so a chunk can overrun
// convergence; past the threshold alpha = beta = 0 freezes the iterate
// instead of driving an FP32 recurrence residual to zero (and 0/0).
__device__ __forceinline__ bool cg_frozen(const double* scal) {
  return scal[S_STOP] > 0.0 && scal[S_RR] <= scal[S_STOP];
}

__device__ __forceinline__ void k_alpha_body(double* scal) {
  if (cg_frozen(scal)) {
    scal[S_ALPHA] = 0.0;
    return;
  }
  const double pq = scal[S_PQ];
  const double a = scal[S_RZ] / pq;
  scal[S_ALPHA] = isfinite(a) ? a : 0.0;
  if (!isfinite(a)) scal[S_BAD] = 1.0;
}
__global__ void k_alpha(double* scal) { k_alpha_body(scal); }
__global__ void k_beta(double* scal) {
  if (cg_frozen(scal)) {
    scal[S_BETA] = 0.0;
    return;
  }
  const double b = scal[S_RZNEW] / scal[S_RZ];
  scal[S_BETA] = isfinite(b) ? b : 0.0;
  if (!isfinite(b)) scal[S_BAD] = 1.0;
  scal[S_RZ] = scal[S_RZNEW];
}

// x += a p ; r -= a q ; z = M^-1 r (Jacobi) ; partials r.z and r.r
template <class T>
__global__ void __launch_bounds__(kRedThreads) k_cg_update(int64_t n, const double* __restrict__ scal, T* __restrict__ x,
                                                           const T* __restrict__ p, T* __restrict__ r,
                                                           const T* __restrict__ q, T* __restrict__ z,
                                                           const T* __restrict__ dinv, double* __restrict__ partial,
                                                           int write_z) {
  __shared__ double sh[32];
  const double a = scal[S_ALPHA];
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = (T)((double)x[i] + a * (double)p[i]);
    const double ri = (double)r[i] - a * (double)q[i];
    r[i] = (T)ri;
    const double zi = (double)dinv[i] * ri;
    if (write_z) z[i] = (T)zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  const double t1 = block_sum<double>(rz, sh);
  const double t2 = block_sum<double>(rr, sh);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = t1;
    partial[gridDim.x + blockIdx.x] = t2;
  }
}

// p = z + beta p
template <class T>
__global__ void k_p_update(int64_t n, const double* __restrict__ scal, const T* __restrict__ z, T* __restrict__ p) {
  const double b = scal[S_BETA];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = (T)((double)z[i] + b * (double)p[i]);
}

// inverse diagonal and identity-row mask
template <class VT, class T>
__global__ void k_dinv(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                       const VT* __restrict__ v, T* __restrict__ dinv, uint8_t* __restrict__ idmask) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  bool off_zero = true;
  for (int64_t j = rp[i]; j < rp[i + 1]; ++j) {
    if (ci[j] == i) d = (double)v[j];
    else if (v[j] != (VT)0) off_zero = false;
  }
  dinv[i] = (T)(d != 0.0 ? 1.0 / d : 1.0);
  if (idmask) idmask[i] = (off_zero && d == 1.0) ? 1 : 0;
}

// x0: zero (or kept), then identity rows take x = b
__global__ void k_init_x(int64_t n, double* __restrict__ x, const double* __restrict__ b,
                         const uint8_t* __restrict__ idmask, int zero) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = zero ? 0.0 : x[i];
  if (idmask[i]) v = b[i];
  x[i] = v;
}

template <class A, class B>
__global__ void k_convert(int64_t n, const A* __restrict__ a, B* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (B)a[i];
}

template <class T>
__global__ void k_copy_scale(int64_t n, const T* __restrict__ a, T* __restrict__ b, const double* __restrict__ dinv_d,
                             const T* __restrict__ dinv) {
  // b = dinv .* a
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (T)((double)dinv[i] * (double)a[i]);
}

// x += y (FP64 += T)
template <class T>
__global__ void k_add_to(int64_t n, double* __restrict__ x, const T* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += (double)y[i];
}

// ---------------------------------------------------------------------------
// GMRES helpers: dots of w against k+1 basis vectors, axpys, normalisation
// ---------------------------------------------------------------------------
// Finish of `nparts` per-block partial arrays (part p of block column b at
// partial[p * gridDim.x + b], stored by thread 0 of the block that owns it)
// into dst[p]: the block that arrives last (of gridDim.x * gridDim.y) sums
// every part, one warp per part, in a fixed order, and resets the counter.
__device__ __forceinline__ void last_block_finish(const double* partial, int nparts, unsigned* counter,
                                                  double* __restrict__ dst) {
  __shared__ unsigned ticket;
  if (counter == nullptr) return;  // the caller finishes with k_finish
  if (threadIdx.x == 0) {
    __threadfence();
    ticket = atomicAdd(counter, 1u);
  }
  __syncthreads();
  if (ticket != gridDim.x * gridDim.y - 1) return;
  __threadfence();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int p = wid; p < nparts; p += nw) {
    double s = 0.0;
#pragma unroll 8
    for (int i = lane; i < (int)gridDim.x; i += 32) s += __ldcg(partial + (size_t)p * gridDim.x + i);
    s = warp_sum(s);
    if (lane == 0) dst[p] = s;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// dst[j] = V_j . w for j < k (V column-major, n per column).  Eight dots per
// block row (blockIdx.y = j / 8, so the column groups run side by side);
// the column index is clamped so that all eight loads issue unconditionally
// (the duplicates past k hit the cache and are not summed).  Per-thread sums
// in T, block and grid sums in FP64.  A 1-D grid loops over the groups.
template <class T>
__global__ void __launch_bounds__(kRedThreads) k_multi_dot(int64_t n, int k, const T* __restrict__ V,
                                                           const T* __restrict__ w, double* __restrict__ partial,
                                                           unsigned* __restrict__ counter, double* __restrict__ dst) {
  __shared__ double sh[32];
  constexpr int C = 8;
  for (int j0 = (int)blockIdx.y * C; j0 < k; j0 += (int)gridDim.y * C) {
    const T* vp[C];
#pragma unroll
    for (int u = 0; u < C; ++u) vp[u] = V + (int64_t)min(j0 + u, k - 1) * n;
    T s[C];
#pragma unroll
    for (int u = 0; u < C; ++u) s[u] = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      const T wi = w[i];
      T a[C];
#pragma unroll
      for (int u = 0; u < C; ++u) a[u] = vp[u][i];
#pragma unroll
      for (int u = 0; u < C; ++u) s[u] += a[u] * wi;
    }
#pragma unroll
    for (int u = 0; u < C; ++u) {
      if (j0 + u >= k) break;  // uniform over the block
      const double t = block_sum<double>((double)s[u], sh);
      if (threadIdx.x == 0) partial[(size_t)(j0 + u) * gridDim.x + blockIdx.x] = t;
    }
  }
  last_block_finish(partial, k, counter, dst);
}

// w -= sum_j h_j V_j (j < k), then dst[0] = |w|^2.  Arithmetic in T; the
// coefficients are staged in dynamic shared memory, zero-padded to a
// multiple of eight so that eight clamped loads issue per step.
template <class T>
__global__ void __launch_bounds__(kRedThreads) k_multi_axpy(int64_t n, int k, const T* __restrict__ V, T* __restrict__ w,
                                                            const double* __restrict__ h, double* __restrict__ partial,
                                                            unsigned* __restrict__ counter, double* __restrict__ dst) {
  __shared__ double sh[32];
  extern __shared__ unsigned char dyn[];
  T* hs = reinterpret_cast<T*>(dyn);
  constexpr int C = 8;
  const int kp = (k + C - 1) / C * C;
  for (int j = threadIdx.x; j < kp; j += blockDim.x) hs[j] = j < k ? (T)h[j] : (T)0;
  __syncthreads();
  T ww = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T s = w[i];
    for (int j0 = 0; j0 < k; j0 += C) {
      T a[C];
#pragma unroll
      for (int u = 0; u < C; ++u) a[u] = V[(int64_t)min(j0 + u, k - 1) * n + i];
#pragma unroll
      for (int u = 0; u < C; ++u) s -= hs[j0 + u] * a[u];
    }
    w[i] = s;
    ww += s * s;
  }
  const double wt = block_sum<double>((double)ww, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = wt;
  last_block_finish(partial, 1, counter, dst);
}

template <class T>
inline size_t multi_axpy_smem(int k) { return sizeof(T) * (size_t)((k + 7) / 8 * 8); }
template <class T>
__global__ void k_scale_into(int64_t n, const T* __restrict__ w, T* __restrict__ out, const double* __restrict__ s,
                             int inv_sqrt) {
  const T f = (T)(inv_sqrt ? (s[0] > 0 ? 1.0 / sqrt(s[0]) : 0.0) : s[0]);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = f * w[i];
}
// z = sum_j y_j V_j (combination), into T
template <class T>
__global__ void k_combine(int64_t n, int k, const T* __restrict__ V, const double* __restrict__ y, T* __restrict__ z) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += y[j] * (double)V[(int64_t)j * n + i];
    z[i] = (T)s;
  }
}

namespace {

inline unsigned grid_for(int64_t n, int t) {
  const int64_t g = (n + t - 1) / t;
  return (unsigned)(g < kRedBlocks ? (g < 1 ? 1 : g) : kRedBlocks);
}

// Matrix view in a given value precision
template <class VT>
struct Mat {
  int64_t n;
  const int64_t* rp;
  const int32_t* ci;
  const VT* v;
  int tpr;
  // optional FP32 3x3-block copy (3-dof systems): used by spmv_launch when set
  const int64_t* brp = nullptr;
  const int32_t* bcol = nullptr;
  const float* bv = nullptr;
  int64_t nblk = 0;
};

template <class VT, class XT, bool DOT>
void spmv_launch(nalu_ctx* ctx, const Mat<VT>& A, const XT* x, XT* y, double* partial) {
  const int threads = 256;
  if (A.bv) {
    constexpr int TPB = 8;
    const int64_t nb = A.n / 3, npb = threads / TPB;
    k_spmv_b3<XT, TPB, DOT><<<DOT ? kRedBlocks : (unsigned)((nb + npb - 1) / npb), threads, 0, ctx->stream>>>(
        nb, A.nblk, A.brp, A.bcol, A.bv, x, y, partial);
    return;
  }
  if (A.tpr == 16) {
    const int64_t rpb = threads / 16;
    k_spmv<VT, XT, 16, DOT><<<DOT ? kRedBlocks : (unsigned)((A.n + rpb - 1) / rpb), threads, 0, ctx->stream>>>(
        A.n, A.rp, A.ci, A.v, x, y, partial);
  } else {
    const int64_t rpb = threads / 8;
    k_spmv<VT, XT, 8, DOT><<<DOT ? kRedBlocks : (unsigned)((A.n + rpb - 1) / rpb), threads, 0, ctx->stream>>>(
        A.n, A.rp, A.ci, A.v, x, y, partial);
  }
  ctx->launches++;
}

int ensure(nalu_ctx* ctx, DBuf<double>& b, int64_t n) {
  if (b.n < n) NALU_CUDA(ctx, b.alloc(n));
  return NALU_OK;
}
int ensuref(nalu_ctx* ctx, DBuf<float>& b, int64_t n) {
  if (b.n < n) NALU_CUDA(ctx, b.alloc(n));
  return NALU_OK;
}

// workspace per precision
template <class T>
struct Work {
  T *r, *z, *p, *q, *dinv, *x;
  T* V;
};

// Chebyshev polynomial preconditioner in D^-1 A on [lmax/ratio, lmax]
template <class VT, class T>
struct Cheb {
  int degree = 0;
  double lmin = 0, lmax = 0;
};

// one CG "chunk" of iterations recorded into the stream (graph-capturable)
template <class VT, class T>
void cg_chunk(nalu_ctx* ctx, const Mat<VT>& A, Work<T>& w, double* scal, double* partial, int iters, int precond,
              const Cheb<VT, T>& cheb, T* ctmp1, T* ctmp2);

// z = M^-1 r for Chebyshev (Saad, Iterative Methods, Alg. 12.1), recorded
template <class T>
__global__ void k_cheb_init(int64_t n, const T* __restrict__ dinv, const T* __restrict__ r, T* __restrict__ z,
                            T* __restrict__ d, double inv_theta) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double di = inv_theta * (double)dinv[i] * (double)r[i];
    d[i] = (T)di;
    z[i] = (T)di;
  }
}
// d = c1 d + c2 D^-1 (r - A z); z += d   (Az precomputed in az)
template <class T>
__global__ void k_cheb_step(int64_t n, const T* __restrict__ dinv, const T* __restrict__ r, const T* __restrict__ az,
                            T* __restrict__ z, T* __restrict__ d, double c1, double c2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double di = c1 * (double)d[i] + c2 * (double)dinv[i] * ((double)r[i] - (double)az[i]);
    d[i] = (T)di;
    z[i] = (T)((double)z[i] + di);
  }
}

template <class VT, class T>
void cheb_apply(nalu_ctx* ctx, const Mat<VT>& A, const T* dinv, const T* r, T* z, T* d, T* az,
                const Cheb<VT, T>& ch) {
  const int64_t n = A.n;
  const unsigned g = grid_for(n, 256);
  const double theta = 0.5 * (ch.lmax + ch.lmin), delta = 0.5 * (ch.lmax - ch.lmin);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  k_cheb_init<T><<<g, 256, 0, ctx->stream>>>(n, dinv, r, z, d, 1.0 / theta);
  ctx->launches++;
  for (int k = 1; k < ch.degree; ++k) {
    spmv_launch<VT, T, false>(ctx, A, z, az, nullptr);
    const double rho_new = 1.0 / (2.0 * sigma - rho);
    k_cheb_step<T><<<g, 256, 0, ctx->stream>>>(n, dinv, r, az, z, d, rho_new * rho, 2.0 * rho_new / delta);
    ctx->launches++;
    rho = rho_new;
  }
}

template <class VT, class T>
void cg_chunk(nalu_ctx* ctx, const Mat<VT>& A, Work<T>& w, double* scal, double* partial, int iters, int precond,
              const Cheb<VT, T>& cheb, T* ctmp1, T* ctmp2) {
  const int64_t n = A.n;
  const unsigned g = grid_for(n, kRedThreads);
  for (int it = 0; it < iters; ++it) {
    spmv_launch<VT, T, true>(ctx, A, w.p, w.q, partial);
    k_finish<<<1, 256, 0, ctx->stream>>>(partial, kRedBlocks, 1, scal, S_PQ);
    k_alpha<<<1, 1, 0, ctx->stream>>>(scal);
    const bool jac = precond != NALU_PRECOND_CHEBYSHEV;
    k_cg_update<T><<<g, kRedThreads, 0, ctx->stream>>>(n, scal, w.x, w.p, w.r, w.q, w.z, w.dinv, partial, jac ? 1 : 0);
    // r.z (Jacobi) and r.r -> scal[S_RZNEW], scal[S_RR]
    k_finish<<<1, 256, 0, ctx->stream>>>(partial, g, 2, scal, S_RZNEW);
    ctx->launches += 4;
    if (!jac) {
      // z = cheb(r); r.z recomputed with the Chebyshev z
      cheb_apply<VT, T>(ctx, A, w.dinv, w.r, w.z, ctmp1, ctmp2, cheb);
      k_multi_dot<T><<<g, kRedThreads, 0, ctx->stream>>>(n, 1, w.r, w.z, partial, nullptr, nullptr);
      k_finish<<<1, 256, 0, ctx->stream>>>(partial, g, 1, scal, S_RZNEW);
      ctx->launches += 2;
    }
    k_beta<<<1, 1, 0, ctx->stream>>>(scal);
    k_p_update<T><<<g, kRedThreads, 0, ctx->stream>>>(n, scal, w.z, w.p);
    ctx->launches += 3;
  }
}

// Power iteration estimate of lambda_max(D^-1 A)
template <class VT, class T>
double estimate_lmax(nalu_ctx* ctx, const Mat<VT>& A, const T* dinv, T* a, T* b, double* partial, double* scal) {
  const int64_t n = A.n;
  const unsigned g = grid_for(n, 256);
  // deterministic, non-smooth start vector
  {
    std::vector<T> start(n);
    for (int64_t i = 0; i < n; ++i) start[i] = (T)(1.0 + 0.37 * std::sin(0.7 * (double)i));
    cudaMemcpyAsync(a, start.data(), sizeof(T) * n, cudaMemcpyHostToDevice, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
  }
  double lam = 1.0;
  for (int it = 0; it < 30; ++it) {
    spmv_launch<VT, T, false>(ctx, A, a, b, nullptr);
    k_copy_scale<T><<<g, 256, 0, ctx->stream>>>(n, b, b, nullptr, dinv);
    k_multi_dot<T><<<g, kRedThreads, 0, ctx->stream>>>(n, 1, b, b, partial, nullptr, nullptr);
    k_finish<<<1, 256, 0, ctx->stream>>>(partial, g, 1, scal, S_TMP);
    k_scale_into<T><<<g, 256, 0, ctx->stream>>>(n, b, a, scal + S_TMP, 1);
    ctx->launches += 4;
    double nn = 0;
    cudaMemcpyAsync(&nn, scal + S_TMP, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    lam = std::sqrt(nn);
  }
  return lam;
}

double read_scalar(nalu_ctx* ctx, double* d) {
  double h = 0;
  cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  return h;
}

// true residual r = b - A x into sw.r, returns ||r||_2
// ||v|| (FP64, fixed-order reduction)
double vec_norm(nalu_ctx* ctx, const double* v) {
  const int64_t n = ctx->n_rows;
  k_multi_dot<double><<<grid_for(n, kRedThreads), kRedThreads, 0, ctx->stream>>>(n, 1, v, v, ctx->sw.partial.p,
                                                                                  nullptr, nullptr);
  k_finish<<<1, 256, 0, ctx->stream>>>(ctx->sw.partial.p, grid_for(n, kRedThreads), 1, ctx->sw.scal.p, S_TMP);
  ctx->launches += 2;
  return std::sqrt(read_scalar(ctx, ctx->sw.scal.p + S_TMP));
}

double true_residual(nalu_ctx* ctx, const double* x, double* r) {
  const int64_t n = ctx->n_rows;
  k_residual<<<kRedBlocks, 256, 0, ctx->stream>>>(n, ctx->d_rowptr.p, ctx->d_colind.p, ctx->d_values.p, x,
                                                   ctx->d_rhs.p, r, ctx->sw.partial.p);
  k_finish<<<1, 256, 0, ctx->stream>>>(ctx->sw.partial.p, kRedBlocks, 1, ctx->sw.scal.p, S_TMP);
  ctx->launches += 2;
  return std::sqrt(read_scalar(ctx, ctx->sw.scal.p + S_TMP));
}

// Preconditioned CG on A z = r0 (precision T), starting from z = 0.  On
// return w.x holds the correction.  Stops when ||r|| <= rtol * ||r0||.
template <class VT, class T>
int pcg(nalu_ctx* ctx, const Mat<VT>& A, Work<T>& w, double rtol, int max_it, int check_every, int precond,
        const Cheb<VT, T>& cheb, T* ct1, T* ct2, int* iters_out, double r0norm) {
  const int64_t n = A.n;
  const unsigned g = grid_for(n, kRedThreads);
  double* scal = ctx->sw.scal.p;
  double* partial = ctx->sw.partial.p;
  // z = M^-1 r ; p = z ; rz = r.z
  if (precond == NALU_PRECOND_CHEBYSHEV) {
    cheb_apply<VT, T>(ctx, A, w.dinv, w.r, w.z, ct1, ct2, cheb);
  } else {
    k_copy_scale<T><<<g, 256, 0, ctx->stream>>>(n, w.r, w.z, nullptr, w.dinv);
    ctx->launches++;
  }
  cudaMemcpyAsync(w.p, w.z, sizeof(T) * n, cudaMemcpyDeviceToDevice, ctx->stream);
  k_multi_dot<T><<<g, kRedThreads, 0, ctx->stream>>>(n, 1, w.r, w.z, partial, nullptr, nullptr);
  k_finish<<<1, 256, 0, ctx->stream>>>(partial, g, 1, scal, S_RZ);
  ctx->launches += 2;
  // capture a chunk into a graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const int chunk = check_every > 0 ? check_every : 25;
  cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  cg_chunk<VT, T>(ctx, A, w, scal, partial, chunk, precond, cheb, ct1, ct2);
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "capture CG chunk");
  ce = cudaGraphInstantiate(&exec, graph, 0);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cuda_check(ctx, ce, "instantiate CG chunk");
  }
  int it = 0;
  int rc = NALU_OK;
  const double stop = rtol * r0norm;
  const double rr0 = r0norm * r0norm, stop2 = stop * stop;
  cudaMemcpyAsync(scal + S_RR, &rr0, sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(scal + S_STOP, &stop2, sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  while (it < max_it) {
    cudaGraphLaunch(exec, ctx->stream);
    it += chunk;
    double h[2] = {0, 0};
    cudaMemcpyAsync(h, scal + S_RR, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(h + 1, scal + S_BAD, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      rc = cuda_check(ctx, e, "CG");
      break;
    }
    if (h[1] != 0.0 || !std::isfinite(h[0])) {
      rc = set_error(ctx, NALU_ERR_NONFINITE, "CG breakdown (non-finite scalar)");
      break;
    }
    if (std::sqrt(h[0]) <= stop) break;
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  *iters_out = it;
  if (rc == NALU_OK && it >= max_it) rc = NALU_ERR_NOT_CONVERGED;
  return rc;
}

// Right-preconditioned GMRES(m) on A x = r0 (x from 0), Jacobi or none.
template <class VT, class T>
int gmres(nalu_ctx* ctx, const Mat<VT>& A, Work<T>& w, double rtol, int max_it, int m, int precond,
          int* iters_out, double r0norm) {
  const int64_t n = A.n;
  const unsigned g = grid_for(n, kRedThreads);
  // Gram-Schmidt kernels: one resident wave (k_multi_dot holds 16 sums and
  // 8 column pointers per thread, so fewer blocks fit than kRedBlocks)
  const unsigned gw = std::min(g, wave_grid(ctx, (const void*)k_multi_dot<T>, kRedThreads));
  double* scal = ctx->sw.scal.p;
  double* partial = ctx->sw.partial.p;
  // r (T) holds the initial residual; x (T) accumulates the solution
  // dh: pass-1 and pass-2 Gram-Schmidt coefficients side by side, each
  // [h_0..h_k, .., |w|^2 at m+1]; both come back to the host together, once
  // per column, into one of two pinned slots, while the device already
  // works on the next column (the host's Givens step overlaps it)
  const int hs = m + 2;
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), gv(m + 1), y(m);
  DBuf<double> dh;
  NALU_CUDA(ctx, dh.alloc(2 * hs));
  if (ctx->sw.ccount.n < 1) NALU_CUDA(ctx, ctx->sw.ccount.alloc(1));
  unsigned* cnt = ctx->sw.ccount.p;
  NALU_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(unsigned), ctx->stream));
  double* hpin = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaError_t he = cudaMallocHost(&hpin, sizeof(double) * 4 * hs);
  if (he == cudaSuccess) he = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
  if (he == cudaSuccess) he = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
  auto release = [&]() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (hpin) cudaFreeHost(hpin);
    dh.free();
  };
  if (he != cudaSuccess) {
    release();
    return cuda_check(ctx, he, "GMRES host buffers");
  }
  cudaMemsetAsync(w.x, 0, sizeof(T) * n, ctx->stream);
  int it = 0;
  const double stop = rtol * r0norm;
  // residual of the current x: r_cur (T) = r0 - A x ; w.q is scratch
  T* rcur = w.z;
  cudaMemcpyAsync(rcur, w.r, sizeof(T) * n, cudaMemcpyDeviceToDevice, ctx->stream);
  double beta = r0norm;
  int rc = NALU_OK;
  T* V = w.V;
  // column k: w = A M^-1 v_k, CGS2 against v_0..v_k, v_k+1 = w / |w| (the
  // norm read on the device), coefficients to pinned slot k % 2 + event
  auto enqueue_column = [&](int k) {
    T* vk = V + (int64_t)k * n;
    T* wv = V + (int64_t)(k + 1) * n;
    if (precond == NALU_PRECOND_JACOBI) {
      k_copy_scale<T><<<g, 256, 0, ctx->stream>>>(n, vk, w.q, nullptr, w.dinv);
      spmv_launch<VT, T, false>(ctx, A, w.q, wv, nullptr);
      ctx->launches++;
    } else {
      spmv_launch<VT, T, false>(ctx, A, vk, wv, nullptr);
    }
    // classical Gram-Schmidt, twice (CGS2)
    for (int pass = 0; pass < 2; ++pass) {
      double* hp = dh.p + pass * hs;
      // one resident wave in all: the 8-column groups side by side
      const unsigned gy = (unsigned)(k + 1 + 7) / 8, gx = std::max(1u, gw / gy);
      k_multi_dot<T><<<dim3(gx, gy), kRedThreads, 0, ctx->stream>>>(n, k + 1, V, wv, partial, cnt, hp);
      k_multi_axpy<T><<<g, kRedThreads, multi_axpy_smem<T>(k + 1), ctx->stream>>>(
          n, k + 1, V, wv, hp, partial + (size_t)(m + 1) * gx, cnt, hp + m + 1);
      ctx->launches += 2;
    }
    k_scale_into<T><<<g, 256, 0, ctx->stream>>>(n, wv, wv, dh.p + hs + m + 1, 1);
    cudaMemcpyAsync(hpin + (k & 1) * 2 * hs, dh.p, sizeof(double) * 2 * hs, cudaMemcpyDeviceToHost, ctx->stream);
    cudaEventRecord(ev[k & 1], ctx->stream);
    ctx->launches++;
  };
  // Givens step for column k once its coefficients are in; true when the
  // cycle ends with it (converged, or a non-finite rotation)
  auto process_column = [&](int k) -> bool {
    const cudaError_t e = cudaEventSynchronize(ev[k & 1]);
    if (e != cudaSuccess) {
      rc = cuda_check(ctx, e, "GMRES column");
      return true;
    }
    const double* hc = hpin + (k & 1) * 2 * hs;
    for (int j = 0; j <= k; ++j) H[(size_t)j * m + k] = hc[j] + hc[hs + j];
    H[(size_t)(k + 1) * m + k] = std::sqrt(hc[hs + m + 1]);
    for (int j = 0; j < k; ++j) {
      const double t = cs[j] * H[(size_t)j * m + k] + sn[j] * H[(size_t)(j + 1) * m + k];
      H[(size_t)(j + 1) * m + k] = -sn[j] * H[(size_t)j * m + k] + cs[j] * H[(size_t)(j + 1) * m + k];
      H[(size_t)j * m + k] = t;
    }
    const double a = H[(size_t)k * m + k], b = H[(size_t)(k + 1) * m + k];
    const double den = std::sqrt(a * a + b * b);
    cs[k] = den > 0 ? a / den : 1.0;
    sn[k] = den > 0 ? b / den : 0.0;
    H[(size_t)k * m + k] = den;
    H[(size_t)(k + 1) * m + k] = 0.0;
    gv[k + 1] = -sn[k] * gv[k];
    gv[k] = cs[k] * gv[k];
    if (!std::isfinite(gv[k + 1])) {
      rc = set_error(ctx, NALU_ERR_NONFINITE, "GMRES breakdown");
      return true;
    }
    return std::fabs(gv[k + 1]) <= stop;
  };
  while (it < max_it) {
    // V_0 = r / beta
    const double inv = 1.0 / beta;
    cudaMemcpyAsync(scal + S_TMP, &inv, sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    k_scale_into<T><<<g, 256, 0, ctx->stream>>>(n, rcur, V, scal + S_TMP, 0);
    ctx->launches++;
    std::fill(gv.begin(), gv.end(), 0.0);
    gv[0] = beta;
    int k = 0;  // columns processed in this cycle
    bool done = false;
    enqueue_column(0);
    int next = 1;  // next column to enqueue
    while (true) {
      // one column ahead (discarded if column k ends the cycle)
      if (next < m && it + (next - k) < max_it) enqueue_column(next++);
      done = process_column(k);
      ++k;
      ++it;
      if (done || k >= m || it >= max_it) break;
      if (next == k) enqueue_column(next++);
    }
    for (int j = k - 1; j >= 0; --j) {
      double s = gv[j];
      for (int l = j + 1; l < k; ++l) s -= H[(size_t)j * m + l] * y[l];
      y[j] = s / H[(size_t)j * m + j];
    }
    // x += M^-1 V y
    cudaMemcpyAsync(dh.p, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, ctx->stream);
    k_combine<T><<<g, 256, 0, ctx->stream>>>(n, k, V, dh.p, w.q);
    if (precond == NALU_PRECOND_JACOBI) k_copy_scale<T><<<g, 256, 0, ctx->stream>>>(n, w.q, w.q, nullptr, w.dinv);
    ctx->launches += 2;
    // x += q  (k_p_update with beta = 1:  p = z + 1 * p)
    const double one = 1.0;
    cudaMemcpyAsync(scal + S_BETA, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    k_p_update<T><<<g, kRedThreads, 0, ctx->stream>>>(n, scal, w.q, w.x);
    ctx->launches++;
    if (done || rc) break;
    // rcur = r0 - A x
    spmv_launch<VT, T, false>(ctx, A, w.x, w.q, nullptr);
    cudaMemcpyAsync(rcur, w.r, sizeof(T) * n, cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(dh.p, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    k_multi_axpy<T><<<g, kRedThreads, multi_axpy_smem<T>(1), ctx->stream>>>(n, 1, w.q, rcur, dh.p, partial, nullptr,
                                                                           nullptr);
    k_finish<<<1, 256, 0, ctx->stream>>>(partial, g, 1, scal, S_TMP);
    ctx->launches += 2;
    beta = std::sqrt(read_scalar(ctx, scal + S_TMP));
    if (beta <= stop) break;
  }
  cudaStreamSynchronize(ctx->stream);
  release();
  *iters_out = it;
  if (rc == NALU_OK && it >= max_it) rc = NALU_ERR_NOT_CONVERGED;
  return rc;
}

}  // namespace

// FP64 inverse diagonal into the solver workspace and the identity-row mask
int compute_dinv(nalu_ctx* ctx) {
  const int64_t n = ctx->n_rows;
  int rc = ensure(ctx, ctx->sw.dinv, n);
  if (rc) return rc;
  if (ctx->d_bcmask.n < n) NALU_CUDA(ctx, ctx->d_bcmask.alloc(n));
  k_dinv<double, double><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
      n, ctx->d_rowptr.p, ctx->d_colind.p, ctx->d_values.p, ctx->sw.dinv.p, ctx->d_bcmask.p);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "dinv");
}

int spmv_fp64(nalu_ctx* ctx, const double* x, double* y) {
  Mat<double> A{ctx->n_rows, ctx->d_rowptr.p, ctx->d_colind.p, ctx->d_values.p, ctx->num_dof >= 3 ? 16 : 8};
  spmv_launch<double, double, false>(ctx, A, x, y, nullptr);
  return cuda_check(ctx, cudaGetLastError(), "spmv");
}

namespace {

// FP32 3x3-block copy of the current FP64 matrix for the mixed-precision
// inner solve of a 3-dof system.  *ok stays false (and nothing is an error)
// when the graph is not of the 3-dof form or NALU_B3=0.
int b3_build(nalu_ctx* ctx, bool* ok) {
  *ok = false;
  SolverWork& s = ctx->sw;
  const int64_t n = ctx->n_rows;
  const char* env = std::getenv("NALU_B3");
  if (ctx->num_dof != 3 || n % 3 || ctx->nnz % 9 || (env && env[0] == '0')) return NALU_OK;
  const int64_t nb = n / 3, nblk = ctx->nnz / 9;
  if (s.b3rp.n < nb + 1) NALU_CUDA(ctx, s.b3rp.alloc(nb + 1));
  if (s.b3col.n < nblk) NALU_CUDA(ctx, s.b3col.alloc(nblk));
  if (s.b3val.n < 9 * nblk) NALU_CUDA(ctx, s.b3val.alloc(9 * nblk));
  if (s.b3flag.n < 1) NALU_CUDA(ctx, s.b3flag.alloc(1));
  NALU_CUDA(ctx, cudaMemsetAsync(s.b3flag.p, 0, sizeof(int), ctx->stream));
  k_b3_struct<<<(unsigned)(((nb + 1) * 32 + 255) / 256), 256, 0, ctx->stream>>>(nb, ctx->d_rowptr.p, ctx->d_colind.p,
                                                                                 s.b3rp.p, s.b3col.p, s.b3flag.p);
  ctx->launches++;
  int bad = 0;
  NALU_CUDA(ctx, cudaMemcpyAsync(&bad, s.b3flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (bad) return NALU_OK;
  k_b3_values<<<(unsigned)((n * 32 + 255) / 256), 256, 0, ctx->stream>>>(n, nblk, ctx->d_rowptr.p, ctx->d_values.p,
                                                                          s.b3val.p);
  ctx->launches++;
  s.b3_nblk = nblk;
  *ok = true;
  return cuda_check(ctx, cudaGetLastError(), "3x3-block copy");
}

template <class T>
int run_inner(nalu_ctx* ctx, const nalu_solver_opts& o, T* r, T* x, T* z, T* p, T* q, T* dinv, T* V, T* ct1, T* ct2,
              const void* vals, bool fp32vals, double rtol, double r0norm, int max_it, int* iters, bool b3 = false) {
  Work<T> w{r, z, p, q, dinv, x, V};
  const int tpr = ctx->num_dof >= 3 ? 16 : 8;
  if (fp32vals) {
    Mat<float> A{ctx->n_rows, ctx->d_rowptr.p, ctx->d_colind.p, (const float*)vals, tpr};
    if (b3) {
      A.brp = ctx->sw.b3rp.p;
      A.bcol = ctx->sw.b3col.p;
      A.bv = ctx->sw.b3val.p;
      A.nblk = ctx->sw.b3_nblk;
    }
    Cheb<float, T> ch;
    if (o.precond == NALU_PRECOND_CHEBYSHEV) {
      ch.degree = o.cheb_degree > 1 ? o.cheb_degree : 4;
      ch.lmax = 1.1 * estimate_lmax<float, T>(ctx, A, dinv, ct1, ct2, ctx->sw.partial.p, ctx->sw.scal.p);
      ch.lmin = ch.lmax / 30.0;
    }
    cudaMemsetAsync(x, 0, sizeof(T) * ctx->n_rows, ctx->stream);
    if (o.method == NALU_SOLVER_GMRES)
      return gmres<float, T>(ctx, A, w, rtol, max_it, o.restart > 0 ? o.restart : 50, o.precond, iters, r0norm);
    return pcg<float, T>(ctx, A, w, rtol, max_it, o.check_every, o.precond, ch, ct1, ct2, iters, r0norm);
  }
  Mat<double> A{ctx->n_rows, ctx->d_rowptr.p, ctx->d_colind.p, (const double*)vals, tpr};
  Cheb<double, T> ch;
  if (o.precond == NALU_PRECOND_CHEBYSHEV) {
    ch.degree = o.cheb_degree > 1 ? o.cheb_degree : 4;
    ch.lmax = 1.1 * estimate_lmax<double, T>(ctx, A, dinv, ct1, ct2, ctx->sw.partial.p, ctx->sw.scal.p);
    ch.lmin = ch.lmax / 30.0;
  }
  cudaMemsetAsync(x, 0, sizeof(T) * ctx->n_rows, ctx->stream);
  if (o.method == NALU_SOLVER_GMRES)
    return gmres<double, T>(ctx, A, w, rtol, max_it, o.restart > 0 ? o.restart : 50, o.precond, iters, r0norm);
  return pcg<double, T>(ctx, A, w, rtol, max_it, o.check_every, o.precond, ch, ct1, ct2, iters, r0norm);
}

}  // namespace

int solve(nalu_ctx* ctx, const nalu_solver_opts& o, nalu_solve_info* info) {
  const auto t0 = std::chrono::steady_clock::now();
  const int64_t n = ctx->n_rows;
  SolverWork& s = ctx->sw;
  const int m = o.restart > 0 ? o.restart : 50;
  if (o.method == NALU_SOLVER_GMRES && m > kMaxRestart)
    return set_error(ctx, NALU_ERR_ARG, "GMRES restart (Krylov space size) above 1000");
  int rc = NALU_OK;
  if ((rc = ensure(ctx, s.scal, 16))) return rc;
  if ((rc = ensure(ctx, s.partial, (int64_t)kRedBlocks * (m + 3)))) return rc;
  if ((rc = ensure(ctx, s.tmp, n))) return rc;
  if (ctx->d_bcmask.n < n) NALU_CUDA(ctx, ctx->d_bcmask.alloc(n));
  NALU_CUDA(ctx, cudaMemsetAsync(s.scal.p, 0, sizeof(double) * 16, ctx->stream));
  const unsigned g256 = (unsigned)((n + 255) / 256);
  const bool mixed = o.precision == NALU_PRECISION_FP32_INNER_IR;
  // identity rows and FP64 inverse diagonal
  if ((rc = ensure(ctx, s.dinv, n))) return rc;
  k_dinv<double, double><<<g256, 256, 0, ctx->stream>>>(n, ctx->d_rowptr.p, ctx->d_colind.p, ctx->d_values.p,
                                                        s.dinv.p, ctx->d_bcmask.p);
  k_init_x<<<g256, 256, 0, ctx->stream>>>(n, ctx->d_x.p, ctx->d_rhs.p, ctx->d_bcmask.p, o.x0_zero ? 1 : 0);
  ctx->launches += 2;
  // ||b||
  const double bnorm = [&]() {
    k_multi_dot<double><<<grid_for(n, kRedThreads), kRedThreads, 0, ctx->stream>>>(n, 1, ctx->d_rhs.p, ctx->d_rhs.p,
                                                                                    s.partial.p, nullptr, nullptr);
    k_finish<<<1, 256, 0, ctx->stream>>>(s.partial.p, grid_for(n, kRedThreads), 1, s.scal.p, S_BB);
    ctx->launches += 2;
    return std::sqrt(read_scalar(ctx, s.scal.p + S_BB));
  }();
  const double bref = bnorm > 0 ? bnorm : 1.0;
  const bool learned = o.precond == NALU_PRECOND_LEARNED;
  if (learned && (o.method != NALU_SOLVER_CG || mixed))
    return set_error(ctx, NALU_ERR_ARG, "the learned preconditioner runs in FP64 flexible CG only");
  const bool multilevel = o.precond == NALU_PRECOND_MULTILEVEL || o.precond == NALU_PRECOND_LEARNED_MULTILEVEL;
  if (multilevel && (o.method != NALU_SOLVER_CG || mixed || ctx->num_dof != 1))
    return set_error(ctx, NALU_ERR_ARG, "the multilevel preconditioner runs in FP64 flexible CG on scalar systems");
  bool fallback = false, probe_chose_jacobi = false;
  int learned_its = 0, probe_its = 0, pace_its = 0;
  double probe_rj = 0.0, probe_rl = 0.0;
  double setup_s = 0.0;
  nalu_solver_opts fb = o;  // Chebyshev-Jacobi PCG after a stall of the learned FCG
  fb.precond = NALU_PRECOND_CHEBYSHEV;
  int total_it = 0, outer = 0;
  bool b3 = false;  // the mixed-precision inner solve runs on the 3x3-block copy
  double res = true_residual(ctx, ctx->d_x.p, s.tmp.p) / bref;
  const int max_outer = mixed ? 60 : 8;
  while (res > o.tol && outer < max_outer && total_it < o.max_iters) {
    ++outer;
    const double r0 = res * bref;
    int its = 0;
    // inner target: full tolerance in FP64; a fixed reduction in FP32
    const double rtol = mixed ? (o.inner_tol > 0 ? o.inner_tol : 1e-4) : std::max(o.tol * bref / r0 * 0.5, 1e-15);
    if (!mixed) {
      if ((rc = ensure(ctx, s.r, n)) || (rc = ensure(ctx, s.z, n)) || (rc = ensure(ctx, s.p, n)) ||
          (rc = ensure(ctx, s.q, n)) || (rc = ensure(ctx, s.w, n)) || (rc = ensure(ctx, s.ap, n)))
        return rc;
      if (o.method == NALU_SOLVER_GMRES && (rc = ensure(ctx, s.V, (int64_t)(m + 1) * n))) return rc;
      cudaMemcpyAsync(s.r.p, s.tmp.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream);
      if (learned && !fallback) {
        // flexible CG with the learned stencil (learned.cu)
        const auto ts = std::chrono::steady_clock::now();
        const float2* sv2 = nullptr;
        if (outer == 1 && ((rc = sell_build<float2>(ctx, s.sell, &sv2)) || (rc = learned_prepare(ctx)))) return rc;
        NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        setup_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count();
        const int window = o.stall_window > 0 ? o.stall_window : 20;
        bool use_jacobi = false;
        if (outer == 1 && o.learned_probe) {
          // probe: a short run of each method from the same start; keep the one
          // that reduces the residual faster per unit of device time
          const int probe = std::max(40, 2 * window);
          cudaEvent_t pe[1];
          for (auto& e : pe) NALU_CUDA(ctx, cudaEventCreate(&e));
          int itj = 0, itl = 0, stl = 0;
          float msj = 0.f, msl = 0.f;  // device time of the iterations (set-up excluded)
          rc = pcg_df(ctx, s.sell, s.w.p, s.r.p, s.z.p, s.q.p, s.dinv.p, rtol, r0, probe, 10, &itj, &msj);
          const double resj = vec_norm(ctx, s.r.p);
          cudaMemcpyAsync(s.r.p, s.tmp.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream);
          const int rcl = fcg_learned(ctx, s.w.p, s.r.p, rtol, r0, probe, 10, 1 << 30, &itl, &stl, &msl);
          const double resl = vec_norm(ctx, s.r.p);
          for (auto& e : pe) cudaEventDestroy(e);
          // residual reduction per millisecond of iterations
          const double tj = itj * (double)msj / std::max(1, itj - 1), tl = itl * (double)msl / std::max(1, itl - 1);
          const double ratej = std::log(std::max(resj, 1e-300) / r0) / std::max(tj, 1e-3);
          const double ratel = std::log(std::max(resl, 1e-300) / r0) / std::max(tl, 1e-3);
          use_jacobi = stl || (rcl != NALU_OK && rcl != NALU_ERR_NOT_CONVERGED) || !(ratel < ratej);
          probe_rj = ratej;
          probe_rl = ratel;
          // pace: Jacobi-CG's probe rate, extrapolated, gives the iterations it
          // would need; the learned FCG gets at most twice as many
          if (resj < r0 && resj > 0.0) {
            const double need = itj * std::log(std::max(rtol, 1e-300)) / std::log(resj / r0);
            pace_its = (int)std::min(2.0 * need + probe, 2.0e9);
          }
          probe_its = itj + itl;
          learned_its += itl;
          rc = NALU_OK;
          cudaMemcpyAsync(s.r.p, s.tmp.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream);
        }
        if (use_jacobi) {
          probe_chose_jacobi = true;
          fallback = true;  // the rest of the solve runs Jacobi-CG
          rc = pcg_df(ctx, s.sell, s.w.p, s.r.p, s.z.p, s.q.p, s.dinv.p, rtol, r0, o.max_iters - total_it,
                      o.check_every, &its);
        } else {
          int stalled = 0;
          const int room = o.max_iters - total_it;
          const int budget = pace_its > 0 ? std::min(room, pace_its) : room;
          rc = fcg_learned(ctx, s.w.p, s.r.p, rtol, r0, budget, o.check_every, window, &its, &stalled);
          learned_its += its;
          if (stalled) {
            fallback = true;  // Chebyshev-Jacobi PCG from here
            rc = NALU_OK;
          } else if (rc == NALU_ERR_NOT_CONVERGED && budget < room) {
            probe_chose_jacobi = true;  // behind Jacobi-CG's pace: Jacobi-CG from the current iterate
            fallback = true;
            rc = NALU_OK;
          }
        }
      } else if (multilevel) {
        // aggregation multigrid in flexible CG (multilevel.cu), the hierarchy
        // built for this matrix once per call
        if (outer == 1) {
          const auto ts = std::chrono::steady_clock::now();
          const float2* sv2 = nullptr;  // the outer flexible CG's df64 SpMV and the fine-level cycle run
          if ((rc = sell_build<float2>(ctx, s.sell, &sv2)) || (rc = sell_c16_ensure(ctx, s.sell))) return rc;
          if (o.precond == NALU_PRECOND_LEARNED_MULTILEVEL && (rc = learned_prepare(ctx))) return rc;
          if ((rc = ml_setup(ctx, o.precond == NALU_PRECOND_LEARNED_MULTILEVEL))) return rc;
          NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
          setup_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count();
        }
        rc = fcg_multilevel(ctx, s.w.p, s.r.p, rtol, r0, o.max_iters - total_it, o.check_every, o.ml_kcycle_levels, o.ml_learned_sweeps,
                            &its);
      } else if (o.method == NALU_SOLVER_CG && (o.precond == NALU_PRECOND_JACOBI || probe_chose_jacobi)) {
        // two-kernel Jacobi-CG on the SELL-32 copy (cg_fast.cu)
        const float2* sv2 = nullptr;
        if (outer == 1 && (rc = sell_build<float2>(ctx, s.sell, &sv2))) return rc;
        rc = pcg_df(ctx, s.sell, s.w.p, s.r.p, s.z.p, s.q.p, s.dinv.p, rtol, r0, o.max_iters - total_it,
                    o.check_every, &its);
      } else {
        rc = run_inner<double>(ctx, learned ? fb : o, s.r.p, s.w.p, s.z.p, s.p.p, s.q.p, s.dinv.p, s.V.p, s.ap.p,
                               s.tmp.p, ctx->d_values.p, false, rtol, r0, o.max_iters - total_it, &its);
      }
      k_add_to<double><<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, ctx->d_x.p, s.w.p);
    } else {
      const bool fast_cg = o.method == NALU_SOLVER_CG && o.precond == NALU_PRECOND_JACOBI;
      if (outer == 1 && !fast_cg && (rc = b3_build(ctx, &b3))) return rc;
      if ((!b3 && (rc = ensuref(ctx, s.fvals, ctx->nnz))) || (rc = ensuref(ctx, s.fr, n)) || (rc = ensuref(ctx, s.fz, n)) ||
          (rc = ensuref(ctx, s.fp, n)) || (rc = ensuref(ctx, s.fq, n)) || (rc = ensuref(ctx, s.fdinv, n)) ||
          (rc = ensuref(ctx, s.fx, n)) || (rc = ensure(ctx, s.ap, n)))
        return rc;
      if (o.method == NALU_SOLVER_GMRES && (rc = ensuref(ctx, s.fV, (int64_t)(m + 1) * n))) return rc;
      DBuf<float> ft1, ft2;
      NALU_CUDA(ctx, ft1.alloc(n));
      NALU_CUDA(ctx, ft2.alloc(n));
      if (outer == 1) {
        if (!b3) k_convert<double, float><<<kRedBlocks, 256, 0, ctx->stream>>>(ctx->nnz, ctx->d_values.p, s.fvals.p);
        k_convert<double, float><<<kRedBlocks, 256, 0, ctx->stream>>>(n, s.dinv.p, s.fdinv.p);
        ctx->launches += b3 ? 1 : 2;
      }
      k_convert<double, float><<<kRedBlocks, 256, 0, ctx->stream>>>(n, s.tmp.p, s.fr.p);
      ctx->launches++;
      if (o.method == NALU_SOLVER_CG && o.precond == NALU_PRECOND_JACOBI) {
        const float* sv = nullptr;
        if (outer == 1 && (rc = sell_build<float>(ctx, s.sell, &sv))) return rc;
        sv = s.sell.valf.p;
        rc = pcg_fast<float, float>(ctx, sv, s.sell, s.fx.p, s.fr.p, s.fz.p, s.fp.p, ft1.p, s.fq.p, s.fdinv.p, rtol,
                                    r0, o.max_iters - total_it, o.check_every, &its);
      } else {
        rc = run_inner<float>(ctx, o, s.fr.p, s.fx.p, s.fz.p, s.fp.p, s.fq.p, s.fdinv.p, s.fV.p, ft1.p, ft2.p,
                              s.fvals.p, true, rtol, r0, o.max_iters - total_it, &its, b3);
      }
      k_add_to<float><<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, ctx->d_x.p, s.fx.p);
      cudaStreamSynchronize(ctx->stream);
      ft1.free();
      ft2.free();
      // an inner solve that stops at max iterations still improves x; the
      // outer loop decides convergence on the true residual
      if (rc == NALU_ERR_NOT_CONVERGED) rc = NALU_OK;
    }
    ctx->launches++;
    total_it += its;
    if (rc && rc != NALU_ERR_NOT_CONVERGED) break;
    res = true_residual(ctx, ctx->d_x.p, s.tmp.p) / bref;
    if (rc == NALU_ERR_NOT_CONVERGED) break;
  }
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  info->iterations = total_it + probe_its;
  info->outer_iterations = outer;
  info->fallback = probe_chose_jacobi ? 2 : (fallback ? 1 : 0);
  info->learned_iterations = learned_its;
  info->setup_seconds = setup_s;
  info->probe_rate_jacobi = probe_rj;
  info->probe_rate_learned = probe_rl;
  info->true_rel_res = res;
  info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rc == NALU_OK && res > o.tol) rc = set_error(ctx, NALU_ERR_NOT_CONVERGED, "tolerance not reached");
  if (rc == NALU_ERR_NOT_CONVERGED && ctx->last_error.empty()) ctx->last_error = "max iterations";
  info->status = rc;
  return rc;
}

}  // namespace nalu_gb300

// ---------------------------------------------------------------------------
// Jacobi-PCG that allocates no device memory: nalu_pcg_jacobi_noalloc.
//
// Its scratch (residual, preconditioned residual, search direction, A*p,
// inverse diagonal, block partial sums, device scalars and the identity-row
// mask) lives in one file-scope device array of fixed size, sized for
// kNoAllocMaxRows rows.  Every GPU that loads this library holds the array
// (about 10.8 MB) until the process exits.  Host code cannot use the array's
// name as a device address, so the first call on each device, with that
// device current, looks its address up with cudaGetSymbolAddress and caches
// it.  All calls on a device share the array, so calls whose work overlaps on
// the GPU (different streams, or different host threads) race on it.
// ---------------------------------------------------------------------------
namespace nalu_gb300 {
namespace {
constexpr int64_t kNoAllocMaxRows = 262144;
constexpr int64_t kNoAllocScalars = 16;
constexpr int64_t kNoAllocDoubles = 5 * kNoAllocMaxRows + 2 * kRedBlocks + kNoAllocScalars;
constexpr int64_t kNoAllocMaskDoubles = kNoAllocMaxRows / 8;  // one byte per row
constexpr int kNoAllocMaxDevices = 64;
}  // namespace

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles + kNoAllocMaskDoubles];

namespace {
std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// device address of the scratch array on the current device (looked up once)
cudaError_t noalloc_scratch(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[device]) {
    double* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[device] = p;
  }
  *out = g_noalloc_ptr[device];
  return cudaSuccess;
}

double read_scalar_on(cudaStream_t s, const double* d, cudaError_t* err) {
  double h = 0.0;
  *err = cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (*err == cudaSuccess) *err = cudaStreamSynchronize(s);
  return h;
}

// scalar slot counting the iterations that moved the iterate (alpha taken
// while the recurrence residual was still above the stop threshold)
constexpr int S_NA_ITS = 10;

__global__ void k_alpha_counted(double* scal) {
  if (!cg_frozen(scal)) scal[S_NA_ITS] += 1.0;
  k_alpha_body(scal);
}

template <int TPR>
void noalloc_cg_chunk(cudaStream_t s, int64_t n, const int64_t* rp, const int32_t* ci, const double* v, double* x,
                      double* r, double* z, double* p, double* q, const double* dinv, double* partial, double* scal,
                      int iters) {
  const unsigned g = grid_for(n, kRedThreads);
  for (int it = 0; it < iters; ++it) {
    k_spmv<double, double, TPR, true><<<kRedBlocks, 256, 0, s>>>(n, rp, ci, v, p, q, partial);
    k_finish<<<1, 256, 0, s>>>(partial, kRedBlocks, 1, scal, S_PQ);
    k_alpha_counted<<<1, 1, 0, s>>>(scal);
    k_cg_update<double><<<g, kRedThreads, 0, s>>>(n, scal, x, p, r, q, z, dinv, partial, 1);
    k_finish<<<1, 256, 0, s>>>(partial, g, 2, scal, S_RZNEW);
    k_beta<<<1, 1, 0, s>>>(scal);
    k_p_update<double><<<g, kRedThreads, 0, s>>>(n, scal, z, p);
  }
}
}  // namespace

}  // namespace nalu_gb300

extern "C" int nalu_pcg_jacobi_noalloc(int64_t n, const int64_t* rowptr, const int32_t* colind, const double* values,
                                       const double* rhs, double* x, double tol, int max_iters, int* iterations,
                                       double* true_rel_res, void* stream) {
  using namespace nalu_gb300;
  if (n <= 0 || !rowptr || !colind || !values || !rhs || !x || !(tol > 0.0) || max_iters <= 0) return NALU_ERR_ARG;
  if (n > kNoAllocMaxRows) return NALU_ERR_CAPACITY;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kNoAllocMaxDevices) return NALU_ERR_NO_DEVICE;
  double* base = nullptr;
  if (noalloc_scratch(device, &base) != cudaSuccess) return NALU_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t M = kNoAllocMaxRows;
  double *r = base, *z = base + M, *p = base + 2 * M, *q = base + 3 * M, *dinv = base + 4 * M;
  double* partial = base + 5 * M;
  double* scal = partial + 2 * kRedBlocks;
  uint8_t* mask = reinterpret_cast<uint8_t*>(base + kNoAllocDoubles);
  cudaError_t err = cudaMemsetAsync(scal, 0, sizeof(double) * kNoAllocScalars, s);
  if (err != cudaSuccess) return NALU_ERR_CUDA;
  const unsigned g256 = (unsigned)((n + 255) / 256);
  const unsigned g = grid_for(n, kRedThreads);
  k_dinv<double, double><<<g256, 256, 0, s>>>(n, rowptr, colind, values, dinv, mask);
  k_init_x<<<g256, 256, 0, s>>>(n, x, rhs, mask, 1);
  k_multi_dot<double><<<g, kRedThreads, 0, s>>>(n, 1, rhs, rhs, partial, nullptr, nullptr);
  k_finish<<<1, 256, 0, s>>>(partial, g, 1, scal, S_BB);
  if ((err = cudaGetLastError()) != cudaSuccess) return NALU_ERR_CUDA;
  int64_t nnz = 0;
  if ((err = cudaMemcpyAsync(&nnz, rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return NALU_ERR_CUDA;
  const double bnorm = std::sqrt(read_scalar_on(s, scal + S_BB, &err));
  if (err != cudaSuccess) return NALU_ERR_CUDA;
  const bool wide = nnz > 40 * n;  // 3-dof rows (81 entries) use 16 threads per row
  const double bref = bnorm > 0 ? bnorm : 1.0;
  int total = 0;  // iterations issued (whole chunks); the reported count comes from the device
  double res = 0.0;
  int status = NALU_OK;
  for (int outer = 0; outer < 8; ++outer) {
    k_residual<<<kRedBlocks, 256, 0, s>>>(n, rowptr, colind, values, x, rhs, r, partial);
    k_finish<<<1, 256, 0, s>>>(partial, kRedBlocks, 1, scal, S_TMP);
    if ((err = cudaGetLastError()) != cudaSuccess) return NALU_ERR_CUDA;
    const double r0sq = read_scalar_on(s, scal + S_TMP, &err);
    if (err != cudaSuccess) return NALU_ERR_CUDA;
    const double r0 = std::sqrt(r0sq);
    res = r0 / bref;
    if (res <= tol || total >= max_iters) break;
    const double stop = std::max(tol * bref * 0.5, 1e-15 * r0);
    // seed the recurrence residual and the stop threshold: once r.r falls to
    // stop^2 inside a chunk, alpha = beta = 0 freeze the iterate (an exactly
    // converged residual would otherwise give p.Ap = 0 and 0/0)
    const double seed[2] = {r0sq, stop * stop};
    k_copy_scale<double><<<g256, 256, 0, s>>>(n, r, z, nullptr, dinv);
    if ((err = cudaMemcpyAsync(p, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
      return NALU_ERR_CUDA;
    if ((err = cudaMemcpyAsync(scal + S_RR, &seed[0], sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return NALU_ERR_CUDA;
    if ((err = cudaMemcpyAsync(scal + S_STOP, &seed[1], sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return NALU_ERR_CUDA;
    k_multi_dot<double><<<g, kRedThreads, 0, s>>>(n, 1, r, z, partial, nullptr, nullptr);
    k_finish<<<1, 256, 0, s>>>(partial, g, 1, scal, S_RZ);
    while (total < max_iters) {
      const int chunk = std::min(25, max_iters - total);
      if (wide) noalloc_cg_chunk<16>(s, n, rowptr, colind, values, x, r, z, p, q, dinv, partial, scal, chunk);
      else noalloc_cg_chunk<8>(s, n, rowptr, colind, values, x, r, z, p, q, dinv, partial, scal, chunk);
      if ((err = cudaGetLastError()) != cudaSuccess) return NALU_ERR_CUDA;
      total += chunk;
      const double rr = read_scalar_on(s, scal + S_RR, &err);
      if (err != cudaSuccess) return NALU_ERR_CUDA;
      const double bad = read_scalar_on(s, scal + S_BAD, &err);
      if (err != cudaSuccess) return NALU_ERR_CUDA;
      if (bad != 0.0 || !std::isfinite(rr)) {
        status = NALU_ERR_NONFINITE;
        break;
      }
      if (std::sqrt(rr) <= stop) break;
    }
    if (status != NALU_OK) break;
  }
  k_residual<<<kRedBlocks, 256, 0, s>>>(n, rowptr, colind, values, x, rhs, r, partial);
  k_finish<<<1, 256, 0, s>>>(partial, kRedBlocks, 1, scal, S_TMP);
  if ((err = cudaGetLastError()) != cudaSuccess) return NALU_ERR_CUDA;
  res = std::sqrt(read_scalar_on(s, scal + S_TMP, &err)) / bref;
  if (err != cudaSuccess) return NALU_ERR_CUDA;
  const double its = read_scalar_on(s, scal + S_NA_ITS, &err);
  if (err != cudaSuccess) return NALU_ERR_CUDA;
  if (iterations) *iterations = (int)its;
  if (true_rel_res) *true_rel_res = res;
  if (status != NALU_OK) return status;
  return res <= tol ? NALU_OK : NALU_ERR_NOT_CONVERGED;
}
