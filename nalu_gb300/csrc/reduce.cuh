// reduce.cuh -- deterministic block reductions shared by the CG kernels.
#pragma once
#include <cuda_runtime.h>

namespace nalu_gb300 {
namespace red {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum of `n` partials, identical in every block (fixed order), broadcast
__device__ __forceinline__ double block_total(const double* __restrict__ part, int n, double* sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  s = warp_sum_d(s);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = s;
  __syncthreads();
  if (w == 0) {
    double t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    t = warp_sum_d(t);
    if (lane == 0) sh[32] = t;
  }
  __syncthreads();
  const double total = sh[32];
  __syncthreads();
  return total;
}

// block sum of v written to *out by thread 0 (fixed order)
__device__ __forceinline__ void block_store(double v, double* __restrict__ out, double* sh) {
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    t = warp_sum_d(t);
    if (lane == 0) *out = t;
  }
  __syncthreads();
}

}  // namespace red
}  // namespace nalu_gb300

namespace nalu_gb300 {
namespace red {

// sum of v over the block, returned to every thread (fixed order)
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    t = warp_sum_d(t);
    if (lane == 0) sh[32] = t;
  }
  __syncthreads();
  const double total = sh[32];
  __syncthreads();
  return total;
}

// Grid-wide sums of K values without a second kernel: every block stores its
// block sums in part[k * stride + block]; the last block to arrive (atomic
// ticket after a fence) re-reads all partials in a fixed order, so the
// totals are deterministic, and returns true with them in tot[]; the other
// blocks return false.  The last block resets the counter for the next use.
template <int K>
__device__ __forceinline__ bool grid_reduce(const double (&v)[K], double* __restrict__ part, int stride,
                                            unsigned* __restrict__ counter, double (&tot)[K], double* sh) {
  __shared__ unsigned ticket;
#pragma unroll
  for (int k = 0; k < K; ++k) block_store(v[k], part + k * stride + blockIdx.x, sh);
  if (threadIdx.x == 0) {
    __threadfence();
    ticket = atomicAdd(counter, 1u);
  }
  __syncthreads();
  if (ticket != gridDim.x - 1) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += __ldcg(part + k * stride + i);
    tot[k] = block_sum(s, sh);
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

}  // namespace red
}  // namespace nalu_gb300
