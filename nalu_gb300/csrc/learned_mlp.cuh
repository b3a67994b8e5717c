// learned_mlp.cuh -- the learned preconditioner's MLP: parameter layout and
// the warp-level BF16 tensor-core pieces shared by the stencil kernel
// (inference) and the fused training step.
//
// mma.sync m16n8k16 (row.col, BF16 in, FP32 accumulate) fragment layout, with
// g = lane / 4 and t = lane % 4:
//   A 16x16: a0 = A[g][2t..2t+1], a1 = A[g+8][2t..], a2 = A[g][2t+8..], a3 = A[g+8][2t+8..]
//   B 16x8:  b0 = B[2t..2t+1][g], b1 = B[2t+8..2t+9][g]
//   C 16x8:  c0 = C[g][2t], c1 = C[g][2t+1], c2 = C[g+8][2t], c3 = C[g+8][2t+1]
// so the accumulators of n-tiles 2kk and 2kk+1 are exactly the A fragment of
// k-tile kk of the next layer.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/nalu_gb300.h"

namespace nalu_gb300 {

constexpr int kNP = NALU_LEARNED_PARAMS;
constexpr int OFF_W1 = 0;      // [64][108]
constexpr int OFF_B1 = 6912;   // [64]
constexpr int OFF_W2 = 6976;   // [64][64]
constexpr int OFF_B2 = 11072;  // [64]
constexpr int OFF_W3 = 11136;  // [64][64]
constexpr int OFF_B3 = 15232;  // [64]
constexpr int OFF_W4 = 15296;  // [64]
constexpr int OFF_B4 = 15360;  // [1]
static_assert(OFF_B4 + 1 == kNP, "parameter layout");
constexpr int kWStride = 72;   // padded BF16 row stride of W2/W3 in the stencil kernel (conflict-free B loads)
constexpr float kSqrt27 = 5.196152422706632f;

namespace {

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_fast(float x) {
  const float u = 0.7978845608028654f * fmaf(0.044715f * x, x * x, x);
  return 0.5f * x * (1.0f + tanh_fast(u));
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// acc[mt][j] = bias + A[mt] (16 x 64) . W^T  for the 8 n-tiles of 64 outputs
// (no bias when bias is null); W: BF16 [64][kWStride] viewed as u32 (row
// stride kWStride/2)
__device__ __forceinline__ void mlp_layer(float (&acc)[2][8][4], const uint32_t (&a)[2][4][4],
                                          const uint32_t* __restrict__ W, const float* __restrict__ bias, int g,
                                          int t) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float b0 = bias ? bias[8 * j + 2 * t] : 0.0f, b1 = bias ? bias[8 * j + 2 * t + 1] : 0.0f;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      acc[mt][j][0] = b0;
      acc[mt][j][1] = b1;
      acc[mt][j][2] = b0;
      acc[mt][j][3] = b1;
    }
  }
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t* row = W + (8 * j + g) * (kWStride / 2);
      const uint32_t b0 = row[8 * kk + t], b1 = row[8 * kk + 4 + t];
      mma_bf16(acc[0][j], a[0][kk], b0, b1);
      mma_bf16(acc[1][j], a[1][kk], b0, b1);
    }
  }
}

__device__ __forceinline__ void gelu_pack(const float (&acc)[2][8][4], uint32_t (&a)[2][4][4]) {
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const float* c0 = acc[mt][2 * kk];
      const float* c1 = acc[mt][2 * kk + 1];
      a[mt][kk][0] = pack_bf16(gelu_fast(c0[0]), gelu_fast(c0[1]));
      a[mt][kk][1] = pack_bf16(gelu_fast(c0[2]), gelu_fast(c0[3]));
      a[mt][kk][2] = pack_bf16(gelu_fast(c1[0]), gelu_fast(c1[1]));
      a[mt][kk][3] = pack_bf16(gelu_fast(c1[2]), gelu_fast(c1[3]));
    }
}

}  // namespace
}  // namespace nalu_gb300
