// train_tc.cu -- the learned preconditioner's training step fused into two
// launches on the BF16 tensor cores (mma.sync m16n8k16, FP32 accumulation),
// with FP32 master weights and Adam.
//
//   k_train_step   one warp per sample, four samples per block (128 rows: the
//                  27 impulse slots of each sample and 5 zero rows).  The FP32
//                  weights arrive in shared memory by 16-byte async copies
//                  (cp.async, all in flight at once) and are converted there.
//                  Forward:
//                  the static part of layer 1 in FP32, layers 2 and 3 on the
//                  tensor cores with the activations in registers (the
//                  accumulators of one layer are the A fragments of the next),
//                  then output, prediction and squared error by warp shuffles.
//                  Backward: dZ3 in registers; dH2 = dZ3 W3 and dH1 = dZ2 W2 on
//                  the tensor cores against a transposed BF16 copy of W3, W2 in
//                  shared memory; the weight gradients dW3 = dZ3^T H2 and
//                  dW2 = dZ2^T H1 as block-wide MMAs over the 128 rows (the
//                  activations staged transposed in shared memory, each warp
//                  16 output rows); layer 1, the output layer and the biases in
//                  FP32.  Each block writes its partial gradient (no atomics).
//   k_train_adam   sums the block partials in a fixed order (deterministic)
//                  and takes the Adam step on the FP32 master weights.
// An epoch is one CUDA graph of 2 x steps launches.  The FP32 CUDA-core path
// of learned.cu (about twenty launches per step) stays as the exact one.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "internal.h"
#include "learned_mlp.cuh"

namespace nalu_gb300 {
namespace {

constexpr int kTrWarps = 4;                 // samples per block
constexpr int kTrThreads = 32 * kTrWarps;
constexpr int kTrRows = 32 * kTrWarps;      // 27 slots + 5 zero rows per sample
constexpr int kTS = kTrRows + 8;            // BF16 stride of the transposed activations (68 words: no bank conflicts)
constexpr int kW1S = 65;                    // FP32 stride of the layer-1 tables and of dZ1 (odd: no bank conflicts)
constexpr int kPartStride = kNP + 1;        // block partial: gradient, then the sum of squared errors

// shared memory (counts of 4-byte words)
constexpr int kSmW1s = 81 * kW1S;           // static part of W1, [k][o]
constexpr int kSmW1r = 27 * kW1S;           // sqrt27 W1[o][s], [s][o]
constexpr int kSmBB = 4 * 64 + 8;           // b1 | b2 | b3 | w4 | b4
constexpr int kSmZ = kTrWarps * 2048;       // per warp: gelu'(Z2) in fragment order, later dZ1 [27][kW1S]
constexpr int kSmWarp = 84 + 32 + 64 + 4 * 64 + 8;  // per warp: features | rf | hs | 4 vectors | scalars
constexpr int kSmW = 64 * kWStride / 2;     // one BF16 64x64 weight copy
constexpr int kSmT = 64 * kTS / 2;          // one transposed BF16 activation [64][kTS]
constexpr size_t kTrSmem =
    4 * (size_t)(kSmW1s + kSmW1r + kSmBB + kTrWarps * kSmWarp + 4 * kSmW + kSmZ + 3 * kSmT);
constexpr int kStageFloats = OFF_B4;  // P[0, OFF_B4) is staged by 16-byte async copies (b4 is read directly)
static_assert(kTrSmem <= 227 * 1024, "training step shared memory");
static_assert((kSmW1s + kSmW1r + kSmBB + kTrWarps * kSmWarp) % 4 == 0, "16-byte aligned BF16 area");
static_assert(kStageFloats % 4 == 0 && 4 * kStageFloats <= 4 * (kSmZ + 3 * kSmT), "staging area");

__device__ __forceinline__ uint16_t bf16_bits(float x) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  return *reinterpret_cast<const uint16_t*>(&h);
}

// GELU (tanh form) and its derivative from one tanh
__device__ __forceinline__ void gelu_both(float x, float& h, float& dh) {
  const float c = 0.7978845608028654f;
  const float th = tanh_fast(c * fmaf(0.044715f * x, x * x, x));
  h = 0.5f * x * (1.0f + th);
  dh = 0.5f * (1.0f + th) + 0.5f * x * (1.0f - th * th) * c * fmaf(3.0f * 0.044715f, x * x, 1.0f);
}
__device__ __forceinline__ float gelu_grad_fast(float x) {
  float h, d;
  gelu_both(x, h, d);
  return d;
}

// a warp's accumulator tile (rows 0..31 of its sample, 64 columns) stored
// transposed as BF16: T[col][32 warp + row]
__device__ __forceinline__ void store_t(const float (&acc)[2][8][4], uint16_t* T, int warp, int g, int t) {
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int row = 16 * mt + g + 8 * (e >> 1), col = 8 * j + 2 * t + (e & 1);
        T[col * kTS + 32 * warp + row] = bf16_bits(acc[mt][j][e]);
      }
}

// accumulators (final values) into the next layer's A fragments
__device__ __forceinline__ void pack_a(const float (&acc)[2][8][4], uint32_t (&a)[2][4][4]) {
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const float* c0 = acc[mt][2 * kk];
      const float* c1 = acc[mt][2 * kk + 1];
      a[mt][kk][0] = pack_bf16(c0[0], c0[1]);
      a[mt][kk][1] = pack_bf16(c0[2], c0[3]);
      a[mt][kk][2] = pack_bf16(c1[0], c1[1]);
      a[mt][kk][3] = pack_bf16(c1[2], c1[3]);
    }
}

// out[o][i] (64 x 64, row-major) = sum over the block's 128 rows of
// D[row][o] H[row][i], from DT[o][row] and HT[i][row] (BF16, stride kTS);
// warp w computes the rows o in [16 w, 16 w + 16)
__device__ __forceinline__ void block_wgrad(const uint32_t* DT, const uint32_t* HT, float* out, int warp, int g,
                                            int t) {
  constexpr int RS = kTS / 2;
  float c[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.0f;
  const uint32_t* d0 = DT + (16 * warp + g) * RS;
  const uint32_t* d1 = d0 + 8 * RS;
#pragma unroll
  for (int kk = 0; kk < kTrRows / 16; ++kk) {
    const uint32_t a[4] = {d0[8 * kk + t], d1[8 * kk + t], d0[8 * kk + 4 + t], d1[8 * kk + 4 + t]};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t* hb = HT + (8 * j + g) * RS;
      mma_bf16(c[j], a, hb[8 * kk + t], hb[8 * kk + 4 + t]);
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    *reinterpret_cast<float2*>(out + (16 * warp + g) * 64 + 8 * j + 2 * t) = make_float2(c[j][0], c[j][1]);
    *reinterpret_cast<float2*>(out + (16 * warp + g + 8) * 64 + 8 * j + 2 * t) = make_float2(c[j][2], c[j][3]);
  }
}

// sum over g (the 8 lanes that share t)
__device__ __forceinline__ float sum_over_g(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 8);
  v += __shfl_xor_sync(0xffffffffu, v, 16);
  return v;
}

// One step on the samples idx[step * B + b], b < B (step = *epoch x
// steps_per_epoch + k_in_epoch; *epoch taken as 0 when epoch is null).
// Samples b >= nvalid count nothing (the loss and its gradient are means over
// nvalid).  grad = 1: part[block][kPartStride] receives the block's gradient
// and sum of squared errors; grad = 0 (evaluation): part[block] receives the
// sum of squared errors only.
__global__ void __launch_bounds__(kTrThreads, 1)
    k_train_step(const float* __restrict__ P, const float* __restrict__ st, const float* __restrict__ rf,
                 const float* __restrict__ tg, const int32_t* __restrict__ idx, const int* __restrict__ epoch,
                 int k_in_epoch, int steps_per_epoch, int B, int nvalid, int grad, float* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* w1s = reinterpret_cast<float*>(smem);
  float* w1r = w1s + kSmW1s;
  float* bb = w1r + kSmW1r;
  float* wsm = bb + kSmBB;
  uint32_t* w2 = reinterpret_cast<uint32_t*>(wsm + kTrWarps * kSmWarp);
  uint32_t* w3 = w2 + kSmW;
  uint32_t* w2t = w3 + kSmW;
  uint32_t* w3t = w2t + kSmW;
  float* zs = reinterpret_cast<float*>(w3t + kSmW);
  uint32_t* h1t = reinterpret_cast<uint32_t*>(zs + kSmZ);
  uint32_t* h2t = h1t + kSmT;
  uint32_t* dzt = h2t + kSmT;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;

  // the FP32 weights staged into shared memory (zs and the transposed
  // activations, not yet in use) by 16-byte async copies, all in flight at once
  float* stage = zs;
  {
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(stage);
    for (int c = tid; c < kStageFloats / 4; c += kTrThreads)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sbase + 16u * c), "l"(P + 4 * c) : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  // this warp's sample
  float* my = wsm + warp * kSmWarp;
  float* stw = my;         // 81 static features (+3 zero)
  float* rfw = my + 84;    // 27 residual features (+5 zero)
  float* hs = my + 116;    // static part of layer 1
  float* vec = my + 180;   // dW4 | db3 | db2 | dHS
  float* scal = my + 436;  // squared error, db4
  const int b = blockIdx.x * kTrWarps + warp;
  const bool have = b < B;
  const int step = (epoch ? *epoch : 0) * steps_per_epoch + k_in_epoch;
  const int64_t src = have ? idx[(int64_t)step * B + b] : 0;
  for (int k = lane; k < 84; k += 32) stw[k] = (have && k < 81) ? st[src * 81 + k] : 0.0f;
  rfw[lane] = (have && lane < 27) ? rf[src * 27 + lane] : 0.0f;
  const float target = have ? tg[src] : 0.0f;
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  // weights: FP32 layer-1 tables, BF16 W2, W3 ([o][k]) and their transposes
  static_assert(kTrThreads >= 108, "one layer-1 column per thread");
  if (tid < 108) {  // column c = tid of W1[o][c], row by row (no division)
    float* dst = tid < 27 ? w1r + tid * kW1S : w1s + (tid - 27) * kW1S;
    const float sc = tid < 27 ? kSqrt27 : 1.0f;
#pragma unroll 8
    for (int o = 0; o < 64; ++o) dst[o] = sc * stage[OFF_W1 + o * 108 + tid];
  }
  for (int i = tid; i < 64; i += kTrThreads) {
    bb[i] = stage[OFF_B1 + i];
    bb[64 + i] = stage[OFF_B2 + i];
    bb[128 + i] = stage[OFF_B3 + i];
    bb[192 + i] = stage[OFF_W4 + i];
  }
  if (tid == 0) bb[256] = P[OFF_B4];
  {
    uint16_t* w2h = reinterpret_cast<uint16_t*>(w2);
    uint16_t* w3h = reinterpret_cast<uint16_t*>(w3);
    uint16_t* w2th = reinterpret_cast<uint16_t*>(w2t);
    uint16_t* w3th = reinterpret_cast<uint16_t*>(w3t);
    for (int i = tid; i < 64 * 64; i += kTrThreads) {
      const int o = i >> 6, k = i & 63;
      const uint16_t v2 = bf16_bits(stage[OFF_W2 + i]), v3 = bf16_bits(stage[OFF_W3 + i]);
      w2h[o * kWStride + k] = v2;
      w3h[o * kWStride + k] = v3;
      w2th[k * kWStride + o] = v2;
      w3th[k * kWStride + o] = v3;
    }
  }
  __syncthreads();  // the staging area is reused below

  // ---- forward ----
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int o = lane + 32 * h;
    float acc = bb[o];
    for (int k = 0; k < 81; ++k) acc = fmaf(w1s[k * kW1S + o], stw[k], acc);
    hs[o] = acc;
  }
  __syncwarp();
  uint32_t a[2][4][4];
  uint16_t* h1h = reinterpret_cast<uint16_t*>(h1t);
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    const int s0 = 16 * mt + g, s1 = s0 + 8;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const int c0 = 16 * kk + 2 * t;
      const int cols[4] = {c0, c0 + 1, c0 + 8, c0 + 9};
      float x[8];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        x[q] = s0 < 27 ? gelu_fast(hs[cols[q]] + w1r[s0 * kW1S + cols[q]]) : 0.0f;
        x[4 + q] = s1 < 27 ? gelu_fast(hs[cols[q]] + w1r[s1 * kW1S + cols[q]]) : 0.0f;
      }
      a[mt][kk][0] = pack_bf16(x[0], x[1]);
      a[mt][kk][1] = pack_bf16(x[4], x[5]);
      a[mt][kk][2] = pack_bf16(x[2], x[3]);
      a[mt][kk][3] = pack_bf16(x[6], x[7]);
      if (grad) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          h1h[cols[q] * kTS + 32 * warp + s0] = bf16_bits(x[q]);
          h1h[cols[q] * kTS + 32 * warp + s1] = bf16_bits(x[4 + q]);
        }
      }
    }
  }
  float acc[2][8][4];
  mlp_layer(acc, a, w2, bb + 64, g, t);  // Z2
  float* z2w = zs + warp * 2048;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        float hv, dv;
        gelu_both(acc[mt][j][e], hv, dv);
        z2w[((mt * 8 + j) * 4 + e) * 32 + lane] = dv;  // gelu'(Z2), for dZ2 (unused in evaluation)
        acc[mt][j][e] = hv;
      }
  if (grad) store_t(acc, reinterpret_cast<uint16_t*>(h2t), warp, g, t);
  pack_a(acc, a);
  mlp_layer(acc, a, w3, bb + 128, g, t);  // Z3
  // output per row, prediction of the sample, squared error
  float orow[2][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float wa = bb[192 + 8 * j + 2 * t], wb = bb[192 + 8 * j + 2 * t + 1];
      orow[mt][0] = fmaf(gelu_fast(acc[mt][j][0]), wa, fmaf(gelu_fast(acc[mt][j][1]), wb, orow[mt][0]));
      orow[mt][1] = fmaf(gelu_fast(acc[mt][j][2]), wa, fmaf(gelu_fast(acc[mt][j][3]), wb, orow[mt][1]));
    }
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      orow[mt][h] += __shfl_xor_sync(0xffffffffu, orow[mt][h], 1);
      orow[mt][h] += __shfl_xor_sync(0xffffffffu, orow[mt][h], 2);
    }
  const float b4 = bb[256];
  float pp = 0.0f;
  if (t == 0) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int s = 16 * mt + g + 8 * h;
        if (s < 27) pp = fmaf(stw[27 + s] * (orow[mt][h] + b4) * (1.0f / kSqrt27), rfw[s], pp);
      }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) pp += __shfl_xor_sync(0xffffffffu, pp, o);
  const bool valid = have && b < nvalid;
  const float diff = valid ? rfw[13] + pp - target : 0.0f;
  if (lane == 0) scal[0] = diff * diff;

  if (grad) {
    // ---- backward ----
    const float gs = 2.0f * diff / (float)nvalid;
    float dO[2][2];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int s = 16 * mt + g + 8 * h;
        dO[mt][h] = s < 27 ? gs * rfw[s] * stw[27 + s] * (1.0f / kSqrt27) : 0.0f;
      }
    float v1[8][2], v2[8][2];  // dW4 and db3 partials of this lane's columns
#pragma unroll
    for (int j = 0; j < 8; ++j) v1[j][0] = v1[j][1] = v2[j][0] = v2[j][1] = 0.0f;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          float hv, dv;
          gelu_both(acc[mt][j][e], hv, dv);
          const float d = dO[mt][e >> 1];
          v1[j][e & 1] = fmaf(d, hv, v1[j][e & 1]);
          const float dz = d * bb[192 + 8 * j + 2 * t + (e & 1)] * dv;  // dZ3
          acc[mt][j][e] = dz;
          v2[j][e & 1] += dz;
        }
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        v1[j][c] = sum_over_g(v1[j][c]);
        v2[j][c] = sum_over_g(v2[j][c]);
      }
    if (g == 0) {
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          vec[8 * j + 2 * t + c] = v1[j][c];
          vec[64 + 8 * j + 2 * t + c] = v2[j][c];
        }
    }
    float d4 = t == 0 ? (dO[0][0] + dO[0][1]) + (dO[1][0] + dO[1][1]) : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d4 += __shfl_xor_sync(0xffffffffu, d4, o);
    if (lane == 0) scal[1] = d4;
    uint16_t* dzh = reinterpret_cast<uint16_t*>(dzt);
    store_t(acc, dzh, warp, g, t);  // dZ3^T
    pack_a(acc, a);
    mlp_layer(acc, a, w3t, nullptr, g, t);  // dH2 = dZ3 W3
#pragma unroll
    for (int j = 0; j < 8; ++j) v2[j][0] = v2[j][1] = 0.0f;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float dz = acc[mt][j][e] * z2w[((mt * 8 + j) * 4 + e) * 32 + lane];  // dZ2
          acc[mt][j][e] = dz;
          v2[j][e & 1] += dz;
        }
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int c = 0; c < 2; ++c) v2[j][c] = sum_over_g(v2[j][c]);
    if (g == 0) {
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int c = 0; c < 2; ++c) vec[128 + 8 * j + 2 * t + c] = v2[j][c];
    }
    float* out = part + (int64_t)blockIdx.x * kPartStride;
    __syncthreads();  // dZ3^T and H2^T of the four samples
    block_wgrad(dzt, h2t, out + OFF_W3, warp, g, t);
    __syncthreads();  // dzt is rewritten next
    store_t(acc, dzh, warp, g, t);  // dZ2^T
    pack_a(acc, a);
    mlp_layer(acc, a, w2t, nullptr, g, t);  // dH1 = dZ2 W2
    // dZ1 = dH1 gelu'(Z1) on the slot rows, into this warp's Z2 area
    float* d1 = z2w;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int s = 16 * mt + g + 8 * (e >> 1), col = 8 * j + 2 * t + (e & 1);
          if (s < 27) d1[s * kW1S + col] = acc[mt][j][e] * gelu_grad_fast(hs[col] + w1r[s * kW1S + col]);
        }
    __syncwarp();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int o = lane + 32 * h;
      float sum = 0.0f;
      for (int s = 0; s < 27; ++s) sum += d1[s * kW1S + o];
      vec[192 + o] = sum;  // dHS
    }
    __syncthreads();  // dZ2^T, dZ1 and the vectors of the four samples
    block_wgrad(dzt, h1t, out + OFF_W2, warp, g, t);
    // layer 1, output layer and biases: sums over the four samples in order
    if (tid < 108) {  // column c = tid, row by row (coalesced rows of 108)
      const int c = tid;
      float sv[kTrWarps];
#pragma unroll
      for (int w = 0; w < kTrWarps; ++w) sv[w] = c < 27 ? 0.0f : wsm[w * kSmWarp + c - 27];
#pragma unroll 4
      for (int o = 0; o < 64; ++o) {
        float v = 0.0f;
        if (c < 27) {
#pragma unroll
          for (int w = 0; w < kTrWarps; ++w) v += zs[w * 2048 + c * kW1S + o];
          v *= kSqrt27;
        } else {
#pragma unroll
          for (int w = 0; w < kTrWarps; ++w) v = fmaf(wsm[w * kSmWarp + 180 + 192 + o], sv[w], v);
        }
        out[OFF_W1 + o * 108 + c] = v;
      }
    }
    for (int o = tid; o < 64; o += kTrThreads) {
      float s1 = 0.0f, s2 = 0.0f, s3 = 0.0f, s4 = 0.0f;
#pragma unroll
      for (int w = 0; w < kTrWarps; ++w) {
        const float* vw = wsm + w * kSmWarp + 180;
        s4 += vw[o];
        s3 += vw[64 + o];
        s2 += vw[128 + o];
        s1 += vw[192 + o];
      }
      out[OFF_B1 + o] = s1;
      out[OFF_B2 + o] = s2;
      out[OFF_B3 + o] = s3;
      out[OFF_W4 + o] = s4;
    }
  } else {
    __syncthreads();
  }
  if (tid == 0) {
    float l = 0.0f, d4 = 0.0f;
    for (int w = 0; w < kTrWarps; ++w) {
      l += wsm[w * kSmWarp + 436];
      d4 += wsm[w * kSmWarp + 437];
    }
    if (grad) {
      part[(int64_t)blockIdx.x * kPartStride + OFF_B4] = d4;
      part[(int64_t)blockIdx.x * kPartStride + kNP] = l;
    } else {
      part[blockIdx.x] = l;
    }
  }
}

// gradient = sum of the block partials in a fixed order (partial c goes to
// warp c % 8, each warp sums its partials in order, then the eight warp sums
// in order); loss[step] = the mean squared error; with apply, the Adam step
// (beta 0.9 / 0.999, eps 1e-8).  A block covers 32 parameters.
constexpr int kAdamWarps = 8;
__global__ void __launch_bounds__(32 * kAdamWarps)
    k_train_adam(const float* __restrict__ part, int nblk, float* __restrict__ P, float* __restrict__ m,
                 float* __restrict__ v, float* __restrict__ grad_out, float* __restrict__ loss_out,
                 const int* __restrict__ epoch, int k_in_epoch, int steps_per_epoch, int nvalid, float lr, int apply) {
  __shared__ float sh[kAdamWarps][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  float s = 0.0f;
  if (i <= kNP) {
#pragma unroll 4
    for (int c = warp; c < nblk; c += kAdamWarps) s += part[(int64_t)c * kPartStride + i];
  }
  sh[warp][lane] = s;
  __syncthreads();
  if (warp != 0 || i > kNP) return;
  float gsum = 0.0f;
#pragma unroll
  for (int w = 0; w < kAdamWarps; ++w) gsum += sh[w][lane];
  const int step = (epoch ? *epoch : 0) * steps_per_epoch + k_in_epoch;
  if (i == kNP) {
    if (loss_out) loss_out[step] = gsum / (float)nvalid;
    return;
  }
  if (grad_out) grad_out[i] = gsum;
  if (!apply) return;
  const float tt = (float)(step + 1);
  const float mi = 0.9f * m[i] + 0.1f * gsum;
  const float vi = 0.999f * v[i] + 0.001f * gsum * gsum;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.0f - powf(0.9f, tt));
  const float vh = vi / (1.0f - powf(0.999f, tt));
  P[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
}

__global__ void k_epoch_inc(int* e) { *e += 1; }

int set_step_smem(nalu_ctx* ctx) {
  NALU_CUDA(ctx, cudaFuncSetAttribute(k_train_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrSmem));
  return NALU_OK;
}

}  // namespace

int train_tc(nalu_ctx* ctx, const TrainData& d, float* history) {
  LearnedState& L = ctx->learned;
  cudaStream_t st0 = ctx->stream;
  int rc = set_step_smem(ctx);
  if (rc) return rc;
  const int nblk = (d.B + kTrWarps - 1) / kTrWarps;
  const int vblk = (int)((d.n_val + kTrWarps - 1) / kTrWarps);
  DBuf<float> part, vpart, losses;
  DBuf<int> d_epoch;
  NALU_CUDA(ctx, part.alloc((int64_t)nblk * kPartStride));
  NALU_CUDA(ctx, vpart.alloc(std::max(1, vblk)));
  NALU_CUDA(ctx, losses.alloc((int64_t)d.steps_per_epoch * d.epochs));
  NALU_CUDA(ctx, d_epoch.alloc(1));
  NALU_CUDA(ctx, cudaMemsetAsync(d_epoch.p, 0, sizeof(int), st0));
  const unsigned agrid = (unsigned)((kNP + 1 + 31) / 32);
  // one epoch as a graph: (step, Adam) x steps_per_epoch, then epoch += 1
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(st0, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "begin capture");
  for (int k = 0; k < d.steps_per_epoch; ++k) {
    k_train_step<<<nblk, kTrThreads, kTrSmem, st0>>>(L.params.p, d.st, d.rf, d.tg, d.idx, d_epoch.p, k,
                                                     d.steps_per_epoch, d.B, d.B, 1, part.p);
    k_train_adam<<<agrid, 32 * kAdamWarps, 0, st0>>>(part.p, nblk, L.params.p, L.adam_m.p, L.adam_v.p, nullptr, losses.p,
                                         d_epoch.p, k, d.steps_per_epoch, d.B, d.lr, 1);
  }
  k_epoch_inc<<<1, 1, 0, st0>>>(d_epoch.p);
  ce = cudaStreamEndCapture(st0, &graph);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "end capture");
  ce = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return cuda_check(ctx, ce, "instantiate");
  std::vector<float> vl(std::max(1, vblk));
  for (int e = 0; e < d.epochs && rc == NALU_OK; ++e) {
    ce = cudaGraphLaunch(exec, st0);
    if (ce != cudaSuccess) {
      rc = cuda_check(ctx, ce, "train epoch");
      break;
    }
    ctx->launches += 2 * d.steps_per_epoch + 1;
    if (history && d.n_val > 0) {
      k_train_step<<<vblk, kTrThreads, kTrSmem, st0>>>(L.params.p, d.st, d.rf, d.tg, d.vidx, nullptr, 0, 0,
                                                       (int)d.n_val, (int)d.n_val, 0, vpart.p);
      ctx->launches++;
      ce = cudaMemcpyAsync(vl.data(), vpart.p, sizeof(float) * vblk, cudaMemcpyDeviceToHost, st0);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(st0);
      if (ce != cudaSuccess) {
        rc = cuda_check(ctx, ce, "held-out loss");
        break;
      }
      double s = 0.0;
      for (int c = 0; c < vblk; ++c) s += vl[c];
      history[2 * e + 1] = (float)(s / (double)d.n_val);
    } else if (history) {
      history[2 * e + 1] = 0.0f;
    }
  }
  cudaGraphExecDestroy(exec);
  if (rc) return rc;
  if (history) {
    std::vector<float> hl((size_t)d.steps_per_epoch * d.epochs);
    NALU_CUDA(ctx, cudaMemcpyAsync(hl.data(), losses.p, sizeof(float) * hl.size(), cudaMemcpyDeviceToHost, st0));
    NALU_CUDA(ctx, cudaStreamSynchronize(st0));
    for (int e = 0; e < d.epochs; ++e) {
      double m = 0.0;
      for (int k = 0; k < d.steps_per_epoch; ++k) m += hl[(size_t)e * d.steps_per_epoch + k];
      history[2 * e] = (float)(m / d.steps_per_epoch);
    }
  }
  NALU_CUDA(ctx, cudaStreamSynchronize(st0));
  return cuda_check(ctx, cudaGetLastError(), "train (tensor cores)");
}

int gradient_tc(nalu_ctx* ctx, const float* st, const float* rf, const float* tg, const int32_t* idx, int n,
                float* grad_dev, float* loss_dev) {
  int rc = set_step_smem(ctx);
  if (rc) return rc;
  const int nblk = (n + kTrWarps - 1) / kTrWarps;
  DBuf<float> part;
  NALU_CUDA(ctx, part.alloc((int64_t)nblk * kPartStride));
  k_train_step<<<nblk, kTrThreads, kTrSmem, ctx->stream>>>(ctx->learned.params.p, st, rf, tg, idx, nullptr, 0, 0, n,
                                                           n, 1, part.p);
  k_train_adam<<<(unsigned)((kNP + 1 + 31) / 32), 32 * kAdamWarps, 0, ctx->stream>>>(
      part.p, nblk, nullptr, nullptr, nullptr, grad_dev, loss_dev, nullptr, 0, 0, n, 0.0f, 0);
  ctx->launches += 2;
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return cuda_check(ctx, cudaGetLastError(), "gradient (tensor cores)");
}

}  // namespace nalu_gb300
