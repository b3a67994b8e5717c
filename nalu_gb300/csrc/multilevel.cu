// multilevel.cu -- aggregation multigrid preconditioner for the scalar
// (continuity / heat) systems, in flexible CG, with either damped Jacobi or
// the learned 27-point stencil (learned.cu) as the fine-level smoother.
//
// The reference solves the continuity system with Belos CG and either an
// Ifpack2 Jacobi sweep or MueLu (src/LinearSolverConfig.C:81-96); this is the
// GPU counterpart of the second choice, built around the learned smoother:
//
// Set-up, all on the device:
//   * aggregation: three passes of pairwise handshake matching per level on
//     the strong negative couplings (-a_ij >= 0.25 max_k -a_ik).  A row
//     proposes to the unmatched strong neighbour of highest priority: the
//     edge's symmetric strength -a_ij / sqrt(a_ii a_jj) in half-octave bins,
//     ties within a bin broken by a per-round hash of the edge.  Mutual
//     proposals pair up.  Unmatched rows then join the pair of their strongest
//     matched strong neighbour (at most two per matched row), else stay
//     singletons.  Rows without off-diagonal entries (Dirichlet and pinned
//     rows) are on no coarse level: their rows of P are zero and the
//     smoother alone treats them;
//   * coarse operators: Galerkin A_c = P^T A P for the piecewise-constant P of
//     each pass, one warp per coarse row: the member rows' entries are
//     gathered into shared memory, their distinct coarse columns found with a
//     shared hash set, ranked (ascending column order) and summed in the
//     gathered order, so the coarse matrix is deterministic;
//   * FP32 copies, inverse diagonals, and smoothing weights 4 / (3 lambda_max)
//     from power iteration (of D^-1 A, or of M A for the learned smoother);
//   * the coarsest level (at most 256 rows, 1024 if coarsening stalls) is
//     inverted densely: FP32 Gauss-Jordan with partial pivoting in one block.
// Cycle (FP32 vectors and values): one pre- and one post-smoothing step per
// level; the coarse problem of each level solved by a V-cycle, or, on the
// first `ml_kcycle_levels` coarse levels, by a K-cycle (two flexible CG steps
// preconditioned by the next level's cycle, Notay & Vassilevski 2008).  The
// outer flexible CG runs on FP32-pair vectors with the df64 SpMV (learned.cu);
// the solve judges convergence on the true FP64 residual, as every other here.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "internal.h"

namespace nalu_gb300 {
namespace {

constexpr int kMlThreads = 256;
constexpr int kMlBlocks = 1216;       // 8 blocks per SM: grid of the streaming kernels
constexpr float kStrong = 0.25f;      // strong coupling: -a_ij >= kStrong * max_k -a_ik
constexpr int kMatchRounds = 6;       // handshake rounds per pairwise pass
constexpr int kPassesPerLevel = 3;    // pairwise passes per level
constexpr int kMaxLevels = 12;
constexpr int64_t kCoarsest = 256;    // coarsen until at most this many rows
constexpr int64_t kDenseMax = 1024;   // largest coarsest level inverted densely
constexpr int kMaxAttach = 2;         // unmatched rows a matched row takes into its pair (at most)
constexpr int kTpr = 4;               // threads per row of the CRS kernels

__device__ __forceinline__ uint64_t d2u_bits(double d) { return (uint64_t)__double_as_longlong(d); }
__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t gstride() { return (int64_t)gridDim.x * blockDim.x; }

// ---------------------------------------------------------------------------
// aggregation
// ---------------------------------------------------------------------------
// smax[i] = max_{j != i} -a_ij (0 if none; -1 for an isolated row, one
// without off-diagonal entries), diag[i] = 1 / sqrt|a_ii| (0 for a zero diagonal)
__global__ void k_ml_smax(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                          const double* __restrict__ v, double* __restrict__ smax, double* __restrict__ diag) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    double m = 0.0, d = 0.0;
    bool off = false;
    for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
      if (ci[k] != i) {
        m = fmax(m, -v[k]);
        off = off || v[k] != 0.0;
      } else {
        d = fabs(v[k]);
      }
    }
    smax[i] = off ? m : -1.0;
    diag[i] = d > 0.0 ? rsqrt(d) : 0.0;
  }
}

// floor(2 log2 x) for x > 0, from the exponent and the significand
__device__ __forceinline__ int strength_bin(double x) {
  const uint64_t b = d2u_bits(x);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  const double m = __longlong_as_double((long long)((b & 0x000FFFFFFFFFFFFFull) | (1023ull << 52)));
  return 2 * e + (m >= 1.4142135623730951 ? 1 : 0);
}
// symmetric per-round hash of the edge (i, j) (32-bit mix, murmur3 finaliser)
__device__ __forceinline__ uint32_t edge_hash(int32_t i, int32_t j, int round) {
  uint32_t h = (uint32_t)min(i, j) * 0x9E3779B1u ^ ((uint32_t)max(i, j) + 0x7F4A7C15u) * 0x85EBCA77u;
  h ^= (uint32_t)(round + 1) * 0xC2B2AE3Du;
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}

// choice[i]: the unmatched strong neighbour of highest priority (-1: none).
// Binning the strength is what lets handshakes succeed along chains whose
// couplings change monotonically (the z lines of stretched meshes): with exact
// strengths every row there proposes to the same side and few proposals are
// mutual.
__global__ void k_ml_choose(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            const double* __restrict__ v, const double* __restrict__ smax,
                            const double* __restrict__ diag, const int32_t* __restrict__ partner, int round,
                            int32_t* __restrict__ choice) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    int32_t best = -1;
    if (partner[i] < 0 && smax[i] > 0.0) {
      const double thr = kStrong * smax[i];
      int best_bin = -(1 << 30);
      uint32_t best_h = 0;
      const double isd = diag[i];
      for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
        const int32_t j = ci[k];
        const double w = -v[k];
        if (j == i || partner[j] >= 0 || !(w >= thr)) continue;
        const double dd = isd * diag[j];
        const int bin = dd > 0.0 ? strength_bin(w * dd) : -(1 << 29);
        const uint32_t h = edge_hash((int32_t)i, j, round);
        if (bin > best_bin || (bin == best_bin && (h > best_h || (h == best_h && j < best)))) {
          best_bin = bin;
          best_h = h;
          best = j;
        }
      }
    }
    choice[i] = best;
  }
}

// mutual choices become pairs
__global__ void k_ml_match(int64_t n, const int32_t* __restrict__ choice, int32_t* __restrict__ partner) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const int32_t j = choice[i];
    if (partner[i] < 0 && j >= 0 && choice[j] == (int32_t)i) partner[i] = j;
  }
}

// target[i]: for an unmatched row, its strongest matched strong neighbour
// (-1: none); -1 for matched rows
__global__ void k_ml_target(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            const double* __restrict__ v, const double* __restrict__ smax,
                            const int32_t* __restrict__ partner, int32_t* __restrict__ target) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    int32_t best = -1;
    if (partner[i] < 0 && smax[i] > 0.0) {
      const double thr = kStrong * smax[i];
      double bw = 0.0;
      for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
        const int32_t j = ci[k];
        const double w = -v[k];
        if (j == i || partner[j] < 0 || !(w >= thr)) continue;
        if (w > bw || (w == bw && j < best)) bw = w, best = j;
      }
    }
    target[i] = best;
  }
}

// leader of each row: the smaller row of its pair.  An unmatched row joins
// its target's pair if it is among the first kMaxAttach rows (by index) that
// chose that target -- a deterministic bound on aggregate size (the rows that
// chose j are all in row j's pattern, which is structurally symmetric); else
// it leads itself
__global__ void k_ml_attach(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            const double* __restrict__ smax, const int32_t* __restrict__ partner,
                            const int32_t* __restrict__ target, int32_t* __restrict__ leader) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const int32_t p = partner[i];
    if (p >= 0) {
      leader[i] = min((int32_t)i, p);
      continue;
    }
    if (smax[i] < 0.0) {  // isolated row: on no coarse level
      leader[i] = -1;
      continue;
    }
    const int32_t j = target[i];
    int rank = 0;
    if (j >= 0)
      for (int64_t k = rp[j]; k < rp[j + 1]; ++k) {
        const int32_t c = ci[k];
        rank += (c < (int32_t)i && target[c] == j) ? 1 : 0;
      }
    leader[i] = (j >= 0 && rank < kMaxAttach) ? min(j, partner[j]) : (int32_t)i;
  }
}

__global__ void k_ml_flag_leaders(int64_t n, const int32_t* __restrict__ leader, int32_t* __restrict__ flag) {
  for (int64_t i = gtid(); i < n; i += gstride()) flag[i] = leader[i] == (int32_t)i ? 1 : 0;
}
// agg[i] = compact id of i's leader, -1 for rows on no coarse level
__global__ void k_ml_assign(int64_t n, const int32_t* __restrict__ leader, const int32_t* __restrict__ id,
                            int32_t* __restrict__ agg) {
  for (int64_t i = gtid(); i < n; i += gstride()) agg[i] = leader[i] >= 0 ? id[leader[i]] : -1;
}
// map[i] <- agg[map[i]]: compose the passes of one level
__global__ void k_ml_compose(int64_t n, int32_t* __restrict__ map, const int32_t* __restrict__ agg) {
  for (int64_t i = gtid(); i < n; i += gstride()) map[i] = map[i] >= 0 ? agg[map[i]] : -1;
}
__global__ void k_ml_iota(int64_t n, int32_t* __restrict__ a) {
  for (int64_t i = gtid(); i < n; i += gstride()) a[i] = (int32_t)i;
}
__global__ void k_ml_fill_i32(int64_t n, int32_t* __restrict__ a, int32_t v) {
  for (int64_t i = gtid(); i < n; i += gstride()) a[i] = v;
}
// member offsets of each aggregate from the aggregate ids sorted as unsigned
// (every id in [0, nc) has a member, its leader; excluded rows, id -1, sort last)
__global__ void k_ml_member_ptr(int64_t n, int64_t nc, const uint32_t* __restrict__ sorted_agg,
                                int64_t* __restrict__ mptr) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const int64_t a = min((int64_t)sorted_agg[i], nc);
    if (i == 0)
      for (int64_t c = 0; c <= a; ++c) mptr[c] = 0;
    const int64_t next = i + 1 < n ? min((int64_t)sorted_agg[i + 1], nc) : nc;
    for (int64_t c = a + 1; c <= next; ++c) mptr[c] = i + 1;
  }
}

// ---------------------------------------------------------------------------
// Galerkin coarse matrix, one warp per coarse row.  COUNT: the number of
// distinct columns per row into cnt; else the row (ascending columns) at crp[I].
// ---------------------------------------------------------------------------
// Two capacities: rows of up to 256 gathered entries / 128 distinct columns
// (8 warps per block, 45 KB: the usual case), and a large one (2048 / 512,
// 4 warps per block, 120 KB) run only for a pass whose rows overflow the first.
template <int LIST, int HASH, int UNIQ>
struct GalSmem {
  int key[LIST];
  double val[LIST];
  int hash[HASH];
  int uniq[UNIQ];
};
template <int LIST, int HASH, int UNIQ, int WARPS>
struct GalCfg {
  static constexpr int kList = LIST, kHash = HASH, kUnique = UNIQ, kWarps = WARPS;
  using Smem = GalSmem<LIST, HASH, UNIQ>;
};
using GalSmall = GalCfg<256, 512, 128, 8>;
using GalLarge = GalCfg<2048, 1024, 512, 4>;

template <bool COUNT, class CFG>
__global__ void __launch_bounds__(32 * CFG::kWarps) k_ml_galerkin(
    int64_t nc, const int64_t* __restrict__ mptr, const int32_t* __restrict__ mem, const int64_t* __restrict__ rp,
    const int32_t* __restrict__ ci, const double* __restrict__ v, const int32_t* __restrict__ agg,
    const int64_t* __restrict__ crp, int64_t* __restrict__ cnt, int32_t* __restrict__ cci, double* __restrict__ cv,
    int* __restrict__ overflow) {
  constexpr int kGalWarps = CFG::kWarps, kGalList = CFG::kList, kGalHash = CFG::kHash, kGalUnique = CFG::kUnique;
  extern __shared__ unsigned char smraw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  typename CFG::Smem& S = reinterpret_cast<typename CFG::Smem*>(smraw)[w];
  const int64_t warps = (int64_t)gridDim.x * kGalWarps;
  for (int64_t I = (int64_t)blockIdx.x * kGalWarps + w; I < nc; I += warps) {
    // the member rows' entries, as coarse columns, in member then entry order
    int L = 0;
    bool over = false;
    for (int64_t m = mptr[I]; m < mptr[I + 1]; ++m) {
      const int32_t i = mem[m];
      const int64_t b = rp[i];
      const int len = (int)(rp[i + 1] - b);
      if (L + len > kGalList) {
        over = true;
        break;
      }
      for (int k = lane; k < len; k += 32) {
        S.key[L + k] = agg[ci[b + k]];  // -1: a column on no coarse level (dropped)
        S.val[L + k] = v[b + k];
      }
      L += len;
    }
    // hash set of the row's size: a power of two >= 2 L (at least 64 slots),
    // so short rows clear and scan few slots
    const int hbits = max(6, 32 - __clz(max(2 * L - 1, 1)));
    const int hsize = min(1 << hbits, kGalHash);
    const int hshift = 32 - __ffs(hsize) + 1;  // top log2(hsize) bits of the product
    for (int h = lane; h < hsize; h += 32) S.hash[h] = -1;
    __syncwarp();
    // distinct keys into the hash set (bounded linear probing)
    for (int p = lane; p < L; p += 32) {
      const int key = S.key[p];
      if (key < 0) continue;
      int h = (int)(((unsigned)key * 2654435761u) >> hshift) & (hsize - 1);
      for (int probe = 0; probe < hsize; ++probe) {
        const int prev = atomicCAS(&S.hash[h], -1, key);
        if (prev == -1 || prev == key) break;
        h = (h + 1) & (hsize - 1);
      }
    }
    __syncwarp();
    int U = 0;
    for (int h0 = 0; h0 < hsize; h0 += 32) {
      const int key = S.hash[h0 + lane];
      const unsigned has = __ballot_sync(0xffffffffu, key >= 0);
      const int pos = U + __popc(has & ((1u << lane) - 1u));
      if (key >= 0 && pos < kGalUnique) S.uniq[pos] = key;
      U += __popc(has);
    }
    __syncwarp();
    if (U > kGalUnique) over = true;
    if (over) {
      if (lane == 0) {
        atomicAdd(overflow, 1);
        if (COUNT) cnt[I] = 0;
      }
      __syncwarp();
      continue;
    }
    if (COUNT) {
      if (lane == 0) cnt[I] = U;
    } else {
      const int64_t base = crp[I];
      for (int u = lane; u < U; u += 32) {
        const int key = S.uniq[u];
        int rank = 0;
        for (int q = 0; q < U; ++q) rank += S.uniq[q] < key ? 1 : 0;
        double sum = 0.0;
        for (int p = 0; p < L; ++p)
          if (S.key[p] == key) sum += S.val[p];
        cci[base + rank] = key;
        cv[base + rank] = sum;
      }
    }
    __syncwarp();
  }
}

// FP32 values and inverse diagonal of a level
__global__ void k_ml_prep(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                          const double* __restrict__ vd, float* __restrict__ vf, float* __restrict__ dinv) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    double d = 0.0;
    for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
      vf[k] = (float)vd[k];
      if (ci[k] == i) d = vd[k];
    }
    dinv[i] = d != 0.0 ? (float)(1.0 / d) : 0.0f;
  }
}

// learned smoother values from A's SELL-32 layout (entry k of row i at
// sptr[i / 32] + 32 k + i % 32, in the row's CRS order) to CRS order
__global__ void k_ml_sell_to_crs(int64_t n, const int64_t* __restrict__ rp, const int64_t* __restrict__ sptr,
                                 const float* __restrict__ ws, float* __restrict__ m) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const int64_t base = sptr[i / 32] + (i % 32);
    const int64_t b = rp[i], len = rp[i + 1] - b;
    for (int64_t k = 0; k < len; ++k) m[b + k] = ws[base + 32 * k];
  }
}

// ---------------------------------------------------------------------------
// cycle kernels (FP32), kTpr threads per row.  The row loop runs the same
// number of times in every lane (rows past n repeat row n-1 and write
// nothing), so the width-kTpr shuffles always see their whole group.
// ---------------------------------------------------------------------------
#define ML_ROW_LOOP(n)                                                                    \
  const int sub = threadIdx.x % kTpr;                                                     \
  const int64_t rstride = (int64_t)gridDim.x * (blockDim.x / kTpr);                       \
  const int64_t rend = (n) + (rstride - (n) % rstride) % rstride;                         \
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kTpr; i < rend; i += rstride)

__device__ __forceinline__ float row_dot(const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                         const float* __restrict__ v, const float* __restrict__ x, int64_t i,
                                         int sub) {
  float s = 0.0f;
  for (int64_t k = rp[i] + sub; k < rp[i + 1]; k += kTpr) s = fmaf(__ldg(v + k), __ldg(x + ci[k]), s);
#pragma unroll
  for (int o = kTpr / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kTpr);
  return s;
}

// t = b - A x
__global__ void __launch_bounds__(kMlThreads) k_ml_residual(int64_t n, const int64_t* __restrict__ rp,
                                                            const int32_t* __restrict__ ci,
                                                            const float* __restrict__ v, const float* __restrict__ x,
                                                            const float* __restrict__ b, float* __restrict__ t) {
  ML_ROW_LOOP(n) {
    const int64_t r = i < n ? i : n - 1;
    const float ax = row_dot(rp, ci, v, x, r, sub);
    if (i < n && sub == 0) t[i] = b[i] - ax;
  }
}

// damped Jacobi from zero fused with the residual: z = w D^-1 b; t = b - A z
__global__ void __launch_bounds__(kMlThreads) k_ml_jac0_residual(int64_t n, const int64_t* __restrict__ rp,
                                                                 const int32_t* __restrict__ ci,
                                                                 const float* __restrict__ v,
                                                                 const float* __restrict__ dinv, float omega,
                                                                 const float* __restrict__ b, float* __restrict__ z,
                                                                 float* __restrict__ t) {
  ML_ROW_LOOP(n) {
    const int64_t r = i < n ? i : n - 1;
    float s = 0.0f;
    for (int64_t k = rp[r] + sub; k < rp[r + 1]; k += kTpr) {
      const int32_t j = ci[k];
      s = fmaf(__ldg(v + k), omega * __ldg(dinv + j) * __ldg(b + j), s);
    }
#pragma unroll
    for (int o = kTpr / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kTpr);
    if (i < n && sub == 0) {
      z[i] = omega * dinv[i] * b[i];
      t[i] = b[i] - s;
    }
  }
}

// damped Jacobi step fused with the residual: zo = z + w D^-1 (b - A z)
__global__ void __launch_bounds__(kMlThreads) k_ml_jac_step(int64_t n, const int64_t* __restrict__ rp,
                                                            const int32_t* __restrict__ ci,
                                                            const float* __restrict__ v,
                                                            const float* __restrict__ dinv, float omega,
                                                            const float* __restrict__ b, const float* __restrict__ z,
                                                            float* __restrict__ zo) {
  ML_ROW_LOOP(n) {
    const int64_t r = i < n ? i : n - 1;
    const float ax = row_dot(rp, ci, v, z, r, sub);
    if (i < n && sub == 0) zo[i] = z[i] + omega * dinv[i] * (b[i] - ax);
  }
}

// learned smoother step: zo = (z or 0) + w M t
__global__ void __launch_bounds__(kMlThreads) k_ml_mstep(int64_t n, const int64_t* __restrict__ rp,
                                                         const int32_t* __restrict__ ci, const float* __restrict__ m,
                                                         float omega, const float* __restrict__ t,
                                                         const float* __restrict__ z, float* __restrict__ zo) {
  ML_ROW_LOOP(n) {
    const int64_t r = i < n ? i : n - 1;
    const float mt = row_dot(rp, ci, m, t, r, sub);
    if (i < n && sub == 0) zo[i] = (z ? z[i] : 0.0f) + omega * mt;
  }
}

// ---- fine-level cycle kernels on A's SELL-32 copy (one thread per row;
// entry k of row i at ptr[i / 32] + 32 k + i % 32; padding entries carry a zero
// value; 16-bit column offsets from per-slice bases unless the slice is wide) --
template <bool WIDE, class XGet>
__device__ __forceinline__ float sell_row_f_impl(const SellMatrix::View& S, const float* __restrict__ val,
                                                 int64_t base, int len, const int32_t* __restrict__ cb, XGet x) {
  float acc = 0.0f;
  for (int k = 0; k < len; k += 8) {  // loads of a group issued before the gathers
    int32_t c[8];
    float a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool in = k + u < len;
      const int64_t e = base + (int64_t)(k + u) * 32;
      c[u] = in ? (WIDE ? __ldg(S.col + e) : __ldg(cb + k + u) + (int32_t)__ldg(S.col16 + e)) : -1;
      a[u] = in ? __ldg(val + e) : 0.0f;
    }
    float b[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) b[u] = c[u] >= 0 ? x(c[u]) : 0.0f;
#pragma unroll
    for (int u = 0; u < 8; ++u) acc = fmaf(a[u], b[u], acc);
  }
  return acc;
}
// the wide / 16-bit column choice is made once per row, so each path keeps
// its group of loads ahead of the gathers
template <class XGet>
__device__ __forceinline__ float sell_row_f(const SellMatrix::View& S, const float* __restrict__ val, int64_t row,
                                            XGet x) {
  const int64_t s = row >> 5;
  const int64_t b0 = __ldg(S.ptr + s);
  const int len = __ldg(S.len + s);
  const int64_t base = b0 + (row & 31);
  const int32_t* cb = S.cbase + (b0 >> 5);
  return __ldg(S.wide + s) ? sell_row_f_impl<true>(S, val, base, len, cb, x)
                           : sell_row_f_impl<false>(S, val, base, len, cb, x);
}
// z = w D^-1 b; t = b - A z
__global__ void __launch_bounds__(kMlThreads) k_ml0_jac0_residual(int64_t n, SellMatrix::View S,
                                                                  const float* __restrict__ val,
                                                                  const float* __restrict__ dinv, float omega,
                                                                  const float* __restrict__ b, float* __restrict__ z,
                                                                  float* __restrict__ t) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const float az = sell_row_f(S, val, i, [&](int32_t c) { return omega * __ldg(dinv + c) * __ldg(b + c); });
    z[i] = omega * dinv[i] * b[i];
    t[i] = b[i] - az;
  }
}
// zo = z + w D^-1 (b - A z)
__global__ void __launch_bounds__(kMlThreads) k_ml0_jac_step(int64_t n, SellMatrix::View S,
                                                             const float* __restrict__ val,
                                                             const float* __restrict__ dinv, float omega,
                                                             const float* __restrict__ b, const float* __restrict__ z,
                                                             float* __restrict__ zo) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const float az = sell_row_f(S, val, i, [&](int32_t c) { return __ldg(z + c); });
    zo[i] = z[i] + omega * dinv[i] * (b[i] - az);
  }
}
// t = b - A x
__global__ void __launch_bounds__(kMlThreads) k_ml0_residual(int64_t n, SellMatrix::View S,
                                                             const float* __restrict__ val, const float* __restrict__ x,
                                                             const float* __restrict__ b, float* __restrict__ t) {
  for (int64_t i = gtid(); i < n; i += gstride())
    t[i] = b[i] - sell_row_f(S, val, i, [&](int32_t c) { return __ldg(x + c); });
}
// zo = (z or 0) + w M t, M on the same SELL pattern
__global__ void __launch_bounds__(kMlThreads) k_ml0_mstep(int64_t n, SellMatrix::View S, const float* __restrict__ m,
                                                          float omega, const float* __restrict__ t,
                                                          const float* __restrict__ z, float* __restrict__ zo) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const float mt = sell_row_f(S, m, i, [&](int32_t c) { return __ldg(t + c); });
    zo[i] = (z ? z[i] : 0.0f) + omega * mt;
  }
}
// FP32 SELL values: the high words of the FP32-pair copy
__global__ void k_ml0_sell_f32(int64_t stored, const float2* __restrict__ v2, float* __restrict__ vf) {
  for (int64_t e = gtid(); e < stored; e += gstride()) vf[e] = v2[e].x;
}

// restriction rc[I] = sum of t over the members of I (member order)
__global__ void k_ml_restrict(int64_t nc, const int64_t* __restrict__ mptr, const int32_t* __restrict__ mem,
                              const float* __restrict__ t, float* __restrict__ rc) {
  for (int64_t I = gtid(); I < nc; I += gstride()) {
    float s = 0.0f;
    for (int64_t m = mptr[I]; m < mptr[I + 1]; ++m) s += t[mem[m]];
    rc[I] = s;
  }
}

// prolongation z[i] += e[agg[i]]
__global__ void k_ml_prolong(int64_t n, const int32_t* __restrict__ agg, const float* __restrict__ e,
                             float* __restrict__ z) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    const int32_t a = agg[i];
    if (a >= 0) z[i] += e[a];
  }
}

// ---- deterministic dot products: block partials, the last block finishes ---
__device__ __forceinline__ double ml_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// NP block sums of vals[] into partial[p * gridDim + block]; the last block to
// arrive (ticket after a fence) sums every column in block order into out[p]
// and resets the ticket
template <int NP>
__device__ __forceinline__ void ml_reduce(double (&vals)[NP], double* __restrict__ partial,
                                          unsigned* __restrict__ counter, double* __restrict__ out) {
  __shared__ double sh[NP][32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const double s = ml_warp_sum(vals[p]);
    if (lane == 0) sh[p][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const double s = ml_warp_sum(lane < nw ? sh[p][lane] : 0.0);
      if (lane == 0) partial[p * gridDim.x + blockIdx.x] = s;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    double s = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) s += partial[p * gridDim.x + b];
    s = ml_warp_sum(s);
    if (lane == 0) sh[p][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const double s = ml_warp_sum(lane < nw ? sh[p][lane] : 0.0);
      if (lane == 0) out[p] = s;
    }
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// ---- K-cycle at one coarse level (device scalars ks[0..4]) ------------------
// y = A x; out[0] = x . y, out[1] = x . r (and out[2] = x . w1 when W1)
template <bool W1>
__global__ void __launch_bounds__(kMlThreads) k_ml_kspmv(int64_t n, const int64_t* __restrict__ rp,
                                                         const int32_t* __restrict__ ci, const float* __restrict__ a,
                                                         const float* __restrict__ x, float* __restrict__ y,
                                                         const float* __restrict__ r, const float* __restrict__ w1,
                                                         double* __restrict__ partial, unsigned* __restrict__ counter,
                                                         double* __restrict__ out) {
  constexpr int NP = W1 ? 3 : 2;
  double acc[NP] = {};
  ML_ROW_LOOP(n) {
    const int64_t rr = i < n ? i : n - 1;
    const float ax = row_dot(rp, ci, a, x, rr, sub);
    if (i < n && sub == 0) {
      y[i] = ax;
      const double xi = x[i];
      acc[0] += xi * ax;
      acc[1] += xi * r[i];
      if (W1) acc[NP - 1] += xi * w1[i];
    }
  }
  ml_reduce<NP>(acc, partial, counter, out);
}

// rt = r - (alpha1 / rho1) w1 (no step when rho1 is not positive)
__global__ void k_ml_kstep1(int64_t n, const double* __restrict__ ks, const float* __restrict__ r,
                            const float* __restrict__ w1, float* __restrict__ rt) {
  const double rho1 = ks[0];
  const float a = rho1 > 0.0 && isfinite(rho1) ? (float)(ks[1] / rho1) : 0.0f;
  for (int64_t i = gtid(); i < n; i += gstride()) rt[i] = r[i] - a * w1[i];
}
// e = c1 v1 + c2 v2: rho1 = ks[0], alpha1 = ks[1], beta = ks[2] (v2.w2),
// alpha2 = ks[3] (v2.rt), gamma = ks[4] (v2.w1)
__global__ void k_ml_kcombine(int64_t n, const double* __restrict__ ks, const float* __restrict__ v1,
                              const float* __restrict__ v2, float* __restrict__ e) {
  const double rho1 = ks[0], a1 = ks[1], beta = ks[2], a2 = ks[3], gam = ks[4];
  double c1 = 0.0, c2 = 0.0;
  if (rho1 > 0.0 && isfinite(rho1)) {
    c1 = a1 / rho1;
    const double rho2 = beta - gam * gam / rho1;
    if (rho2 > 1e-12 * beta && isfinite(rho2)) {
      c2 = a2 / rho2;
      c1 -= gam * a2 / (rho1 * rho2);
    }
  }
  const float f1 = (float)c1, f2 = (float)c2;
  for (int64_t i = gtid(); i < n; i += gstride()) e[i] = f1 * v1[i] + f2 * v2[i];
}

// ---- independent problems (a batch's union system) --------------------------
// Rows of a problem that is already at or below the coarsest size get no
// strong neighbour: they stay singletons, and the problem keeps its size on
// the next levels while larger ones coarsen on.  off [P+1]: the problems' row
// ranges on this level.
__global__ void k_ml_freeze(int64_t n, const int64_t* __restrict__ off, int P, int64_t target,
                            double* __restrict__ smax) {
  for (int64_t i = gtid(); i < n; i += gstride()) {
    int lo = 0, hi = P;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (off[mid] <= i) lo = mid;
      else hi = mid;
    }
    if (off[lo + 1] - off[lo] <= target && smax[i] > 0.0) smax[i] = 0.0;
  }
}
// the problems' row ranges on the next level: the leaders before each range
// (coarse rows are numbered in the order of their leaders)
__global__ void k_ml_next_offsets(int P, const int64_t* __restrict__ off, const int32_t* __restrict__ id,
                                  int64_t* __restrict__ out) {
  for (int64_t p = gtid(); p <= P; p += gstride()) out[p] = id[off[p]];
}

// ---- coarsest level: dense inverse (FP32 Gauss-Jordan, one block) -----------
// D [n][2n] row-major: the matrix and the identity beside it
__global__ void k_ml_dense_fill(int n, float* __restrict__ D) {
  for (int64_t t = gtid(); t < (int64_t)n * 2 * n; t += gstride()) {
    const int i = (int)(t / (2 * n)), j = (int)(t % (2 * n));
    D[t] = j >= n ? (j - n == i ? 1.0f : 0.0f) : 0.0f;
  }
}
__global__ void k_ml_dense_scatter(int n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                   const double* __restrict__ v, float* __restrict__ D) {
  for (int64_t i = gtid(); i < n; i += gstride())
    for (int64_t k = rp[i]; k < rp[i + 1]; ++k) D[i * 2 * n + ci[k]] += (float)v[k];
}
// [A | I] -> [I | A^-1] with partial pivoting, by the whole block; a zero
// pivot sets *bad
__device__ void gauss_jordan_block(int n, float* __restrict__ D, int* __restrict__ bad) {
  __shared__ float bv[32];
  __shared__ int bi[32];
  __shared__ int piv;
  __shared__ float pinv;
  const int m = 2 * n;
  for (int k = 0; k < n; ++k) {
    float best = -1.0f;
    int bidx = k;
    for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
      const float a = fabsf(D[(int64_t)i * m + k]);
      if (a > best) best = a, bidx = i;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
      if (ob > best || (ob == best && oi < bidx)) best = ob, bidx = oi;
    }
    if ((threadIdx.x & 31) == 0) bv[threadIdx.x >> 5] = best, bi[threadIdx.x >> 5] = bidx;
    __syncthreads();
    if (threadIdx.x < 32) {
      best = threadIdx.x < (blockDim.x >> 5) ? bv[threadIdx.x] : -1.0f;
      bidx = threadIdx.x < (blockDim.x >> 5) ? bi[threadIdx.x] : k;
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (ob > best || (ob == best && oi < bidx)) best = ob, bidx = oi;
      }
      if (threadIdx.x == 0) {
        piv = bidx;
        if (!(best > 0.0f)) *bad = 1;
      }
    }
    __syncthreads();
    const int p = piv;
    if (p != k)
      for (int j = threadIdx.x; j < m; j += blockDim.x) {
        const float a = D[(int64_t)k * m + j];
        D[(int64_t)k * m + j] = D[(int64_t)p * m + j];
        D[(int64_t)p * m + j] = a;
      }
    __syncthreads();
    if (threadIdx.x == 0) {
      const float d = D[(int64_t)k * m + k];
      pinv = d != 0.0f ? 1.0f / d : 0.0f;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) D[(int64_t)k * m + j] *= pinv;
    __syncthreads();
    // eliminate column k from every other row (columns left of k are done):
    // one warp per row, lanes along the columns (coalesced, no index division)
    {
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      const float* pk = D + (int64_t)k * m;
      for (int i = warp; i < n; i += nw) {
        if (i == k) continue;
        float* pi = D + (int64_t)i * m;
        const float f = pi[k];
        if (f == 0.0f) continue;
        for (int j = k + 1 + lane; j < m; j += 32) pi[j] -= f * pk[j];
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      if (i != k) D[(int64_t)i * m + k] = 0.0f;
    __syncthreads();
  }
}
__global__ void __launch_bounds__(1024) k_ml_gauss_jordan(int n, float* __restrict__ D, int* __restrict__ bad) {
  gauss_jordan_block(n, D, bad);
}
// one block per diagonal block: block b's [A | I] at D + doff[b], of order
// boff[b+1] - boff[b]
__global__ void __launch_bounds__(1024) k_ml_gauss_jordan_blocks(const int64_t* __restrict__ boff,
                                                                 const int64_t* __restrict__ doff,
                                                                 float* __restrict__ D, int* __restrict__ bad) {
  const int b = blockIdx.x;
  const int n = (int)(boff[b + 1] - boff[b]);
  if (n > 0) gauss_jordan_block(n, D + doff[b], bad);
}
// one diagonal block [b0, b0 + n) of a block-diagonal matrix (rp offset to
// its first row); entries outside the block are not expected and are skipped
__global__ void k_ml_dense_scatter_block(int n, int64_t b0, const int64_t* __restrict__ rp,
                                         const int32_t* __restrict__ ci, const double* __restrict__ v,
                                         float* __restrict__ D) {
  for (int64_t i = gtid(); i < n; i += gstride())
    for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
      const int64_t c = (int64_t)ci[k] - b0;
      if (c >= 0 && c < n) D[i * 2 * n + c] += (float)v[k];
    }
}
// Inv [n][n] <- right half of D
__global__ void k_ml_dense_extract(int n, const float* __restrict__ D, float* __restrict__ Inv) {
  for (int64_t t = gtid(); t < (int64_t)n * n; t += gstride()) {
    const int i = (int)(t / n), j = (int)(t % n);
    Inv[t] = D[(int64_t)i * 2 * n + n + j];
  }
}
// e = Inv r, one warp per row
__global__ void k_ml_dense_apply(int n, const float* __restrict__ Inv, const float* __restrict__ r,
                                 float* __restrict__ e) {
  const int64_t row = gtid() >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  float s = 0.0f;
  for (int j = lane; j < n; j += 32) s = fmaf(Inv[row * n + j], r[j], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) e[row] = s;
}

// e = Inv r for a block-diagonal inverse: row's block brow[row], blocks at
// rows [boff[b], boff[b+1]), their inverses at inv + ioff[b]; one warp per row
__global__ void k_ml_dense_apply_blocks(int64_t n, const int32_t* __restrict__ brow, const int64_t* __restrict__ boff,
                                        const int64_t* __restrict__ ioff, const float* __restrict__ inv,
                                        const float* __restrict__ r, float* __restrict__ e) {
  const int64_t row = gtid() >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const int b = brow[row];
  const int64_t b0 = boff[b], nb = boff[b + 1] - b0;
  const float* I = inv + ioff[b] + (row - b0) * nb;
  float s = 0.0f;
  for (int64_t j = lane; j < nb; j += 32) s = fmaf(I[j], r[b0 + j], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) e[row] = s;
}

// ---- power iteration for the smoothing weight -------------------------------
__global__ void __launch_bounds__(kMlThreads) k_ml_power_ax(int64_t n, const int64_t* __restrict__ rp,
                                                            const int32_t* __restrict__ ci,
                                                            const float* __restrict__ a, const float* __restrict__ x,
                                                            float* __restrict__ t) {
  ML_ROW_LOOP(n) {
    const int64_t r = i < n ? i : n - 1;
    const float ax = row_dot(rp, ci, a, x, r, sub);
    if (i < n && sub == 0) t[i] = ax;
  }
}
// y = S t (S = M, or D^-1 when m is null); out[0] = y . y
__global__ void __launch_bounds__(kMlThreads) k_ml_power_s(int64_t n, const int64_t* __restrict__ rp,
                                                           const int32_t* __restrict__ ci, const float* __restrict__ m,
                                                           const float* __restrict__ dinv, const float* __restrict__ t,
                                                           float* __restrict__ y, double* __restrict__ partial,
                                                           unsigned* __restrict__ counter, double* __restrict__ out) {
  double acc[1] = {0.0};
  ML_ROW_LOOP(n) {
    const int64_t r = i < n ? i : n - 1;
    const float st = m ? row_dot(rp, ci, m, t, r, sub) : dinv[r] * t[r];
    if (i < n && sub == 0) {
      y[i] = st;
      acc[0] += (double)st * st;
    }
  }
  ml_reduce<1>(acc, partial, counter, out);
}
__global__ void k_ml_scale(int64_t n, const double* __restrict__ ks, const float* __restrict__ y,
                           float* __restrict__ x) {
  const double nrm = sqrt(ks[0]);
  const float s = nrm > 0.0 ? (float)(1.0 / nrm) : 0.0f;
  for (int64_t i = gtid(); i < n; i += gstride()) x[i] = s * y[i];
}
// a positive, unit-norm-ish start vector
__global__ void k_ml_seed(int64_t n, float* __restrict__ x) {
  const float s = (float)(1.0 / sqrt((double)n));
  for (int64_t i = gtid(); i < n; i += gstride()) {
    uint32_t h = (uint32_t)i * 2654435761u + 12345u;
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    x[i] = s * (0.5f + (float)(h & 0xffffu) / 65536.0f);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct MlLevel {
  int64_t n = 0, nnz = 0;
  const int64_t* rp = nullptr;
  const int32_t* ci = nullptr;
  const double* vd = nullptr;
  DBuf<int64_t> own_rp;
  DBuf<int32_t> own_ci;
  DBuf<double> own_vd;
  DBuf<float> vf, dinv, msm;  // FP32 values, inverse diagonal, learned smoother (level 0)
  DBuf<int32_t> agg;          // row -> next level's row
  DBuf<int64_t> mptr;         // members of the next level's rows
  DBuf<int32_t> mem;
  DBuf<float> z, t, z2, b;    // cycle vectors
  DBuf<float> v1, v2, w1, w2, rt, e;  // K-cycle vectors (as a coarse level)
  DBuf<float> inv;            // dense inverse (coarsest level)
  float omega = 0.6f;    // smoothing weight (of the learned smoother at level 0 when it is used)
  float omega_j = 0.6f;  // damped-Jacobi weight at level 0 beside the learned smoother
  // level 0: the cycle's SpMVs on A's SELL-32 copy (FP32 values; the learned
  // smoother's values are on the same pattern)
  bool sell = false;
  SellMatrix::View sv{};
  DBuf<float> sellv;
  const float* sellm = nullptr;
};

// set-up temporaries, grown to the largest level and kept between solves
struct MlScratch {
  DBuf<double> smax, diag;
  DBuf<int32_t> partner, choice, leader, target, flag, id, agg, iota, mem;
  DBuf<uint32_t> keys;
  DBuf<int64_t> cnt, mptr;
  DBuf<int> flagd;
  DBuf<unsigned char> cub;
  DBuf<int64_t> rp[2];  // ping-pong coarse matrices of the passes within a level
  DBuf<int32_t> ci[2];
  DBuf<double> v[2];
  DBuf<int64_t> off, off2;  // problems' row ranges on the current level, and the next
};

struct MlState {
  std::vector<MlLevel> lv;
  MlScratch sc;
  DBuf<double> partial, ks;   // reduction partials; device scalars (8 per level)
  DBuf<unsigned> counter;     // reduction tickets
  bool learned = false;
  bool ready = false;
  int klevels = 0;            // coarse levels 1..klevels solved by K-cycle, deeper ones by V-cycle
  int lsweeps = 3;            // learned smoother: pre-smoothing (bit 0), post-smoothing (bit 1); else Jacobi
  // independent problems: the coarsest level's diagonal blocks (one per problem)
  std::vector<int64_t> boff;  // block row ranges [P+1] (one block without problems)
  DBuf<int64_t> boff_d, ioff_d;
  DBuf<int32_t> brow;         // block of each coarsest row
};

namespace {

constexpr int kCounters = 64;

unsigned grid_n(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + kMlThreads - 1) / kMlThreads, kMlBlocks));
}
unsigned grid_rows(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n * kTpr + kMlThreads - 1) / kMlThreads, 4 * kMlBlocks));
}

template <class T>
cudaError_t grow(DBuf<T>& b, int64_t n) {
  return b.n >= n ? cudaSuccess : b.alloc(n);
}

template <class T>
int exclusive_scan(nalu_ctx* ctx, MlScratch& S, const T* in, T* out, int64_t n) {
  size_t tmp = 0;
  NALU_CUDA(ctx, cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, (int)n, ctx->stream));
  NALU_CUDA(ctx, grow(S.cub, (int64_t)tmp + 1));
  NALU_CUDA(ctx, cub::DeviceScan::ExclusiveSum(S.cub.p, tmp, in, out, (int)n, ctx->stream));
  return NALU_OK;
}
template <class T>
T read_one(nalu_ctx* ctx, const T* d) {
  T h{};
  cudaMemcpyAsync(&h, d, sizeof(T), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  return h;
}

// one pairwise pass on (n, rp, ci, v): S.agg [n] -> [0, *nc) or -1
int pairwise_pass(nalu_ctx* ctx, MlScratch& S, int64_t n, const int64_t* rp, const int32_t* ci, const double* v,
                  int P, int64_t* nc_out) {
  cudaStream_t s = ctx->stream;
  NALU_CUDA(ctx, grow(S.smax, n));
  NALU_CUDA(ctx, grow(S.diag, n));
  for (DBuf<int32_t>* b : {&S.partner, &S.choice, &S.leader, &S.target, &S.agg}) NALU_CUDA(ctx, grow(*b, n));
  NALU_CUDA(ctx, grow(S.flag, n + 1));
  NALU_CUDA(ctx, grow(S.id, n + 1));
  const unsigned g = grid_n(n);
  k_ml_smax<<<g, kMlThreads, 0, s>>>(n, rp, ci, v, S.smax.p, S.diag.p);
  if (P > 1) {
    k_ml_freeze<<<g, kMlThreads, 0, s>>>(n, S.off.p, P, kCoarsest, S.smax.p);
    ctx->launches++;
  }
  k_ml_fill_i32<<<g, kMlThreads, 0, s>>>(n, S.partner.p, -1);
  for (int r = 0; r < kMatchRounds; ++r) {
    k_ml_choose<<<g, kMlThreads, 0, s>>>(n, rp, ci, v, S.smax.p, S.diag.p, S.partner.p, r, S.choice.p);
    k_ml_match<<<g, kMlThreads, 0, s>>>(n, S.choice.p, S.partner.p);
  }
  k_ml_target<<<g, kMlThreads, 0, s>>>(n, rp, ci, v, S.smax.p, S.partner.p, S.target.p);
  k_ml_attach<<<g, kMlThreads, 0, s>>>(n, rp, ci, S.smax.p, S.partner.p, S.target.p, S.leader.p);
  k_ml_flag_leaders<<<g, kMlThreads, 0, s>>>(n, S.leader.p, S.flag.p);
  NALU_CUDA(ctx, cudaMemsetAsync(S.flag.p + n, 0, sizeof(int32_t), s));
  int rc = exclusive_scan<int32_t>(ctx, S, S.flag.p, S.id.p, n + 1);
  if (rc) return rc;
  k_ml_assign<<<g, kMlThreads, 0, s>>>(n, S.leader.p, S.id.p, S.agg.p);
  ctx->launches += 7 + 2 * kMatchRounds;
  *nc_out = read_one(ctx, S.id.p + n);
  return cuda_check(ctx, cudaGetLastError(), "pairwise aggregation");
}

// members of each aggregate, in row order: mptr [nc+1], mem [n] (excluded rows last, not counted)
int build_members(nalu_ctx* ctx, MlScratch& S, int64_t n, int64_t nc, const int32_t* agg, int64_t* mptr,
                  int32_t* mem) {
  cudaStream_t s = ctx->stream;
  NALU_CUDA(ctx, grow(S.keys, n));
  NALU_CUDA(ctx, grow(S.iota, n));
  k_ml_iota<<<grid_n(n), kMlThreads, 0, s>>>(n, S.iota.p);
  const uint32_t* ukeys = reinterpret_cast<const uint32_t*>(agg);  // -1 sorts after every id
  size_t tmp = 0;
  NALU_CUDA(ctx, cub::DeviceRadixSort::SortPairs(nullptr, tmp, ukeys, S.keys.p, S.iota.p, mem, (int)n, 0, 32, s));
  NALU_CUDA(ctx, grow(S.cub, (int64_t)tmp + 1));
  NALU_CUDA(ctx, cub::DeviceRadixSort::SortPairs(S.cub.p, tmp, ukeys, S.keys.p, S.iota.p, mem, (int)n, 0, 32, s));
  k_ml_member_ptr<<<grid_n(n), kMlThreads, 0, s>>>(n, nc, S.keys.p, mptr);
  ctx->launches += 2;
  return cuda_check(ctx, cudaGetLastError(), "aggregate members");
}

// count pass of the Galerkin product with capacity CFG; *ok: no row overflowed
template <class CFG>
int galerkin_count(nalu_ctx* ctx, MlScratch& S, const int64_t* rp, const int32_t* ci, const double* v,
                   const int32_t* agg, int64_t nc, const int64_t* mptr, const int32_t* mem, bool* ok) {
  cudaStream_t s = ctx->stream;
  const size_t smem = sizeof(typename CFG::Smem) * CFG::kWarps;
  NALU_CUDA(ctx, cudaFuncSetAttribute(k_ml_galerkin<true, CFG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  NALU_CUDA(ctx, cudaMemsetAsync(S.flagd.p, 0, sizeof(int), s));
  const unsigned g =
      (unsigned)std::max<int64_t>(1, std::min<int64_t>((nc + CFG::kWarps - 1) / CFG::kWarps, 8 * kMlBlocks));
  k_ml_galerkin<true, CFG><<<g, 32 * CFG::kWarps, smem, s>>>(nc, mptr, mem, rp, ci, v, agg, nullptr, S.cnt.p,
                                                              nullptr, nullptr, S.flagd.p);
  ctx->launches++;
  *ok = read_one(ctx, S.flagd.p) == 0;
  return cuda_check(ctx, cudaGetLastError(), "Galerkin count");
}
template <class CFG>
int galerkin_fill(nalu_ctx* ctx, MlScratch& S, const int64_t* rp, const int32_t* ci, const double* v,
                  const int32_t* agg, int64_t nc, const int64_t* mptr, const int32_t* mem, int slot) {
  cudaStream_t s = ctx->stream;
  const size_t smem = sizeof(typename CFG::Smem) * CFG::kWarps;
  NALU_CUDA(ctx, cudaFuncSetAttribute(k_ml_galerkin<false, CFG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  const unsigned g =
      (unsigned)std::max<int64_t>(1, std::min<int64_t>((nc + CFG::kWarps - 1) / CFG::kWarps, 8 * kMlBlocks));
  k_ml_galerkin<false, CFG><<<g, 32 * CFG::kWarps, smem, s>>>(nc, mptr, mem, rp, ci, v, agg, S.rp[slot].p, nullptr,
                                                               S.ci[slot].p, S.v[slot].p, S.flagd.p);
  ctx->launches++;
  return cuda_check(ctx, cudaGetLastError(), "Galerkin fill");
}

// Galerkin product of (rp, ci, v) for the aggregation agg -> coarse CRS in
// the scratch matrix `slot` (the small capacity, the large one if a row
// overflows it; NALU_ERR_CAPACITY beyond that)
int galerkin(nalu_ctx* ctx, MlScratch& S, const int64_t* rp, const int32_t* ci, const double* v, const int32_t* agg,
             int64_t nc, const int64_t* mptr, const int32_t* mem, int slot, int64_t* cnnz) {
  cudaStream_t s = ctx->stream;
  NALU_CUDA(ctx, grow(S.cnt, nc + 1));
  NALU_CUDA(ctx, grow(S.rp[slot], nc + 1));
  NALU_CUDA(ctx, grow(S.flagd, 1));
  NALU_CUDA(ctx, cudaMemsetAsync(S.cnt.p + nc, 0, sizeof(int64_t), s));
  bool ok = false, large = false;
  int rc = galerkin_count<GalSmall>(ctx, S, rp, ci, v, agg, nc, mptr, mem, &ok);
  if (rc) return rc;
  if (!ok) {
    large = true;
    if ((rc = galerkin_count<GalLarge>(ctx, S, rp, ci, v, agg, nc, mptr, mem, &ok))) return rc;
    if (!ok) return set_error(ctx, NALU_ERR_CAPACITY, "multilevel: coarse row too long");
  }
  if ((rc = exclusive_scan<int64_t>(ctx, S, S.cnt.p, S.rp[slot].p, nc + 1))) return rc;
  *cnnz = read_one(ctx, S.rp[slot].p + nc);
  NALU_CUDA(ctx, grow(S.ci[slot], std::max<int64_t>(*cnnz, 1)));
  NALU_CUDA(ctx, grow(S.v[slot], std::max<int64_t>(*cnnz, 1)));
  return large ? galerkin_fill<GalLarge>(ctx, S, rp, ci, v, agg, nc, mptr, mem, slot)
               : galerkin_fill<GalSmall>(ctx, S, rp, ci, v, agg, nc, mptr, mem, slot);
}

// lambda_max of S A (S = D^-1, or the learned M) by power iteration
float power_lambda(nalu_ctx* ctx, MlState& M, MlLevel& L, const float* m, int iters) {
  cudaStream_t s = ctx->stream;
  const int64_t n = L.n;
  float *x = L.z.p, *t = L.t.p, *y = L.z2.p;
  k_ml_seed<<<grid_n(n), kMlThreads, 0, s>>>(n, x);
  for (int it = 0; it < iters; ++it) {
    k_ml_power_ax<<<grid_rows(n), kMlThreads, 0, s>>>(n, L.rp, L.ci, L.vf.p, x, t);
    k_ml_power_s<<<grid_rows(n), kMlThreads, 0, s>>>(n, L.rp, L.ci, m, L.dinv.p, t, y, M.partial.p, M.counter.p,
                                                      M.ks.p);
    k_ml_scale<<<grid_n(n), kMlThreads, 0, s>>>(n, M.ks.p, y, x);
    ctx->launches += 3;
  }
  // x was unit before the last product: lambda ~ ||S A x||
  const double yy = read_one(ctx, M.ks.p);
  return (float)std::sqrt(std::max(yy, 0.0));
}

int alloc_level_vectors(nalu_ctx* ctx, MlLevel& L, bool kcycle) {
  const int64_t n = std::max<int64_t>(L.n, 1);
  for (DBuf<float>* b : {&L.z, &L.t, &L.z2, &L.b}) NALU_CUDA(ctx, grow(*b, n));
  if (kcycle)
    for (DBuf<float>* b : {&L.v1, &L.v2, &L.w1, &L.w2, &L.rt, &L.e}) NALU_CUDA(ctx, grow(*b, n));
  return NALU_OK;
}

}  // namespace

// Build the hierarchy for the current scalar matrix (for the learned smoother,
// learned_prepare has run on it).
int ml_setup(nalu_ctx* ctx, bool learned, const std::vector<int64_t>* row_off) {
  if (!ctx->ml) ctx->ml = new MlState();
  MlState& M = *ctx->ml;
  M.ready = false;
  M.learned = learned;
  M.klevels = 0;  // V-cycle unless the flexible CG that uses it asks otherwise
  cudaStream_t s = ctx->stream;
  NALU_CUDA(ctx, grow(M.partial, 3 * 4 * kMlBlocks + 64));
  NALU_CUDA(ctx, grow(M.ks, 8 * (kMaxLevels + 2)));
  NALU_CUDA(ctx, grow(M.counter, kCounters));
  NALU_CUDA(ctx, cudaMemsetAsync(M.counter.p, 0, sizeof(unsigned) * kCounters, s));
  NALU_CUDA(ctx, cudaMemsetAsync(M.ks.p, 0, sizeof(double) * 8 * (kMaxLevels + 2), s));
  // levels are rebuilt in place: their buffers are kept between solves and
  // grow only when a level needs more
  M.lv.reserve(kMaxLevels + 1);
  if (M.lv.empty()) M.lv.emplace_back();
  {
    MlLevel& L0 = M.lv[0];
    L0.n = ctx->n_rows;
    L0.nnz = ctx->nnz;
    L0.rp = ctx->d_rowptr.p;
    L0.ci = ctx->d_colind.p;
    L0.vd = ctx->d_values.p;
  }
  int rc = NALU_OK;
  MlScratch& S = M.sc;
  // problems (row ranges of independent blocks): each coarsens down to
  // kCoarsest rows on its own; without them the whole system is one
  std::vector<int64_t> off = row_off ? *row_off : std::vector<int64_t>{0, ctx->n_rows};
  const int P = (int)off.size() - 1;
  if (P < 1 || off[0] != 0 || off[P] != ctx->n_rows) return set_error(ctx, NALU_ERR_ARG, "multilevel: row ranges");
  auto max_block = [&]() {
    int64_t m = 0;
    for (int p = 0; p < P; ++p) m = std::max(m, off[p + 1] - off[p]);
    return m;
  };
  if (P > 1) {
    NALU_CUDA(ctx, grow(S.off, P + 1));
    NALU_CUDA(ctx, grow(S.off2, P + 1));
    NALU_CUDA(ctx, cudaMemcpyAsync(S.off.p, off.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, s));
  }
  // levels of up to three pairwise passes each, down to kCoarsest rows
  int top = 0;  // the level being coarsened
  while (top + 1 < kMaxLevels && max_block() > kCoarsest) {
    MlLevel& F = M.lv[top];
    NALU_CUDA(ctx, grow(F.agg, F.n));
    k_ml_iota<<<grid_n(F.n), kMlThreads, 0, s>>>(F.n, F.agg.p);
    ctx->launches++;
    int64_t n = F.n, nnz = F.nnz;
    const int64_t* rp = F.rp;
    const int32_t* ci = F.ci;
    const double* v = F.vd;
    int slot = -1;
    for (int pass = 0; pass < kPassesPerLevel; ++pass) {
      int64_t nc = 0;
      if ((rc = pairwise_pass(ctx, S, n, rp, ci, v, P, &nc))) return rc;
      if (nc >= n) break;  // nothing left to pair
      if (P > 1) {
        k_ml_next_offsets<<<1, 128, 0, s>>>(P, S.off.p, S.id.p, S.off2.p);
        ctx->launches++;
        NALU_CUDA(ctx, cudaMemcpyAsync(off.data(), S.off2.p, sizeof(int64_t) * (P + 1), cudaMemcpyDeviceToHost, s));
        NALU_CUDA(ctx, cudaMemcpyAsync(S.off.p, S.off2.p, sizeof(int64_t) * (P + 1), cudaMemcpyDeviceToDevice, s));
        NALU_CUDA(ctx, cudaStreamSynchronize(s));
      } else {
        off[1] = nc;
      }
      NALU_CUDA(ctx, grow(S.mptr, nc + 1));
      NALU_CUDA(ctx, grow(S.mem, n));
      if ((rc = build_members(ctx, S, n, nc, S.agg.p, S.mptr.p, S.mem.p))) return rc;
      slot = (slot + 1) & 1;
      int64_t cnnz = 0;
      if ((rc = galerkin(ctx, S, rp, ci, v, S.agg.p, nc, S.mptr.p, S.mem.p, slot, &cnnz))) return rc;
      k_ml_compose<<<grid_n(F.n), kMlThreads, 0, s>>>(F.n, F.agg.p, S.agg.p);
      ctx->launches++;
      rp = S.rp[slot].p;
      ci = S.ci[slot].p;
      v = S.v[slot].p;
      n = nc;
      nnz = cnnz;
      if (max_block() <= kCoarsest) break;
    }
    if (n >= F.n) break;  // no coarsening: F is the coarsest level
    NALU_CUDA(ctx, grow(F.mptr, n + 1));
    NALU_CUDA(ctx, grow(F.mem, F.n));
    if ((rc = build_members(ctx, S, F.n, n, F.agg.p, F.mptr.p, F.mem.p))) return rc;
    if ((int)M.lv.size() < top + 2) M.lv.emplace_back();  // capacity reserved: F stays valid
    MlLevel& C = M.lv[top + 1];
    C.n = n;
    C.nnz = nnz;
    NALU_CUDA(ctx, grow(C.own_rp, n + 1));
    NALU_CUDA(ctx, grow(C.own_ci, std::max<int64_t>(nnz, 1)));
    NALU_CUDA(ctx, grow(C.own_vd, std::max<int64_t>(nnz, 1)));
    NALU_CUDA(ctx, cudaMemcpyAsync(C.own_rp.p, rp, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToDevice, s));
    NALU_CUDA(ctx, cudaMemcpyAsync(C.own_ci.p, ci, sizeof(int32_t) * nnz, cudaMemcpyDeviceToDevice, s));
    NALU_CUDA(ctx, cudaMemcpyAsync(C.own_vd.p, v, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, s));
    C.rp = C.own_rp.p;
    C.ci = C.own_ci.p;
    C.vd = C.own_vd.p;
    ++top;
  }
  M.lv.resize(top + 1);
  const int nl = (int)M.lv.size();
  if (max_block() > kDenseMax)
    return set_error(ctx, NALU_ERR_CAPACITY, "multilevel: coarsest level above 1024 rows (too few strong couplings)");
  M.boff = off;
  // FP32 copies, vectors
  for (int l = 0; l < nl; ++l) {
    MlLevel& L = M.lv[l];
    NALU_CUDA(ctx, grow(L.vf, std::max<int64_t>(L.nnz, 1)));
    NALU_CUDA(ctx, grow(L.dinv, std::max<int64_t>(L.n, 1)));
    k_ml_prep<<<grid_n(L.n), kMlThreads, 0, s>>>(L.n, L.rp, L.ci, L.vd, L.vf.p, L.dinv.p);
    ctx->launches++;
    if ((rc = alloc_level_vectors(ctx, L, l > 0 && l < nl - 1))) return rc;
  }
  if (learned) {
    MlLevel& L0 = M.lv[0];
    NALU_CUDA(ctx, grow(L0.msm, std::max<int64_t>(L0.nnz, 1)));
    k_ml_sell_to_crs<<<grid_n(L0.n), kMlThreads, 0, s>>>(L0.n, L0.rp, ctx->sw.sell.ptr.p, ctx->learned.wsell.p,
                                                         L0.msm.p);
    ctx->launches++;
  }
  {
    // level 0 on the SELL-32 copy (built by the solve for the outer CG)
    MlLevel& L0 = M.lv[0];
    const SellMatrix& SM = ctx->sw.sell;
    L0.sell = false;
    if (SM.c16_valid && SM.val2.p && SM.nslices * 32 >= L0.n) {
      NALU_CUDA(ctx, grow(L0.sellv, std::max<int64_t>(SM.stored, 1)));
      k_ml0_sell_f32<<<grid_n(SM.stored), kMlThreads, 0, s>>>(SM.stored, SM.val2.p, L0.sellv.p);
      ctx->launches++;
      L0.sv = SM.view();
      L0.sellm = learned ? ctx->learned.wsell.p : nullptr;
      L0.sell = true;
    }
  }
  // smoothing weights
  for (int l = 0; l < nl - 1; ++l) {
    MlLevel& L = M.lv[l];
    const float lam = power_lambda(ctx, M, L, (l == 0 && learned) ? L.msm.p : nullptr, 12);
    L.omega = lam > 0.0f && std::isfinite(lam) ? 4.0f / (3.0f * lam) : 0.6f;
    L.omega_j = L.omega;
    if (l == 0 && learned) {  // the Jacobi weight too, for sweeps the learned smoother leaves to Jacobi
      const float lj = power_lambda(ctx, M, L, nullptr, 12);
      L.omega_j = lj > 0.0f && std::isfinite(lj) ? 4.0f / (3.0f * lj) : 0.6f;
    }
  }
  if (P == 1) {
    // coarsest level: dense inverse
    MlLevel& C = M.lv.back();
    const int nc = (int)C.n;
    DBuf<float> D;
    DBuf<int> bad;
    NALU_CUDA(ctx, D.alloc((int64_t)nc * 2 * nc));
    NALU_CUDA(ctx, grow(C.inv, (int64_t)nc * nc));
    NALU_CUDA(ctx, bad.alloc(1));
    NALU_CUDA(ctx, cudaMemsetAsync(bad.p, 0, sizeof(int), s));
    k_ml_dense_fill<<<grid_n((int64_t)nc * 2 * nc), kMlThreads, 0, s>>>(nc, D.p);
    k_ml_dense_scatter<<<grid_n(nc), kMlThreads, 0, s>>>(nc, C.rp, C.ci, C.vd, D.p);
    k_ml_gauss_jordan<<<1, 1024, 0, s>>>(nc, D.p, bad.p);
    k_ml_dense_extract<<<grid_n((int64_t)nc * nc), kMlThreads, 0, s>>>(nc, D.p, C.inv.p);
    ctx->launches += 4;
    if (read_one(ctx, bad.p)) return set_error(ctx, NALU_ERR_NONFINITE, "multilevel: singular coarsest matrix");
  } else {
    // coarsest level of independent problems: one dense inverse per problem
    // (the coarsest matrix is block diagonal), applied by one launch
    MlLevel& C = M.lv.back();
    std::vector<int64_t> ioff(P + 1, 0);
    std::vector<int32_t> brow((size_t)std::max<int64_t>(C.n, 1), 0);
    int64_t nbmax = 0;
    for (int p = 0; p < P; ++p) {
      const int64_t nb = off[p + 1] - off[p];
      ioff[p + 1] = ioff[p] + nb * nb;
      nbmax = std::max(nbmax, nb);
      for (int64_t r = off[p]; r < off[p + 1]; ++r) brow[r] = p;
    }
    (void)nbmax;
    DBuf<float> D;  // every block's [A | I], side by side
    DBuf<int64_t> doff_d;
    DBuf<int> bad;
    NALU_CUDA(ctx, D.alloc(std::max<int64_t>(2 * ioff[P], 1)));
    NALU_CUDA(ctx, grow(C.inv, std::max<int64_t>(ioff[P], 1)));
    NALU_CUDA(ctx, bad.alloc(1));
    NALU_CUDA(ctx, doff_d.alloc(P + 1));
    NALU_CUDA(ctx, cudaMemsetAsync(bad.p, 0, sizeof(int), s));
    std::vector<int64_t> doff(P + 1);
    for (int p = 0; p <= P; ++p) doff[p] = 2 * ioff[p];
    NALU_CUDA(ctx, cudaMemcpyAsync(doff_d.p, doff.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, s));
    NALU_CUDA(ctx, grow(M.boff_d, P + 1));
    NALU_CUDA(ctx, grow(M.ioff_d, P + 1));
    NALU_CUDA(ctx, cudaMemcpyAsync(M.boff_d.p, off.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, s));
    NALU_CUDA(ctx, cudaMemcpyAsync(M.ioff_d.p, ioff.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, s));
    for (int p = 0; p < P; ++p) {
      const int nb = (int)(off[p + 1] - off[p]);
      if (nb == 0) continue;
      k_ml_dense_fill<<<grid_n((int64_t)nb * 2 * nb), kMlThreads, 0, s>>>(nb, D.p + doff[p]);
      k_ml_dense_scatter_block<<<grid_n(nb), kMlThreads, 0, s>>>(nb, off[p], C.rp + off[p], C.ci, C.vd,
                                                                 D.p + doff[p]);
      ctx->launches += 2;
    }
    k_ml_gauss_jordan_blocks<<<P, 1024, 0, s>>>(M.boff_d.p, doff_d.p, D.p, bad.p);
    ctx->launches++;
    for (int p = 0; p < P; ++p) {
      const int nb = (int)(off[p + 1] - off[p]);
      if (nb == 0) continue;
      k_ml_dense_extract<<<grid_n((int64_t)nb * nb), kMlThreads, 0, s>>>(nb, D.p + doff[p], C.inv.p + ioff[p]);
      ctx->launches++;
    }
    NALU_CUDA(ctx, grow(M.brow, (int64_t)brow.size()));
    NALU_CUDA(ctx, cudaMemcpyAsync(M.brow.p, brow.data(), sizeof(int32_t) * brow.size(), cudaMemcpyHostToDevice, s));
    if (read_one(ctx, bad.p)) return set_error(ctx, NALU_ERR_NONFINITE, "multilevel: singular coarsest block");
  }
  NALU_CUDA(ctx, cudaStreamSynchronize(s));
  M.ready = true;
  return cuda_check(ctx, cudaGetLastError(), "multilevel set-up");
}

namespace {

void cycle(nalu_ctx* ctx, MlState& M, int l, const float* b, float* z, int* site);

// e ~ A_l^-1 r at a coarse level l: the dense inverse at the coarsest level,
// else a K-cycle (two flexible CG steps preconditioned by the cycle of level
// l) or, below the K-cycle levels, one cycle
void coarse_solve(nalu_ctx* ctx, MlState& M, int l, const float* r, float* e, int* site) {
  cudaStream_t s = ctx->stream;
  MlLevel& L = M.lv[l];
  const int nl = (int)M.lv.size();
  if (l == nl - 1) {
    const unsigned g = (unsigned)((L.n * 32 + kMlThreads - 1) / kMlThreads);
    if (M.boff.size() > 2)
      k_ml_dense_apply_blocks<<<g, kMlThreads, 0, s>>>(L.n, M.brow.p, M.boff_d.p, M.ioff_d.p, L.inv.p, r, e);
    else
      k_ml_dense_apply<<<g, kMlThreads, 0, s>>>((int)L.n, L.inv.p, r, e);
    ctx->launches++;
    return;
  }
  if (l > M.klevels) {
    cycle(ctx, M, l, r, e, site);
    return;
  }
  double* ks = M.ks.p + 8 * l;
  const unsigned gr = grid_rows(L.n), gn = grid_n(L.n);
  cycle(ctx, M, l, r, L.v1.p, site);
  const int c1 = (*site)++ % kCounters;
  k_ml_kspmv<false><<<gr, kMlThreads, 0, s>>>(L.n, L.rp, L.ci, L.vf.p, L.v1.p, L.w1.p, r, nullptr, M.partial.p,
                                               M.counter.p + c1, ks);  // ks[0] rho1, ks[1] alpha1
  k_ml_kstep1<<<gn, kMlThreads, 0, s>>>(L.n, ks, r, L.w1.p, L.rt.p);
  cycle(ctx, M, l, L.rt.p, L.v2.p, site);
  const int c2 = (*site)++ % kCounters;
  k_ml_kspmv<true><<<gr, kMlThreads, 0, s>>>(L.n, L.rp, L.ci, L.vf.p, L.v2.p, L.w2.p, L.rt.p, L.w1.p, M.partial.p,
                                              M.counter.p + c2, ks + 2);  // ks[2] beta, ks[3] alpha2, ks[4] gamma
  k_ml_kcombine<<<gn, kMlThreads, 0, s>>>(L.n, ks, L.v1.p, L.v2.p, e);
  ctx->launches += 4;
}

// z = B_l b: the cycle at level l from a zero guess (l below the coarsest)
void cycle(nalu_ctx* ctx, MlState& M, int l, const float* b, float* z, int* site) {
  cudaStream_t s = ctx->stream;
  MlLevel& L = M.lv[l];
  MlLevel& C = M.lv[l + 1];
  const unsigned gr = grid_rows(L.n), gn = grid_n(L.n), gc = grid_n(C.n);
  const bool learned_pre = l == 0 && M.learned && (M.lsweeps & 1);
  const bool learned_post = l == 0 && M.learned && (M.lsweeps & 2);
  const float wj = L.omega_j;  // the Jacobi weight (equal to omega without the learned smoother)
  if (L.sell) {
    // level 0 on the SELL-32 copy
    const unsigned gs = grid_n(L.n);
    if (learned_pre) {
      k_ml0_mstep<<<gs, kMlThreads, 0, s>>>(L.n, L.sv, L.sellm, L.omega, b, nullptr, z);
      k_ml0_residual<<<gs, kMlThreads, 0, s>>>(L.n, L.sv, L.sellv.p, z, b, L.t.p);
      ctx->launches += 2;
    } else {
      k_ml0_jac0_residual<<<gs, kMlThreads, 0, s>>>(L.n, L.sv, L.sellv.p, L.dinv.p, wj, b, z, L.t.p);
      ctx->launches++;
    }
    float* ec = (l + 1 == (int)M.lv.size() - 1) ? C.z.p : C.e.p;
    k_ml_restrict<<<gc, kMlThreads, 0, s>>>(C.n, L.mptr.p, L.mem.p, L.t.p, C.b.p);
    coarse_solve(ctx, M, l + 1, C.b.p, ec, site);
    k_ml_prolong<<<gn, kMlThreads, 0, s>>>(L.n, L.agg.p, ec, z);
    ctx->launches += 2;
    if (learned_post) {
      k_ml0_residual<<<gs, kMlThreads, 0, s>>>(L.n, L.sv, L.sellv.p, z, b, L.t.p);
      k_ml0_mstep<<<gs, kMlThreads, 0, s>>>(L.n, L.sv, L.sellm, L.omega, L.t.p, z, L.z2.p);
    } else {
      k_ml0_jac_step<<<gs, kMlThreads, 0, s>>>(L.n, L.sv, L.sellv.p, L.dinv.p, wj, b, z, L.z2.p);
    }
    cudaMemcpyAsync(z, L.z2.p, sizeof(float) * L.n, cudaMemcpyDeviceToDevice, s);
    ctx->launches += learned_post ? 2 : 1;
    return;
  }
  // pre-smoothing from zero, then the residual
  if (learned_pre) {
    k_ml_mstep<<<gr, kMlThreads, 0, s>>>(L.n, L.rp, L.ci, L.msm.p, L.omega, b, nullptr, z);
    k_ml_residual<<<gr, kMlThreads, 0, s>>>(L.n, L.rp, L.ci, L.vf.p, z, b, L.t.p);
    ctx->launches += 2;
  } else {
    k_ml_jac0_residual<<<gr, kMlThreads, 0, s>>>(L.n, L.rp, L.ci, L.vf.p, L.dinv.p, wj, b, z, L.t.p);
    ctx->launches++;
  }
  // coarse correction
  float* ec = (l + 1 == (int)M.lv.size() - 1) ? C.z.p : C.e.p;
  k_ml_restrict<<<gc, kMlThreads, 0, s>>>(C.n, L.mptr.p, L.mem.p, L.t.p, C.b.p);
  coarse_solve(ctx, M, l + 1, C.b.p, ec, site);
  k_ml_prolong<<<gn, kMlThreads, 0, s>>>(L.n, L.agg.p, ec, z);
  ctx->launches += 2;
  // post-smoothing
  if (learned_post) {
    k_ml_residual<<<gr, kMlThreads, 0, s>>>(L.n, L.rp, L.ci, L.vf.p, z, b, L.t.p);
    k_ml_mstep<<<gr, kMlThreads, 0, s>>>(L.n, L.rp, L.ci, L.msm.p, L.omega, L.t.p, z, L.z2.p);
  } else {
    k_ml_jac_step<<<gr, kMlThreads, 0, s>>>(L.n, L.rp, L.ci, L.vf.p, L.dinv.p, wj, b, z, L.z2.p);
  }
  cudaMemcpyAsync(z, L.z2.p, sizeof(float) * L.n, cudaMemcpyDeviceToDevice, s);
  ctx->launches += learned_post ? 2 : 1;
}

}  // namespace

// Flexible CG preconditioned by the multilevel cycle (the FP32-pair flexible
// CG of learned.cu with the df64 SELL-32 SpMV; the cycle runs on the FP32
// residual), on the residual r (FP64, updated in place) for the correction x
// (FP64, from zero), to ||r|| <= rtol r0norm.
int fcg_multilevel(nalu_ctx* ctx, double* x, double* r, double rtol, double r0norm, int max_it, int check_every,
                   int klevels, int learned_sweeps, int* iters_out) {
  *iters_out = 0;
  if (!ctx->ml || !ctx->ml->ready || ctx->ml->lv.empty())
    return set_error(ctx, NALU_ERR_STATE, "multilevel hierarchy not built");
  MlState& M = *ctx->ml;
  M.klevels = std::max(klevels, 0);
  // default: the learned smoother in both sweeps, which keeps the cycle
  // symmetric (at 128^3: 83 steps, 92.4 ms; pre-smoothing only 89 steps,
  // 83.7 ms, but that unsymmetric cycle took 1960 steps instead of 273 on the
  // 64-mesh union system)
  M.lsweeps = learned_sweeps > 0 ? (learned_sweeps & 3) : 3;
  auto prec = [&](const float* rf, float* zf) {
    int site = 0;
    if (M.lv.size() == 1) coarse_solve(ctx, M, 0, rf, zf, &site);  // one level: the dense inverse
    else cycle(ctx, M, 0, rf, zf, &site);
  };
  return fcg_df_external(ctx, x, r, rtol, r0norm, max_it, check_every, prec, iters_out);
}

int ml_apply(nalu_ctx* ctx, const float* rf, float* zf) {
  if (!ctx->ml || !ctx->ml->ready || ctx->ml->lv.empty())
    return set_error(ctx, NALU_ERR_STATE, "multilevel hierarchy not built");
  MlState& M = *ctx->ml;
  int site = 0;
  if (M.lv.size() == 1) coarse_solve(ctx, M, 0, rf, zf, &site);
  else cycle(ctx, M, 0, rf, zf, &site);
  return NALU_OK;
}

void ml_free(nalu_ctx* ctx) {
  delete ctx->ml;
  ctx->ml = nullptr;
}

int ml_levels(const nalu_ctx* ctx, int max_levels, int64_t* rows, int64_t* nnz) {
  if (!ctx->ml || !ctx->ml->ready) return 0;
  const int nl = (int)ctx->ml->lv.size();
  for (int l = 0; l < nl && l < max_levels; ++l) {
    if (rows) rows[l] = ctx->ml->lv[l].n;
    if (nnz) nnz[l] = ctx->ml->lv[l].nnz;
  }
  return nl;
}

}  // namespace nalu_gb300
