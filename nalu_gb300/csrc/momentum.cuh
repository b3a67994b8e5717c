// momentum.cuh -- arguments, shared-memory layout and ip table of the 24x24
// momentum element kernels (momentum.cu: FP64, momentum_df.cu: df64).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace nalu_gb300 {

constexpr int kMomElems = 16;
constexpr int kMomThreads = kMomElems * 12;  // 192

struct MomArgs {
  const int32_t* __restrict__ conn;
  const double* __restrict__ x;
  const double* __restrict__ u;
  const double* __restrict__ vrtm;
  const double* __restrict__ rho;
  const double* __restrict__ mu;
  const double* __restrict__ gju;
  const double* __restrict__ mdot;  // [E][12]
  double include_divu, alpha, alpha_upw, upw, hf;
  int use_limiter;
  const int64_t* __restrict__ rowptr;
  const uint8_t* __restrict__ slots;
  double* __restrict__ values;
  double* __restrict__ rhs;
  const int32_t* __restrict__ elems;
  int64_t count;
  int32_t* flags;
  double* cap_lhs;
  double* cap_rhs;
  int64_t cap_elem;
};

// shared-memory layout per element (doubles)
struct MomLayout {
  static constexpr int X = 0, U = 24, MU = 48, MD = 56, VR = 68, RHO = 92, GJU = 100;
  static constexpr int NODE_END = 172;
  static constexpr int DNDX = NODE_END;          // [12][8][3]
  static constexpr int AA = DNDX + 288;          // [12][3]   -mu_ip * A_j
  static constexpr int DIAG = AA + 36;           // [12][8]   same-dof factor
  static constexpr int RIP = DIAG + 96;          // [12][3]   residual per ip
  static constexpr int ALHS = RIP + 36;          // [12][2]   upwind L/R factors
  // 652 used, padded to 657 so that the element stride (2 SIZE 32-bit words)
  // is 2 mod 32: equal offsets of the 16 elements fall in different banks
  static constexpr int SIZE = ALHS + 24 + 5;     // 657
};
static_assert((2 * MomLayout::SIZE) % 32 == 2, "element stride");

// ips adjacent to node r, ascending
__device__ __forceinline__ int node_ip(int r, int k) {
  // node 0: 0 3 8 | 1: 0 1 9 | 2: 1 2 10 | 3: 2 3 11 | 4: 4 7 8 | 5: 4 5 9 | 6: 5 6 10 | 7: 6 7 11
  const int tab[8][3] = {{0, 3, 8}, {0, 1, 9}, {1, 2, 10}, {2, 3, 11}, {4, 7, 8}, {4, 5, 9}, {5, 6, 10}, {6, 7, 11}};
  return tab[r][k];
}


int launch_momentum_df(nalu_ctx* ctx, int kernel, const MomArgs& a, int scatter, int64_t cap_elem, bool shift,
                       bool skew);

}  // namespace nalu_gb300
