// scv.cuh -- HexSCV sub-control volumes on the device.
//
// HexSCV::determinant (src/master_element/Hex8CVFEM.C:149-180): the element
// is cut into eight sub-hexahedra through its 27-point subdivision
// (subdivide_hex_8, Hex8GeometryFunctions.h:263-322), sub-hexahedron ip
// holding node ip (ipNodeMap is the identity), and each volume is Grandy's
// (hex_volume_grandy, Hex8GeometryFunctions.h:78-163): six face centroids and
// 24 triangles whose signed contributions sum to 18 V.  Internal linkage: each
// translation unit that includes it gets its own constant tables.
#pragma once
#include <cstdint>

namespace nalu_gb300 {
namespace {

// point k (0..26) of the 27-point subdivision, component d
__device__ double subpoint(const double (*c)[3], int k, int d) {
  auto m2 = [&](int a, int b) { return 0.5 * (c[a][d] + c[b][d]); };
  auto m4 = [&](int a, int b, int e, int f) { return 0.25 * (c[a][d] + c[b][d] + c[e][d] + c[f][d]); };
  switch (k) {
    case 8: return m2(0, 1);
    case 9: return m2(1, 2);
    case 10: return m2(2, 3);
    case 11: return m2(3, 0);
    case 12: return m4(0, 1, 2, 3);
    case 13: return m2(4, 5);
    case 14: return m2(5, 6);
    case 15: return m2(6, 7);
    case 16: return m2(7, 4);
    case 17: return m4(4, 5, 6, 7);
    case 18: return m2(1, 5);
    case 19: return m2(0, 4);
    case 20: return m4(0, 1, 4, 5);
    case 21: return m2(3, 7);
    case 22: return m2(2, 6);
    case 23: return m4(2, 3, 6, 7);
    case 24: return m4(1, 2, 5, 6);
    case 25: return m4(0, 3, 4, 7);
    case 26: {
      double s = 0.0;
      for (int n = 0; n < 8; ++n) s += c[n][d];
      return s * 0.125;
    }
    default: return c[k][d];
  }
}

__constant__ int8_t c_sub[8][8] = {{0, 8, 12, 11, 19, 20, 26, 25},  {8, 1, 9, 12, 20, 18, 24, 26},
                                   {12, 9, 2, 10, 26, 24, 22, 23},  {11, 12, 10, 3, 25, 26, 23, 21},
                                   {19, 20, 26, 25, 4, 13, 17, 16}, {20, 18, 24, 26, 13, 5, 14, 17},
                                   {26, 24, 22, 23, 17, 14, 6, 15}, {25, 26, 23, 21, 16, 17, 15, 7}};
__constant__ int8_t c_gface[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {2, 3, 7, 6}, {1, 2, 6, 5}, {0, 4, 3, 7}};
__constant__ int8_t c_gtri[24][3] = {{0, 8, 1},  {8, 2, 1},   {3, 2, 8},   {3, 8, 0},  {6, 9, 5},   {7, 9, 6},
                                     {4, 9, 7},  {4, 5, 9},   {10, 0, 1},  {5, 10, 1}, {4, 10, 5},  {4, 0, 10},
                                     {7, 6, 11}, {6, 2, 11},  {2, 3, 11},  {3, 7, 11}, {6, 12, 2},  {5, 12, 6},
                                     {5, 1, 12}, {1, 2, 12},  {0, 4, 13},  {4, 7, 13}, {7, 3, 13},  {3, 0, 13}};

// Grandy's hexahedron volume: six face centroids, 24 triangles
__device__ double grandy_volume(const double (&h)[8][3]) {
  double cv[14][3];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int d = 0; d < 3; ++d) cv[n][d] = h[n][d];
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      cv[k + 8][d] = 0.25 * (cv[c_gface[k][0]][d] + cv[c_gface[k][1]][d] + cv[c_gface[k][2]][d] + cv[c_gface[k][3]][d]);
  double volume = 0.0;
#pragma unroll
  for (int k = 0; k < 24; ++k) {
    const int p = c_gtri[k][0], q = c_gtri[k][1], r = c_gtri[k][2];
    const double m0 = cv[p][0] + cv[q][0] + cv[r][0], m1 = cv[p][1] + cv[q][1] + cv[r][1],
                 m2 = cv[p][2] + cv[q][2] + cv[r][2];
    const double d0 = (cv[q][1] - cv[p][1]) * (cv[r][2] - cv[p][2]) - (cv[r][1] - cv[p][1]) * (cv[q][2] - cv[p][2]);
    const double d1 = (cv[r][0] - cv[p][0]) * (cv[q][2] - cv[p][2]) - (cv[q][0] - cv[p][0]) * (cv[r][2] - cv[p][2]);
    const double d2 = (cv[q][0] - cv[p][0]) * (cv[r][1] - cv[p][1]) - (cv[r][0] - cv[p][0]) * (cv[q][1] - cv[p][1]);
    volume += m0 * d0 + m1 * d1 + m2 * d2;
  }
  return volume / 18.0;
}

// volume of sub-control volume ip of the element with corners c
__device__ inline double scv_volume(const double (*c)[3], int ip) {
  double h[8][3];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int d = 0; d < 3; ++d) h[n][d] = subpoint(c, c_sub[ip][n], d);
  return grandy_volume(h);
}

}  // namespace
}  // namespace nalu_gb300
