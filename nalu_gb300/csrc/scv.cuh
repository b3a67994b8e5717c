// scv.cuh -- HexSCV sub-control volumes on the device.
//
// HexSCV::determinant (src/master_element/Hex8CVFEM.C:149-180): the element
// is cut into eight sub-hexahedra through its 27-point subdivision
// (subdivide_hex_8, Hex8GeometryFunctions.h:263-322), sub-hexahedron ip
// holding node ip (ipNodeMap is the identity), and each volume is Grandy's
// (hex_volume_grandy, Hex8GeometryFunctions.h:78-163): six face centroids and
// 24 triangles.  The same volume is evaluated here in a cheaper, equivalent
// form (below); it differs from the reference's evaluation order only by
// rounding, and is the closer of the two to the exact value (the reference's
// corner-coordinate sums cancel by up to ~1e-14 relative on small elements
// far from the origin).
#pragma once
#include <cstdint>

#include "hex8_elem.h"

namespace nalu_gb300 {
namespace {

// Volume of sub-control volume ip: the sub-hexahedron between node ip's
// corner and the parent centre, whose corners are node ip, the three edge
// midpoints, the three face centroids at that node and the element centroid
// (points of subdivide_hex_8).  Grandy's volume of a hexahedron (its faces
// triangulated through their centroids) equals, summed face by face,
//   V = sum_faces ((c - a) x (d - b)) . (a + b + c + d) / 24
// (each face (a,b,c,d) contributes (a x b + b x c + c x d + d x a) . centroid / 6
// and a x b + b x c + c x d + d x a = (c - a) x (d - b)), evaluated here about
// the element centroid, which keeps the cancellation of the corner terms
// small.  The sub-box is labelled in a frame mirrored so that node ip's side
// is "high" on every axis; each mirrored axis flips the orientation, hence the
// sign s0 s1 s2.  Corner k of that frame has the middle on the axes where
// corner_sign(k, .) < 0.
__device__ inline double scv_volume(const double (*c)[3], int ip) {
  const int s0 = corner_sign(ip, 0), s1 = corner_sign(ip, 1), s2 = corner_sign(ip, 2);
  const int nx = node_of(-s0, s1, s2), ny = node_of(s0, -s1, s2), nz = node_of(s0, s1, -s2);
  const int nxy = node_of(-s0, -s1, s2), nxz = node_of(-s0, s1, -s2), nyz = node_of(s0, -s1, -s2);
  double h[8][3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double xb = ((c[0][d] + c[1][d]) + (c[2][d] + c[3][d]) + ((c[4][d] + c[5][d]) + (c[6][d] + c[7][d]))) * 0.125;
    const double y0 = c[ip][d] - xb, yx = c[nx][d] - xb, yy = c[ny][d] - xb, yz = c[nz][d] - xb;
    const double yxy = c[nxy][d] - xb, yxz = c[nxz][d] - xb, yyz = c[nyz][d] - xb;
    h[0][d] = 0.0;                                   // centre
    h[1][d] = ((y0 + yy) + (yz + yyz)) * 0.25;       // y, z middle: face centroid normal to x
    h[2][d] = (y0 + yz) * 0.5;                       // z middle: edge midpoint
    h[3][d] = ((y0 + yx) + (yz + yxz)) * 0.25;       // x, z middle
    h[4][d] = ((y0 + yx) + (yy + yxy)) * 0.25;       // x, y middle
    h[5][d] = (y0 + yy) * 0.5;                       // y middle
    h[6][d] = y0;                                    // node ip
    h[7][d] = (y0 + yx) * 0.5;                       // x middle
  }
  constexpr int kF[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
  double v = 0.0;
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const double* a = h[kF[f][0]];
    const double* b = h[kF[f][1]];
    const double* cc = h[kF[f][2]];
    const double* dd = h[kF[f][3]];
    const double p0 = cc[0] - a[0], p1 = cc[1] - a[1], p2 = cc[2] - a[2];
    const double q0 = dd[0] - b[0], q1 = dd[1] - b[1], q2 = dd[2] - b[2];
    const double m0 = (a[0] + b[0]) + (cc[0] + dd[0]), m1 = (a[1] + b[1]) + (cc[1] + dd[1]),
                 m2 = (a[2] + b[2]) + (cc[2] + dd[2]);
    v += (p1 * q2 - p2 * q1) * m0 + (p2 * q0 - p0 * q2) * m1 + (p0 * q1 - p1 * q0) * m2;
  }
  return (s0 * s1 * s2) * v * (1.0 / 24.0);
}

}  // namespace
}  // namespace nalu_gb300
