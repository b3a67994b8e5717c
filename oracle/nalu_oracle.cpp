// nalu_oracle.cpp -- CPU FP64 oracle (TEST INFRASTRUCTURE ONLY).
//
// Restates, in plain C++, the NaluCFD/Nalu algorithms on the Hex8 CVFEM
// assembly + continuity solve path.  Every routine names the reference
// file:line it follows and keeps that code's floating-point operation order.
// Build with -ffp-contract=off so no multiply-add is fused; the results then
// match the reference's own compiled code bit for bit on x86-64 and aarch64.
//
// Only the tests, the smoke check and the CPU-baseline leg of the benchmark
// load this library.  It is the checker, never the thing measured as the
// product or shipped behind the product's C ABI.

#include "nalu_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>
#include <map>
#include <array>

namespace {

// ---------------------------------------------------------------------------
// HexSCS / HexSCV constant tables.
// lrscv_            : src/master_element/Hex8CVFEM.C:265-276
// intgLoc_ (SCS)    : src/master_element/Hex8CVFEM.C:319-331
// intgLocShift_(SCS): src/master_element/Hex8CVFEM.C:334-346
// intgLoc_ (SCV)    : src/master_element/Hex8CVFEM.C:90-98
// intgLocShift_(SCV): src/master_element/Hex8CVFEM.C:101-109
// ---------------------------------------------------------------------------
const int kLrscv[24] = {0, 1, 1, 2, 2, 3, 0, 3, 4, 5, 5, 6,
                        6, 7, 4, 7, 0, 4, 1, 5, 2, 6, 3, 7};

const double kScsLoc[36] = {
    0.00, -0.25, -0.25, 0.25, 0.00, -0.25, 0.00, 0.25, -0.25, -0.25, 0.00, -0.25,
    0.00, -0.25, 0.25,  0.25, 0.00, 0.25,  0.00, 0.25, 0.25,  -0.25, 0.00, 0.25,
    -0.25, -0.25, 0.00, 0.25, -0.25, 0.00, 0.25, 0.25, 0.00,  -0.25, 0.25, 0.00};

const double kScsLocShift[36] = {
    0.00, -0.50, -0.50, 0.50, 0.00, -0.50, 0.00, 0.50, -0.50, -0.50, 0.00, -0.50,
    0.00, -0.50, 0.50,  0.50, 0.00, 0.50,  0.00, 0.50, 0.50,  -0.50, 0.00, 0.50,
    -0.50, -0.50, 0.00, 0.50, -0.50, 0.00, 0.50, 0.50, 0.00,  -0.50, 0.50, 0.00};

const double kScvLoc[24] = {-0.25, -0.25, -0.25, +0.25, -0.25, -0.25, +0.25, +0.25,
                            -0.25, -0.25, +0.25, -0.25, -0.25, -0.25, +0.25, +0.25,
                            -0.25, +0.25, +0.25, +0.25, +0.25, -0.25, +0.25, +0.25};

const double kScvLocShift[24] = {-0.5, -0.5, -0.5, +0.5, -0.5, -0.5, +0.5, +0.5,
                                 -0.5, -0.5, +0.5, -0.5, -0.5, -0.5, +0.5, +0.5,
                                 -0.5, +0.5, +0.5, +0.5, +0.5, -0.5, +0.5, +0.5};

// tiny_positive_value() of include/master_element/MasterElement.h
inline double tiny_positive_value() { return 1.0e-50; }

// ---------------------------------------------------------------------------
// subdivide_hex_8: include/master_element/Hex8GeometryFunctions.h:263-322
// ---------------------------------------------------------------------------
void subdivide_hex_8(const double* coords, double coordv[27][3]) {
  auto c = [&](int n, int d) { return coords[n * 3 + d]; };
  for (int n = 0; n < 8; ++n) {
    coordv[n][0] = c(n, 0);
    coordv[n][1] = c(n, 1);
    coordv[n][2] = c(n, 2);
  }
  for (int d = 0; d < 3; ++d) {
    coordv[8][d] = 0.5 * (c(0, d) + c(1, d));
    coordv[9][d] = 0.5 * (c(1, d) + c(2, d));
    coordv[10][d] = 0.5 * (c(2, d) + c(3, d));
    coordv[11][d] = 0.5 * (c(3, d) + c(0, d));
    coordv[12][d] = 0.25 * (c(0, d) + c(1, d) + c(2, d) + c(3, d));
    coordv[13][d] = 0.5 * (c(4, d) + c(5, d));
    coordv[14][d] = 0.5 * (c(5, d) + c(6, d));
    coordv[15][d] = 0.5 * (c(6, d) + c(7, d));
    coordv[16][d] = 0.5 * (c(7, d) + c(4, d));
    coordv[17][d] = 0.25 * (c(4, d) + c(5, d) + c(6, d) + c(7, d));
    coordv[18][d] = 0.5 * (c(1, d) + c(5, d));
    coordv[19][d] = 0.5 * (c(0, d) + c(4, d));
    coordv[20][d] = 0.25 * (c(0, d) + c(1, d) + c(4, d) + c(5, d));
    coordv[21][d] = 0.5 * (c(3, d) + c(7, d));
    coordv[22][d] = 0.5 * (c(2, d) + c(6, d));
    coordv[23][d] = 0.25 * (c(2, d) + c(3, d) + c(6, d) + c(7, d));
    coordv[24][d] = 0.25 * (c(1, d) + c(2, d) + c(5, d) + c(6, d));
    coordv[25][d] = 0.25 * (c(0, d) + c(3, d) + c(4, d) + c(7, d));
    coordv[26][d] = 0.;
    for (int n = 0; n < 8; ++n) coordv[26][d] += c(n, d);
    coordv[26][d] *= 0.125;
  }
}

// quad_area_by_triangulation: include/master_element/Hex8GeometryFunctions.h:30-76
void quad_area_by_triangulation(int ics, const double a[4][3], double* area) {
  double* ar = area + 3 * ics;
  ar[0] = 0.0;
  ar[1] = 0.0;
  ar[2] = 0.0;
  const double xmid[3] = {0.25 * (a[0][0] + a[1][0] + a[2][0] + a[3][0]),
                          0.25 * (a[0][1] + a[1][1] + a[2][1] + a[3][1]),
                          0.25 * (a[0][2] + a[1][2] + a[2][2] + a[3][2])};
  double r1[3] = {a[0][0] - xmid[0], a[0][1] - xmid[1], a[0][2] - xmid[2]};
  for (int it = 0; it < 4; ++it) {
    const int t = (it + 1) % 4;
    const double r2[3] = {a[t][0] - xmid[0], a[t][1] - xmid[1], a[t][2] - xmid[2]};
    ar[0] += r1[1] * r2[2] - r2[1] * r1[2];
    ar[1] += r1[2] * r2[0] - r2[2] * r1[0];
    ar[2] += r1[0] * r2[1] - r2[0] * r1[1];
    r1[0] = r2[0];
    r1[1] = r2[1];
    r1[2] = r2[2];
  }
  ar[0] *= 0.5;
  ar[1] *= 0.5;
  ar[2] *= 0.5;
}

// hex_volume_grandy: include/master_element/Hex8GeometryFunctions.h:78-163
double hex_volume_grandy(const double scv[8][3]) {
  double cv[14][3];
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) cv[n][d] = scv[n][d];
  const int fn[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4},
                        {2, 3, 7, 6}, {1, 2, 6, 5}, {0, 4, 3, 7}};
  for (int k = 0; k < 6; ++k)
    for (int d = 0; d < 3; ++d)
      cv[k + 8][d] = 0.25 * (cv[fn[k][0]][d] + cv[fn[k][1]][d] + cv[fn[k][2]][d] + cv[fn[k][3]][d]);
  const int tf[24][3] = {{0, 8, 1},   {8, 2, 1},   {3, 2, 8},   {3, 8, 0},   {6, 9, 5},
                         {7, 9, 6},   {4, 9, 7},   {4, 5, 9},   {10, 0, 1},  {5, 10, 1},
                         {4, 10, 5},  {4, 0, 10},  {7, 6, 11},  {6, 2, 11},  {2, 3, 11},
                         {3, 7, 11},  {6, 12, 2},  {5, 12, 6},  {5, 1, 12},  {1, 2, 12},
                         {0, 4, 13},  {4, 7, 13},  {7, 3, 13},  {3, 0, 13}};
  double volume = 0.0;
  for (int k = 0; k < 24; ++k) {
    const int p = tf[k][0], q = tf[k][1], r = tf[k][2];
    const double mid[3] = {cv[p][0] + cv[q][0] + cv[r][0], cv[p][1] + cv[q][1] + cv[r][1],
                           cv[p][2] + cv[q][2] + cv[r][2]};
    double dxv[3];
    dxv[0] = (cv[q][1] - cv[p][1]) * (cv[r][2] - cv[p][2]) - (cv[r][1] - cv[p][1]) * (cv[q][2] - cv[p][2]);
    dxv[1] = (cv[r][0] - cv[p][0]) * (cv[q][2] - cv[p][2]) - (cv[q][0] - cv[p][0]) * (cv[r][2] - cv[p][2]);
    dxv[2] = (cv[q][0] - cv[p][0]) * (cv[r][1] - cv[p][1]) - (cv[r][0] - cv[p][0]) * (cv[q][1] - cv[p][1]);
    volume += mid[0] * dxv[0] + mid[1] * dxv[1] + mid[2] * dxv[2];
  }
  volume /= 18.0;
  return volume;
}

// shape functions for the 12 SCS ips (standard or shifted), Hex8CVFEM.C:469-517
void scs_shape(bool shifted, double shp[96]) {
  orc_hex8_shape_fcn(12, shifted ? kScsLocShift : kScsLoc, shp);
}

// grad op at the SCS ips (Hex8CVFEM.C:523-541)
void scs_grad(const double* coords, bool shifted, double dndx[288]) {
  double deriv[288];
  orc_hex_scs_grad_op(coords, shifted ? 1 : 0, dndx, deriv);
}

// ---- tiny thread pool helper (the CPU baseline runs on all host cores) ----
template <class F>
void parallel_for(int64_t n, int n_threads, F f) {
  if (n_threads <= 1 || n < 1024) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  const int64_t chunk = (n + n_threads - 1) / n_threads;
  for (int t = 0; t < n_threads; ++t) {
    const int64_t b = t * chunk, e = std::min<int64_t>(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([=]() { f(b, e); });
  }
  for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

void orc_hex_scs_tables(int* lrscv24, double* loc36, double* locs36) {
  if (lrscv24) std::memcpy(lrscv24, kLrscv, sizeof(kLrscv));
  if (loc36) std::memcpy(loc36, kScsLoc, sizeof(kScsLoc));
  if (locs36) std::memcpy(locs36, kScsLocShift, sizeof(kScsLocShift));
}

// HexSCS::hex8_shape_fcn: src/master_element/Hex8CVFEM.C:487-517
void orc_hex8_shape_fcn(int npts, const double* iso, double* shape) {
  const double half = 0.50, one4th = 0.25, one8th = 0.125;
  for (int j = 0; j < npts; ++j) {
    const double s1 = iso[j * 3], s2 = iso[j * 3 + 1], s3 = iso[j * 3 + 2];
    double* sh = shape + 8 * j;
    sh[0] = one8th + one4th * (-s1 - s2 - s3) + half * (s2 * s3 + s3 * s1 + s1 * s2) - s1 * s2 * s3;
    sh[1] = one8th + one4th * (s1 - s2 - s3) + half * (s2 * s3 - s3 * s1 - s1 * s2) + s1 * s2 * s3;
    sh[2] = one8th + one4th * (s1 + s2 - s3) + half * (-s2 * s3 - s3 * s1 + s1 * s2) - s1 * s2 * s3;
    sh[3] = one8th + one4th * (-s1 + s2 - s3) + half * (-s2 * s3 + s3 * s1 - s1 * s2) + s1 * s2 * s3;
    sh[4] = one8th + one4th * (-s1 - s2 + s3) + half * (-s2 * s3 - s3 * s1 + s1 * s2) + s1 * s2 * s3;
    sh[5] = one8th + one4th * (s1 - s2 + s3) + half * (-s2 * s3 + s3 * s1 - s1 * s2) - s1 * s2 * s3;
    sh[6] = one8th + one4th * (s1 + s2 + s3) + half * (s2 * s3 + s3 * s1 + s1 * s2) + s1 * s2 * s3;
    sh[7] = one8th + one4th * (-s1 + s2 + s3) + half * (s2 * s3 - s3 * s1 - s1 * s2) - s1 * s2 * s3;
  }
}

// hex8_derivative: src/master_element/Hex8CVFEM.C:25-70
void orc_hex8_derivative(int npts, const double* loc, double* deriv) {
  const double half = 0.50, one4th = 0.25;
  for (int ip = 0; ip < npts; ++ip) {
    const double s1 = loc[ip * 3], s2 = loc[ip * 3 + 1], s3 = loc[ip * 3 + 2];
    const double s1s2 = s1 * s2, s2s3 = s2 * s3, s1s3 = s1 * s3;
    double* d = deriv + ip * 24;
    d[0 * 3 + 0] = half * (s3 + s2) - s2s3 - one4th;
    d[1 * 3 + 0] = half * (-s3 - s2) + s2s3 + one4th;
    d[2 * 3 + 0] = half * (-s3 + s2) - s2s3 + one4th;
    d[3 * 3 + 0] = half * (s3 - s2) + s2s3 - one4th;
    d[4 * 3 + 0] = half * (-s3 + s2) + s2s3 - one4th;
    d[5 * 3 + 0] = half * (s3 - s2) - s2s3 + one4th;
    d[6 * 3 + 0] = half * (s3 + s2) + s2s3 + one4th;
    d[7 * 3 + 0] = half * (-s3 - s2) - s2s3 - one4th;

    d[0 * 3 + 1] = half * (s3 + s1) - s1s3 - one4th;
    d[1 * 3 + 1] = half * (s3 - s1) + s1s3 - one4th;
    d[2 * 3 + 1] = half * (-s3 + s1) - s1s3 + one4th;
    d[3 * 3 + 1] = half * (-s3 - s1) + s1s3 + one4th;
    d[4 * 3 + 1] = half * (-s3 + s1) + s1s3 - one4th;
    d[5 * 3 + 1] = half * (-s3 - s1) - s1s3 - one4th;
    d[6 * 3 + 1] = half * (s3 + s1) + s1s3 + one4th;
    d[7 * 3 + 1] = half * (s3 - s1) - s1s3 + one4th;

    d[0 * 3 + 2] = half * (s2 + s1) - s1s2 - one4th;
    d[1 * 3 + 2] = half * (s2 - s1) + s1s2 - one4th;
    d[2 * 3 + 2] = half * (-s2 - s1) - s1s2 - one4th;
    d[3 * 3 + 2] = half * (-s2 + s1) + s1s2 - one4th;
    d[4 * 3 + 2] = half * (-s2 - s1) + s1s2 + one4th;
    d[5 * 3 + 2] = half * (-s2 + s1) - s1s2 + one4th;
    d[6 * 3 + 2] = half * (s2 + s1) + s1s2 + one4th;
    d[7 * 3 + 2] = half * (s2 - s1) - s1s2 + one4th;
  }
}

// generic_grad_op<AlgTraitsHex8>: include/master_element/MasterElementFunctions.h:51-108
// (cofactorMatrix: :31-43)
int orc_generic_grad_op(int npts, const double* deriv, const double* coords, double* gradop,
                        double* detj_out) {
  int nbad = 0;
  for (int ip = 0; ip < npts; ++ip) {
    double jact[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) jact[i][j] = 0.0;
    double refGrad[8][3];
    for (int n = 0; n < 8; ++n) {
      for (int i = 0; i < 3; ++i) refGrad[n][i] = deriv[ip * 24 + n * 3 + i];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) jact[i][j] += refGrad[n][j] * coords[n * 3 + i];
    }
    double adj[3][3];
    adj[0][0] = jact[1][1] * jact[2][2] - jact[2][1] * jact[1][2];
    adj[0][1] = jact[1][2] * jact[2][0] - jact[2][2] * jact[1][0];
    adj[0][2] = jact[1][0] * jact[2][1] - jact[2][0] * jact[1][1];
    adj[1][0] = jact[0][2] * jact[2][1] - jact[2][2] * jact[0][1];
    adj[1][1] = jact[0][0] * jact[2][2] - jact[2][0] * jact[0][2];
    adj[1][2] = jact[0][1] * jact[2][0] - jact[2][1] * jact[0][0];
    adj[2][0] = jact[0][1] * jact[1][2] - jact[1][1] * jact[0][2];
    adj[2][1] = jact[0][2] * jact[1][0] - jact[1][2] * jact[0][0];
    adj[2][2] = jact[0][0] * jact[1][1] - jact[1][0] * jact[0][1];
    double det = 0.0;
    for (int i = 0; i < 3; ++i) det += jact[i][0] * adj[i][0];
    if (!(det > tiny_positive_value())) ++nbad;
    if (detj_out) detj_out[ip] = det;
    const double inv_detj = 1.0 / det;
    for (int n = 0; n < 8; ++n) {
      for (int i = 0; i < 3; ++i) {
        double w = 0.0;
        for (int j = 0; j < 3; ++j) w += adj[i][j] * refGrad[n][j];
        w *= inv_detj;
        gradop[ip * 24 + n * 3 + i] = w;
      }
    }
  }
  return nbad;
}

// HexSCS::grad_op / shifted_grad_op: src/master_element/Hex8CVFEM.C:523-541
int orc_hex_scs_grad_op(const double* coords, int shifted, double* gradop, double* deriv) {
  orc_hex8_derivative(12, shifted ? kScsLocShift : kScsLoc, deriv);
  return orc_generic_grad_op(12, deriv, coords, gradop, nullptr);
}

// HexSCV::grad_op / shifted_grad_op: src/master_element/Hex8CVFEM.C:185-192, 225-232
int orc_hex_scv_grad_op(const double* coords, int shifted, double* gradop, double* deriv) {
  orc_hex8_derivative(8, shifted ? kScvLocShift : kScvLoc, deriv);
  return orc_generic_grad_op(8, deriv, coords, gradop, nullptr);
}

// HexSCS::determinant (area vectors): src/master_element/Hex8CVFEM.C:547-580
void orc_hex_scs_areav(const double* coords, double* areav) {
  const int table[12][4] = {{20, 8, 12, 26}, {24, 9, 12, 26},  {10, 12, 26, 23}, {11, 25, 26, 12},
                            {13, 20, 26, 17}, {17, 14, 24, 26}, {17, 15, 23, 26}, {16, 17, 26, 25},
                            {19, 20, 26, 25}, {20, 18, 24, 26}, {22, 23, 26, 24}, {21, 25, 26, 23}};
  double cv[27][3];
  subdivide_hex_8(coords, cv);
  for (int ics = 0; ics < 12; ++ics) {
    double sc[4][3];
    for (int n = 0; n < 4; ++n)
      for (int d = 0; d < 3; ++d) sc[n][d] = cv[table[ics][n]][d];
    quad_area_by_triangulation(ics, sc, areav);
  }
}

// HexSCV::determinant (sub-control volumes): src/master_element/Hex8CVFEM.C:149-180
void orc_hex_scv_volume(const double* coords, double* volume) {
  const int sub[8][8] = {{0, 8, 12, 11, 19, 20, 26, 25},  {8, 1, 9, 12, 20, 18, 24, 26},
                         {12, 9, 2, 10, 26, 24, 22, 23},  {11, 12, 10, 3, 25, 26, 23, 21},
                         {19, 20, 26, 25, 4, 13, 17, 16}, {20, 18, 24, 26, 13, 5, 14, 17},
                         {26, 24, 22, 23, 17, 14, 6, 15}, {25, 26, 23, 21, 16, 17, 15, 7}};
  double cv[27][3];
  subdivide_hex_8(coords, cv);
  for (int ip = 0; ip < 8; ++ip) {
    double h[8][3];
    for (int n = 0; n < 8; ++n)
      for (int d = 0; d < 3; ++d) h[n][d] = cv[sub[ip][n]][d];
    volume[ip] = hex_volume_grandy(h);
  }
}

// SCV shape functions: HexSCV::shape_fcn / shifted_shape_fcn
// (src/master_element/Hex8CVFEM.C:236-250, ips at :89-107), ip i in the
// octant of node i
static void scv_shape(int lumped, double* shp /*[8][8]*/) {
  const double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
               sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
  const double a = lumped ? 0.5 : 0.25;
  double iso[24];
  for (int ip = 0; ip < 8; ++ip) {
    iso[3 * ip] = sx[ip] * a;
    iso[3 * ip + 1] = sy[ip] * a;
    iso[3 * ip + 2] = sz[ip] * a;
  }
  orc_hex8_shape_fcn(8, iso, shp);
}

// ContinuityMassElemKernel::execute (src/kernel/ContinuityMassElemKernel.C:84-120)
void orc_continuity_mass_elem(const double* coords, const double* rho_nm1, const double* rho_n,
                              const double* rho_np1, double dt, double gamma1, double gamma2, double gamma3,
                              int lumped, double* lhs, double* rhs) {
  double shp[64], scv[8];
  scv_shape(lumped, shp);
  orc_hex_scv_volume(coords, scv);
  for (int i = 0; i < 64; ++i) lhs[i] = 0.0;
  for (int i = 0; i < 8; ++i) rhs[i] = 0.0;
  const double proj_time_scale = dt / gamma1;
  for (int ip = 0; ip < 8; ++ip) {
    double rNm1 = 0.0, rN = 0.0, rNp1 = 0.0;
    for (int ic = 0; ic < 8; ++ic) {
      const double r = shp[8 * ip + ic];
      rNm1 += r * rho_nm1[ic];
      rN += r * rho_n[ic];
      rNp1 += r * rho_np1[ic];
    }
    rhs[ip] += -(gamma1 * rNp1 + gamma2 * rN + gamma3 * rNm1) * scv[ip] / dt / proj_time_scale;
  }
}

// MomentumMassElemKernel::execute (src/kernel/MomentumMassElemKernel.C:100-171)
void orc_momentum_mass_elem(const double* coords, const double* rho_nm1, const double* rho_n,
                            const double* rho_np1, const double* u_nm1, const double* u_n,
                            const double* u_np1, const double* gpdx, double dt, double gamma1,
                            double gamma2, double gamma3, int lumped, int balanced_force, double* lhs,
                            double* rhs) {
  double shp[64], scv[8];
  scv_shape(lumped, shp);
  orc_hex_scv_volume(coords, scv);
  for (int i = 0; i < 576; ++i) lhs[i] = 0.0;
  for (int i = 0; i < 24; ++i) rhs[i] = 0.0;
  const double dens_fac_on = balanced_force ? 1.0 : 0.0, om_dens_fac = balanced_force ? 0.0 : 1.0;
  for (int ip = 0; ip < 8; ++ip) {
    double rNm1 = 0.0, rN = 0.0, rNp1 = 0.0, uNm1[3] = {0, 0, 0}, uN[3] = {0, 0, 0}, uNp1[3] = {0, 0, 0},
           g[3] = {0, 0, 0};
    for (int ic = 0; ic < 8; ++ic) {
      const double r = shp[8 * ip + ic];
      rNm1 += r * rho_nm1[ic];
      rN += r * rho_n[ic];
      rNp1 += r * rho_np1[ic];
      for (int j = 0; j < 3; ++j) {
        uNm1[j] += r * u_nm1[3 * ic + j];
        uN[j] += r * u_n[3 * ic + j];
        uNp1[j] += r * u_np1[3 * ic + j];
        g[j] += r * gpdx[3 * ic + j];
      }
    }
    const double scV = scv[ip];
    const double dens_fac = rNp1 * dens_fac_on + om_dens_fac;
    for (int j = 0; j < 3; ++j)
      rhs[3 * ip + j] += -(gamma1 * rNp1 * uNp1[j] + gamma2 * rN * uN[j] + gamma3 * rNm1 * uNm1[j]) * scV / dt -
                         g[j] * scV * dens_fac;
    for (int ic = 0; ic < 8; ++ic) {
      const double lhsfac = shp[8 * ip + ic] * gamma1 * rNp1 * scV / dt;
      for (int j = 0; j < 3; ++j) lhs[(3 * ip + j) * 24 + 3 * ic + j] += lhsfac;
    }
  }
}

// ComputeGeometryInteriorAlgorithm (src/ComputeGeometryInteriorAlgorithm.C):
// dualNodalVolume[ipNodeMap[ip]] += scv_volume[ip], element order
void orc_dual_volume(int64_t n_nodes, int64_t n_elems, const int32_t* conn, const double* coords, double* vol) {
  for (int64_t i = 0; i < n_nodes; ++i) vol[i] = 0.0;
  for (int64_t e = 0; e < n_elems; ++e) {
    double c[24], v[8];
    for (int n = 0; n < 8; ++n)
      for (int d = 0; d < 3; ++d) c[3 * n + d] = coords[3 * (int64_t)conn[8 * e + n] + d];
    orc_hex_scv_volume(c, v);
    for (int n = 0; n < 8; ++n) vol[conn[8 * e + n]] += v[n];
  }
}

// AssembleNodalGradElemAlgorithm::execute (src/AssembleNodalGradElemAlgorithm.C:
// the nodalGradientElem functor): qIp = sum N q; grad[il] += qIp A / V_il,
// grad[ir] -= qIp A / V_ir; ncomp = 3 is the velocity form (dudx[i][j])
void orc_nodal_grad_elem(int64_t n_nodes, int64_t n_elems, const int32_t* conn, const double* coords,
                         const double* q, int ncomp, const double* dual_volume, int shifted, double* grad) {
  const int64_t w = 3 * (int64_t)ncomp;
  for (int64_t i = 0; i < n_nodes * w; ++i) grad[i] = 0.0;
  double shp[96];
  scs_shape(shifted != 0, shp);
  for (int64_t e = 0; e < n_elems; ++e) {
    const int32_t* nd = conn + 8 * e;
    double c[24], areav[36];
    for (int n = 0; n < 8; ++n)
      for (int d = 0; d < 3; ++d) c[3 * n + d] = coords[3 * (int64_t)nd[n] + d];
    orc_hex_scs_areav(c, areav);
    for (int ip = 0; ip < 12; ++ip) {
      const int il = kLrscv[2 * ip], ir = kLrscv[2 * ip + 1];
      const double inv_l = 1.0 / dual_volume[nd[il]], inv_r = 1.0 / dual_volume[nd[ir]];
      for (int k = 0; k < ncomp; ++k) {
        double qip = 0.0;
        for (int ic = 0; ic < 8; ++ic) qip += shp[ip * 8 + ic] * q[(int64_t)nd[ic] * ncomp + k];
        for (int j = 0; j < 3; ++j) {
          const double fac = qip * areav[ip * 3 + j];
          grad[(int64_t)nd[il] * w + 3 * k + j] += fac * inv_l;
          grad[(int64_t)nd[ir] * w + 3 * k + j] -= fac * inv_r;
        }
      }
    }
  }
}

// ScalarDiffElemKernel::execute: src/kernel/ScalarDiffElemKernel.C:66-110
void orc_scalar_diff_elem(const double* coords, const double* q, const double* dk,
                          int shifted_grad_op, double* lhs, double* rhs) {
  double shp[96], areav[36], dndx[288];
  scs_shape(false, shp);  // kernel ctor: shape_fcn, :46
  orc_hex_scs_areav(coords, areav);
  scs_grad(coords, shifted_grad_op != 0, dndx);
  for (int i = 0; i < 64; ++i) lhs[i] = 0.0;
  for (int i = 0; i < 8; ++i) rhs[i] = 0.0;
  for (int ip = 0; ip < 12; ++ip) {
    const int il = kLrscv[2 * ip], ir = kLrscv[2 * ip + 1];
    double kIp = 0.0;
    for (int ic = 0; ic < 8; ++ic) {
      const double r = shp[ip * 8 + ic];
      kIp += r * dk[ic];
    }
    double qDiff = 0.0;
    for (int ic = 0; ic < 8; ++ic) {
      double lhsfac = 0.0;
      for (int j = 0; j < 3; ++j) lhsfac += -kIp * dndx[ip * 24 + ic * 3 + j] * areav[ip * 3 + j];
      qDiff += lhsfac * q[ic];
      lhs[il * 8 + ic] += lhsfac;
      lhs[ir * 8 + ic] -= lhsfac;
    }
    rhs[il] -= qDiff;
    rhs[ir] += qDiff;
  }
}

// ContinuityAdvElemKernel::setup/execute: src/kernel/ContinuityAdvElemKernel.C:79-147
void orc_continuity_adv_elem(const double* coords, const double* vel, const double* rho,
                             const double* p, const double* gpdx, double tau, int shift_mdot,
                             int shift_poisson, int reduced_sens, double* lhs, double* rhs) {
  double shp[96], areav[36], dndx[288], dndxs[288];
  scs_shape(shift_mdot != 0, shp);  // ctor :74-77
  orc_hex_scs_areav(coords, areav);
  scs_grad(coords, false, dndx);
  scs_grad(coords, true, dndxs);
  const double* v_dndx = shift_poisson ? dndxs : dndx;                     // :103-104
  const double* v_dndx_lhs = (shift_poisson || reduced_sens) ? dndxs : dndx;  // :105-106
  for (int i = 0; i < 64; ++i) lhs[i] = 0.0;
  for (int i = 0; i < 8; ++i) rhs[i] = 0.0;
  for (int ip = 0; ip < 12; ++ip) {
    const int il = kLrscv[2 * ip], ir = kLrscv[2 * ip + 1];
    double rho_u[3] = {0, 0, 0}, gp[3] = {0, 0, 0}, dpdx[3] = {0, 0, 0};
    for (int ic = 0; ic < 8; ++ic) {
      const double r = shp[ip * 8 + ic];
      const double np = p[ic], nr = rho[ic];
      double lhsfac = 0.0;
      for (int j = 0; j < 3; ++j) {
        gp[j] += r * gpdx[ic * 3 + j];
        rho_u[j] += r * nr * vel[ic * 3 + j];
        dpdx[j] += v_dndx[ip * 24 + ic * 3 + j] * np;
        lhsfac += -v_dndx_lhs[ip * 24 + ic * 3 + j] * areav[ip * 3 + j];
      }
      lhs[il * 8 + ic] += lhsfac;
      lhs[ir * 8 + ic] -= lhsfac;
    }
    double mdot = 0.0;
    for (int j = 0; j < 3; ++j) mdot += (rho_u[j] - tau * (dpdx[j] - gp[j])) * areav[ip * 3 + j];
    rhs[il] -= mdot / tau;
    rhs[ir] += mdot / tau;
  }
}

// MomentumAdvDiffElemKernel::execute: src/kernel/MomentumAdvDiffElemKernel.C:72-185
void orc_momentum_adv_diff_elem(const double* coords, const double* u, const double* mu,
                                const double* mdot, double include_divu, int shifted_grad_op,
                                int skew_symmetric, double* lhs, double* rhs) {
  double shp[96], shpAdv[96], areav[36], dndx[288];
  scs_shape(false, shp);
  scs_shape(skew_symmetric != 0, shpAdv);  // ctor :47-49
  orc_hex_scs_areav(coords, areav);
  scs_grad(coords, shifted_grad_op != 0, dndx);
  for (int i = 0; i < 576; ++i) lhs[i] = 0.0;
  for (int i = 0; i < 24; ++i) rhs[i] = 0.0;
  auto L = [&](int r, int c) -> double& { return lhs[r * 24 + c]; };
  for (int ip = 0; ip < 12; ++ip) {
    const int il = kLrscv[2 * ip], ir = kLrscv[2 * ip + 1];
    const int ilN = il * 3, irN = ir * 3;
    const double tmdot = mdot[ip];
    double muIp = 0.0, divU = 0.0, uIp[3] = {0, 0, 0};
    for (int ic = 0; ic < 8; ++ic) {
      const double r = shp[ip * 8 + ic], rAdv = shpAdv[ip * 8 + ic];
      muIp += r * mu[ic];
      for (int j = 0; j < 3; ++j) {
        const double uj = u[ic * 3 + j];
        uIp[j] += rAdv * uj;
        divU += uj * dndx[ip * 24 + ic * 3 + j];
      }
    }
    for (int i = 0; i < 3; ++i) {
      const double aflux = tmdot * uIp[i];
      const double divUstress = 2.0 / 3.0 * muIp * divU * areav[ip * 3 + i] * include_divu;
      rhs[ilN + i] -= aflux + divUstress;
      rhs[irN + i] += aflux + divUstress;
    }
    for (int ic = 0; ic < 8; ++ic) {
      const int icN = ic * 3;
      const double lhsfacAdv = shpAdv[ip * 8 + ic] * tmdot;
      for (int i = 0; i < 3; ++i) {
        const int iL = ilN + i, iR = irN + i;
        L(iL, icN + i) += lhsfacAdv;
        L(iR, icN + i) -= lhsfacAdv;
        double lhs_riC_i = 0.0;
        for (int j = 0; j < 3; ++j) {
          const double axj = areav[ip * 3 + j];
          const double uj = u[ic * 3 + j];
          const double lhsfacDiff_i = -muIp * dndx[ip * 24 + ic * 3 + j] * axj;
          lhs_riC_i += lhsfacDiff_i;
          const double lhsfacDiff_j = -muIp * dndx[ip * 24 + ic * 3 + i] * axj;
          L(iL, icN + j) += lhsfacDiff_j;
          L(iR, icN + j) -= lhsfacDiff_j;
          rhs[iL] -= lhsfacDiff_j * uj;
          rhs[iR] += lhsfacDiff_j * uj;
        }
        L(iL, icN + i) += lhs_riC_i;
        L(iR, icN + i) -= lhs_riC_i;
        const double ui = u[ic * 3 + i];
        rhs[iL] -= lhs_riC_i * ui;
        rhs[iR] += lhs_riC_i * ui;
      }
    }
  }
}

// MomentumUpwAdvDiffElemKernel::setup/execute/van_leer:
// src/kernel/MomentumUpwAdvDiffElemKernel.C:90-320; ClassicPecletFunction::execute:
// src/PecletFunction.C:77-82 (created with A=5, hf=hybrid factor, src/EquationSystem.C:310-318)
void orc_momentum_upw_adv_diff_elem(const double* coords, const double* u, const double* vrtm,
                                    const double* rho, const double* mu, const double* gju,
                                    const double* mdot, double include_divu, int shifted_grad_op,
                                    int skew_symmetric, double alpha, double alphaUpw,
                                    double hoUpwind, double hf, int useLimiter, double* lhs,
                                    double* rhs) {
  const double small_ = 1.0e-16;  // include/kernel/MomentumUpwAdvDiffElemKernel.h:85
  const double om_alpha = 1.0 - alpha, om_alphaUpw = 1.0 - alphaUpw;
  double shp[96], shpAdv[96], areav[36], dndx[288];
  scs_shape(false, shp);
  scs_shape(skew_symmetric != 0, shpAdv);
  orc_hex_scs_areav(coords, areav);
  scs_grad(coords, shifted_grad_op != 0, dndx);
  for (int i = 0; i < 576; ++i) lhs[i] = 0.0;
  for (int i = 0; i < 24; ++i) rhs[i] = 0.0;
  auto L = [&](int r, int c) -> double& { return lhs[r * 24 + c]; };
  auto X = [&](int n, int d) { return coords[n * 3 + d]; };
  auto G = [&](int n, int i, int j) { return gju[n * 9 + i * 3 + j]; };
  auto van_leer = [&](double dqm, double dqp) {
    return (2.0 * (dqm * dqp + std::fabs(dqm * dqp))) / ((dqm + dqp) * (dqm + dqp) + small_);
  };
  double limitL[3] = {1.0, 1.0, 1.0}, limitR[3] = {1.0, 1.0, 1.0};
  for (int ip = 0; ip < 12; ++ip) {
    const int il = kLrscv[2 * ip], ir = kLrscv[2 * ip + 1];
    const int ilN = il * 3, irN = ir * 3;
    const double tmdot = mdot[ip];
    double muIp = 0.0, divU = 0.0, uIp[3] = {0, 0, 0}, cIp[3] = {0, 0, 0};
    for (int ic = 0; ic < 8; ++ic) {
      const double r = shp[ip * 8 + ic], rAdv = shpAdv[ip * 8 + ic];
      muIp += r * mu[ic];
      for (int j = 0; j < 3; ++j) {
        const double uj = u[ic * 3 + j];
        uIp[j] += rAdv * uj;
        cIp[j] += rAdv * X(ic, j);
        divU += uj * dndx[ip * 24 + ic * 3 + j];
      }
    }
    double udotx = 0.0, duL[3], duR[3];
    for (int i = 0; i < 3; ++i) {
      const double dxi = X(ir, i) - X(il, i);
      const double ui = 0.5 * (vrtm[il * 3 + i] + vrtm[ir * 3 + i]);
      udotx += ui * dxi;
      duL[i] = 0.0;
      duR[i] = 0.0;
      for (int j = 0; j < 3; ++j) {
        const double dxjL = cIp[j] - X(il, j);
        const double dxjR = X(ir, j) - cIp[j];
        duL[i] += dxjL * G(il, i, j);
        duR[i] += dxjR * G(ir, i, j);
      }
    }
    const double diffIp = 0.5 * (mu[il] / rho[il] + mu[ir] / rho[ir]);
    const double pecArg = std::fabs(udotx) / (diffIp + small_);
    const double modPe = hf * pecArg;
    const double pecfac = modPe * modPe / (5.0 + modPe * modPe);
    const double om_pecfac = 1.0 - pecfac;
    if (useLimiter) {
      for (int i = 0; i < 3; ++i) {
        const double dq = u[ir * 3 + i] - u[il * 3 + i];
        const double dqMl = 2.0 * 2.0 * duL[i] - dq;
        const double dqMr = 2.0 * 2.0 * duR[i] - dq;
        limitL[i] = van_leer(dqMl, dq);
        limitR[i] = van_leer(dqMr, dq);
      }
    }
    double uIpL[3], uIpR[3];
    for (int i = 0; i < 3; ++i) {
      uIpL[i] = u[il * 3 + i] + duL[i] * hoUpwind * limitL[i];
      uIpR[i] = u[ir * 3 + i] - duR[i] * hoUpwind * limitR[i];
    }
    for (int i = 0; i < 3; ++i) {
      const double uiIp = uIp[i];
      const double uiUpwind = (tmdot > 0) ? alphaUpw * uIpL[i] + om_alphaUpw * uiIp
                                          : alphaUpw * uIpR[i] + om_alphaUpw * uiIp;
      const double uiHatL = alpha * uIpL[i] + om_alpha * uiIp;
      const double uiHatR = alpha * uIpR[i] + om_alpha * uiIp;
      const double uiCds = 0.5 * (uiHatL + uiHatR);
      const double aflux = tmdot * (pecfac * uiUpwind + om_pecfac * uiCds);
      const double divUstress = 2.0 / 3.0 * muIp * divU * areav[ip * 3 + i] * include_divu;
      const int iL = ilN + i, iR = irN + i;
      rhs[iL] -= aflux + divUstress;
      rhs[iR] += aflux + divUstress;
      const double alhsfacL = 0.5 * (tmdot + std::fabs(tmdot)) * pecfac * alphaUpw + 0.5 * alpha * om_pecfac * tmdot;
      L(iL, iL) += alhsfacL;
      L(iR, iL) -= alhsfacL;
      const double alhsfacR = 0.5 * (tmdot - std::fabs(tmdot)) * pecfac * alphaUpw + 0.5 * alpha * om_pecfac * tmdot;
      L(iR, iR) -= alhsfacR;
      L(iL, iR) += alhsfacR;
    }
    for (int ic = 0; ic < 8; ++ic) {
      const int icN = ic * 3;
      const double lhsfacAdv = shpAdv[ip * 8 + ic] * tmdot * (pecfac * om_alphaUpw + om_pecfac * om_alpha);
      for (int i = 0; i < 3; ++i) {
        const int iL = ilN + i, iR = irN + i;
        L(iL, icN + i) += lhsfacAdv;
        L(iR, icN + i) -= lhsfacAdv;
        double lhs_riC_i = 0.0;
        for (int j = 0; j < 3; ++j) {
          const double axj = areav[ip * 3 + j];
          const double uj = u[ic * 3 + j];
          const double lhsfacDiff_i = -muIp * dndx[ip * 24 + ic * 3 + j] * axj;
          lhs_riC_i += lhsfacDiff_i;
          const double lhsfacDiff_j = -muIp * dndx[ip * 24 + ic * 3 + i] * axj;
          L(iL, icN + j) += lhsfacDiff_j;
          L(iR, icN + j) -= lhsfacDiff_j;
          rhs[iL] -= lhsfacDiff_j * uj;
          rhs[iR] += lhsfacDiff_j * uj;
        }
        L(iL, icN + i) += lhs_riC_i;
        L(iR, icN + i) -= lhs_riC_i;
        const double ui = u[ic * 3 + i];
        rhs[iL] -= lhs_riC_i * ui;
        rhs[iR] += lhs_riC_i * ui;
      }
    }
  }
}

// ComputeMdotElemAlgorithm::execute per element: src/ComputeMdotElemAlgorithm.C:200-245
// (restated with the SharedMemView geometry; the unit-test helper
// calc_mass_flow_rate_scs, unit_tests/kernels/UnitTestKernelUtils.C:547-625, is
// the special case pressure = Gpdx = 0).
void orc_mdot_elem(const double* coords, const double* rho, const double* vrtm, const double* p,
                   const double* gpdx, double tau, int shift_mdot, int shift_poisson,
                   double* mdot) {
  double shp[96], areav[36], dndx[288];
  scs_shape(shift_mdot != 0, shp);
  orc_hex_scs_areav(coords, areav);
  scs_grad(coords, shift_poisson != 0, dndx);
  for (int ip = 0; ip < 12; ++ip) {
    double rho_u[3] = {0, 0, 0}, gp[3] = {0, 0, 0}, dpdx[3] = {0, 0, 0};
    for (int ic = 0; ic < 8; ++ic) {
      const double r = shp[ip * 8 + ic];
      for (int j = 0; j < 3; ++j) {
        gp[j] += r * gpdx[ic * 3 + j];
        rho_u[j] += r * rho[ic] * vrtm[ic * 3 + j];
        dpdx[j] += dndx[ip * 24 + ic * 3 + j] * p[ic];
      }
    }
    double t = 0.0;
    for (int j = 0; j < 3; ++j) t += (rho_u[j] - tau * (dpdx[j] - gp[j])) * areav[ip * 3 + j];
    mdot[ip] = t;
  }
}

// ---------------------------------------------------------------------------
// Graph: TpetraLinearSystem::beginLinearSystemConstruction (:189-327),
// insert_connection/addConnections (:329-367), buildConnectedNodeGraph
// (:392-413), finalizeLinearSystem (:1256-1353) with compute_graph_row_lengths,
// insert_graph_connections (:878-922), LocalGraphArrays::insertIndices
// (include/LinearSolver.h:77-88,106-122), fill_in_extra_dof_rows_per_node
// (:1227-1246) and remove_invalid_indices (:1193-1225).  One rank: every node
// is owned and the column LID of a node equals its row LID.
// ---------------------------------------------------------------------------
int orc_graph_build(int64_t n_nodes, int64_t n_elems, const int32_t* conn,
                    const int64_t* node_gid, int num_dof, int64_t* n_rows_out, int64_t* nnz_out,
                    int64_t* rowptr, int32_t* colind, int32_t* node_lid_out) {
  if (n_nodes <= 0 || num_dof <= 0) return -1;
  auto gid = [&](int64_t i) -> int64_t { return node_gid ? node_gid[i] : i + 1; };
  // owned nodes sorted by global id; localId in that order (:262-275)
  std::vector<int64_t> order(n_nodes);
  for (int64_t i = 0; i < n_nodes; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return gid(a) < gid(b); });
  std::vector<int32_t> lid(n_nodes);
  for (int64_t k = 0; k < n_nodes; ++k) lid[order[k]] = (int32_t)k;
  if (node_lid_out)
    for (int64_t i = 0; i < n_nodes; ++i) node_lid_out[i] = lid[i];
  // connections_ indexed by node lid, entries are node indices (:329-349)
  std::vector<std::vector<int32_t>> connections(n_nodes);
  auto insert_connection = [&](int32_t a, int32_t b) {
    auto& vec = connections[lid[a]];
    if (std::find(vec.begin(), vec.end(), b) == vec.end()) vec.push_back(b);
  };
  for (int64_t e = 0; e < n_elems; ++e) {  // addConnections (:351-367)
    const int32_t* nodes = conn + 8 * e;
    for (int a = 0; a < 8; ++a) {
      const int32_t ea = nodes[a];
      if (ea < 0 || ea >= n_nodes) return -2;
      insert_connection(ea, ea);
      for (int b = a + 1; b < 8; ++b) {
        const int32_t eb = nodes[b];
        if (eb < 0 || eb >= n_nodes) return -2;
        const bool a_then_b = gid(ea) < gid(eb);
        insert_connection(a_then_b ? ea : eb, a_then_b ? eb : ea);
      }
    }
  }
  // sort_connections (:659-664): the sort key (entity handle) does not affect
  // the finished graph because insertIndices keeps every row sorted.
  // compute_graph_row_lengths (:516-557 region) -> per dof row length
  const int64_t nrows = (int64_t)n_nodes * num_dof;
  std::vector<int64_t> rowLen(nrows, 0);
  for (int64_t a = 0; a < n_nodes; ++a) {
    const int32_t node_a = (int32_t)order[a];
    const auto& cols = connections[a];
    for (int d = 0; d < num_dof; ++d) rowLen[(int64_t)num_dof * a + d] += (int64_t)num_dof * cols.size();
    for (int32_t b : cols) {
      if (b == node_a) continue;
      const int64_t lb = lid[b];
      for (int d = 0; d < num_dof; ++d) rowLen[(int64_t)num_dof * lb + d] += num_dof;
    }
  }
  std::vector<int64_t> rp(nrows + 1, 0);
  for (int64_t i = 0; i < nrows; ++i) rp[i + 1] = rp[i] + rowLen[i];
  const int64_t nnz_alloc = rp[nrows];
  if (!colind) {
    // row lengths are exact on one rank; report the sizes only
    *n_rows_out = nrows;
    *nnz_out = nnz_alloc;
    return 0;
  }
  const int32_t INVALID = std::numeric_limits<int32_t>::max();
  std::vector<int32_t> ci(nnz_alloc, INVALID);
  // LocalGraphArrays::insertIndices (include/LinearSolver.h:77-88)
  auto insertIndices = [&](int64_t row, int64_t numInds, const int32_t* inds) {
    int32_t* r = ci.data() + rp[row];
    const int64_t len = rp[row + 1] - rp[row];
    int32_t* rowEnd = std::find(r, r + len, INVALID);
    for (int64_t i = 0; i < numInds; ++i) {
      int32_t* ip = std::lower_bound(r, rowEnd, inds[i]);
      if (ip <= rowEnd && *ip != inds[i]) {
        // insert(inds[i], numDof, insertPoint, rowEnd+numDof) (:106-122)
        int32_t* end = rowEnd + num_dof;
        for (int32_t* p = end - 1; p != ip; --p) *p = *(p - num_dof);
        for (int k = 0; k < num_dof; ++k) *ip++ = inds[i] + k;
        rowEnd += num_dof;
      }
    }
  };
  // insert_graph_connections (:878-922): column ids are numDof*colLid
  std::vector<int32_t> colsb;
  for (int64_t a = 0; a < n_nodes; ++a) {
    const auto& ents = connections[a];
    if (ents.empty()) continue;
    const int32_t node_a = (int32_t)order[a];
    colsb.resize(ents.size());
    for (size_t j = 0; j < ents.size(); ++j) colsb[j] = (int32_t)((int64_t)num_dof * lid[ents[j]]);
    insertIndices((int64_t)num_dof * a, (int64_t)ents.size(), colsb.data());
    const int32_t cola = (int32_t)((int64_t)num_dof * a);
    for (size_t j = 0; j < ents.size(); ++j)
      if (ents[j] != node_a) insertIndices((int64_t)num_dof * lid[ents[j]], 1, &cola);
  }
  // fill_in_extra_dof_rows_per_node (:1227-1246)
  if (num_dof > 1) {
    for (int64_t i = 0; i < nrows; i += num_dof) {
      const int64_t len = rp[i + 1] - rp[i];
      for (int d = 1; d < num_dof; ++d)
        for (int64_t j = 0; j < len; ++j) ci[rp[i] + len * d + j] = ci[rp[i] + j];
    }
  }
  // remove_invalid_indices (:1193-1225)
  std::vector<int64_t> newLen(nrows, 0);
  int64_t newNnz = 0;
  for (int64_t i = 0; i < nrows; ++i) {
    const int64_t len = rp[i + 1] - rp[i];
    newLen[i] = rowLen[i];
    for (int64_t j = len - 1; j >= 0; --j)
      if (ci[rp[i] + j] != INVALID) {
        newLen[i] = j + 1;
        break;
      }
    newNnz += newLen[i];
  }
  if (*nnz_out < newNnz) return -3;  // caller buffer too small
  int64_t idx = 0;
  rowptr[0] = 0;
  for (int64_t i = 0; i < nrows; ++i) {
    for (int64_t j = 0; j < newLen[i]; ++j) colind[idx++] = ci[rp[i] + j];
    rowptr[i + 1] = idx;
  }
  *n_rows_out = nrows;
  *nnz_out = newNnz;
  return 0;
}

}  // extern "C"

namespace {

// TpetraLinearSystem::sumInto + sum_into_row(_vec_3): src/TpetraLinearSystem.C:1377-1522.
// Column ids are sorted with their permutation (the reference calls
// Tpetra::Details::shellSortKeysAndValues; ids of one element are distinct,
// so any stable key sort gives the same permutation), then each row is
// merge-scanned once against the sorted CSR row.
void sum_into(int num_dof, const int32_t* elem_nodes_lid, const double* lhs, const double* rhs,
              const int64_t* rowptr, const int32_t* colind, double* values, double* sysrhs) {
  const int nrows = 8 * num_dof;
  int localIds[24], perm[24];
  for (int i = 0; i < 8; ++i)
    for (int d = 0; d < num_dof; ++d) localIds[i * num_dof + d] = elem_nodes_lid[i] * num_dof + d;
  for (int i = 0; i < nrows; ++i) perm[i] = i;
  // insertion sort of (key, perm) pairs
  for (int i = 1; i < nrows; ++i) {
    const int k = localIds[i], p = perm[i];
    int j = i - 1;
    while (j >= 0 && localIds[j] > k) {
      localIds[j + 1] = localIds[j];
      perm[j + 1] = perm[j];
      --j;
    }
    localIds[j + 1] = k;
    perm[j + 1] = p;
  }
  for (int r = 0; r < nrows; ++r) {
    const int i = perm[r] / num_dof;
    const int64_t rowLid = (int64_t)elem_nodes_lid[i] * num_dof + perm[r] % num_dof;
    const double* cur_lhs = lhs + (int64_t)perm[r] * nrows;
    const int64_t rb = rowptr[rowLid];
    const int64_t length = rowptr[rowLid + 1] - rb;
    if (num_dof == 3) {
      int64_t offset = 0;
      for (int j = 0; j < 8; ++j) {
        const int id_index = 3 * j;
        const int32_t cur = localIds[id_index];
        bool found = true;
        while (colind[rb + offset] != cur) {
          offset += 3;
          if (offset >= length) { found = false; break; }
        }
        if (!found) break;
        const int entry = perm[id_index];
        values[rb + offset + 0] += cur_lhs[entry + 0];
        values[rb + offset + 1] += cur_lhs[entry + 1];
        values[rb + offset + 2] += cur_lhs[entry + 2];
        offset += 3;
      }
    } else {
      int64_t offset = 0;
      for (int j = 0; j < nrows; ++j) {
        const int pidx = perm[j];
        const int32_t cur = localIds[j];
        while (offset < length && colind[rb + offset] != cur) ++offset;
        if (offset < length) values[rb + offset] += cur_lhs[pidx];
      }
    }
    sysrhs[rowLid] += rhs[perm[r]];
  }
}

}  // namespace

extern "C" {

// AssembleElemSolverAlgorithm::execute (src/AssembleElemSolverAlgorithm.C:75-100)
// in serial element order (the reference runs Kokkos::Serial), optionally
// parallelised over a greedy element colouring when n_threads > 1.
int orc_assemble(int kernel, int64_t n_nodes, int64_t n_elems, const int32_t* conn,
                 const int32_t* node_lid, const double* coords, const double* f_scalar,
                 const double* f_coeff, const double* f_vec, const double* f_vec2,
                 const double* f_rho, const double* f_gju, const double* elem_mdot,
                 const double* opts, int num_dof, const int64_t* rowptr, const int32_t* colind,
                 double* values, double* rhs, int n_threads) {
  const bool shifted = opts[0] != 0.0, shift_mdot = opts[1] != 0.0, shift_poisson = opts[2] != 0.0,
             reduced = opts[3] != 0.0;
  const double tau = opts[4], divu = opts[5];
  const bool skew = opts[6] != 0.0;
  const int nd = (kernel >= 2) ? 3 : 1;
  if (nd != num_dof) return -1;
  auto one = [&](int64_t e) {
    double c[24], a[8], b[8], v[24], w[24], r8[8], g[72];
    int32_t elid[8];
    double lhs[576], erhs[24];
    const int32_t* en = conn + 8 * e;
    for (int n = 0; n < 8; ++n) {
      const int64_t i = en[n];
      elid[n] = node_lid ? node_lid[i] : (int32_t)i;
      for (int d = 0; d < 3; ++d) c[n * 3 + d] = coords[i * 3 + d];
    }
    auto gather1 = [&](const double* f, double* out) {
      for (int n = 0; n < 8; ++n) out[n] = f ? f[en[n]] : 0.0;
    };
    auto gather3 = [&](const double* f, double* out) {
      for (int n = 0; n < 8; ++n)
        for (int d = 0; d < 3; ++d) out[n * 3 + d] = f ? f[(int64_t)en[n] * 3 + d] : 0.0;
    };
    switch (kernel) {
      case 0:
        gather1(f_scalar, a);
        gather1(f_coeff, b);
        orc_scalar_diff_elem(c, a, b, shifted, lhs, erhs);
        break;
      case 1:
        gather1(f_scalar, a);
        gather1(f_coeff, b);
        gather3(f_vec, v);
        gather3(f_vec2, w);
        orc_continuity_adv_elem(c, v, b, a, w, tau, shift_mdot, shift_poisson, reduced, lhs, erhs);
        break;
      case 2:
        gather1(f_coeff, b);
        gather3(f_vec, v);
        orc_momentum_adv_diff_elem(c, v, b, elem_mdot + 12 * e, divu, shifted, skew, lhs, erhs);
        break;
      default:
        gather1(f_coeff, b);
        gather1(f_rho, r8);
        gather3(f_vec, v);
        gather3(f_vec2, w);
        for (int n = 0; n < 8; ++n)
          for (int k = 0; k < 9; ++k) g[n * 9 + k] = f_gju[(int64_t)en[n] * 9 + k];
        orc_momentum_upw_adv_diff_elem(c, v, w, r8, b, g, elem_mdot + 12 * e, divu, shifted, skew,
                                       opts[7], opts[8], opts[9], opts[10], opts[11] != 0.0, lhs,
                                       erhs);
        break;
    }
    sum_into(num_dof, elid, lhs, erhs, rowptr, colind, values, rhs);
  };
  if (n_threads <= 1) {
    for (int64_t e = 0; e < n_elems; ++e) one(e);
    return 0;
  }
  // greedy colouring: elements of one colour share no node
  std::vector<uint64_t> mask(n_nodes, 0);
  std::vector<int> colour(n_elems);
  int ncol = 0;
  for (int64_t e = 0; e < n_elems; ++e) {
    uint64_t used = 0;
    for (int n = 0; n < 8; ++n) used |= mask[conn[8 * e + n]];
    int cidx = 0;
    while (cidx < 64 && (used >> cidx) & 1) ++cidx;
    if (cidx >= 64) return -4;
    colour[e] = cidx;
    ncol = std::max(ncol, cidx + 1);
    for (int n = 0; n < 8; ++n) mask[conn[8 * e + n]] |= (1ull << cidx);
  }
  std::vector<std::vector<int64_t>> lists(ncol);
  for (int64_t e = 0; e < n_elems; ++e) lists[colour[e]].push_back(e);
  for (int cc = 0; cc < ncol; ++cc) {
    const auto& L = lists[cc];
    parallel_for((int64_t)L.size(), n_threads, [&](int64_t b, int64_t en) {
      for (int64_t k = b; k < en; ++k) one(L[k]);
    });
  }
  return 0;
}

int orc_assemble_mass(int momentum, int64_t n_nodes, int64_t n_elems, const int32_t* conn,
                      const int32_t* node_lid, const double* coords, const double* rho_nm1,
                      const double* rho_n, const double* rho_np1, const double* u_nm1,
                      const double* u_n, const double* u_np1, const double* gpdx, const double* tp,
                      const int64_t* rowptr, const int32_t* colind, double* values, double* rhs) {
  (void)n_nodes;
  for (int64_t e = 0; e < n_elems; ++e) {
    double c[24], a[8], b[8], d[8], u0[24], u1[24], u2[24], g[24], lhs[576], erhs[24];
    int32_t elid[8];
    const int32_t* en = conn + 8 * e;
    for (int n = 0; n < 8; ++n) {
      const int64_t i = en[n];
      elid[n] = node_lid ? node_lid[i] : (int32_t)i;
      a[n] = rho_nm1[i];
      b[n] = rho_n[i];
      d[n] = rho_np1[i];
      for (int k = 0; k < 3; ++k) {
        c[3 * n + k] = coords[3 * i + k];
        if (momentum) {
          u0[3 * n + k] = u_nm1[3 * i + k];
          u1[3 * n + k] = u_n[3 * i + k];
          u2[3 * n + k] = u_np1[3 * i + k];
          g[3 * n + k] = gpdx[3 * i + k];
        }
      }
    }
    if (momentum) {
      orc_momentum_mass_elem(c, a, b, d, u0, u1, u2, g, tp[0], tp[1], tp[2], tp[3], tp[4] != 0.0, tp[5] != 0.0,
                             lhs, erhs);
      sum_into(3, elid, lhs, erhs, rowptr, colind, values, rhs);
    } else {
      orc_continuity_mass_elem(c, a, b, d, tp[0], tp[1], tp[2], tp[3], tp[4] != 0.0, lhs, erhs);
      sum_into(1, elid, lhs, erhs, rowptr, colind, values, rhs);
    }
  }
  return 0;
}

// ---- boundary faces -------------------------------------------------------
static const int kSide[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};

void orc_hex_side_nodes(int side, int* nodes4) {
  for (int k = 0; k < 4; ++k) nodes4[k] = kSide[side][k];
}

// quad3d_scs_det (src/master_element/MasterElementWork.F:1467-1590)
void orc_quad3d_scs_areav(const double* fc, double* areav) {
  const double half = 0.5, one4th = 1.0 / 4.0;
  double p[4][3], e[4][3], c[3];
  for (int i = 0; i < 4; ++i)
    for (int d = 0; d < 3; ++d) p[i][d] = fc[3 * i + d];
  for (int d = 0; d < 3; ++d) {
    e[0][d] = (p[0][d] + p[1][d]) * half;
    e[1][d] = (p[1][d] + p[2][d]) * half;
    e[2][d] = (p[2][d] + p[3][d]) * half;
    e[3][d] = (p[3][d] + p[0][d]) * half;
    c[d] = (p[0][d] + p[1][d] + p[2][d] + p[3][d]) * one4th;
  }
  for (int k = 0; k < 4; ++k) {
    const int prev = (k + 3) % 4;  // sub-face k: corner p_k, edge midpoints e_{k-1}, e_k, centre c
    const double dx13 = c[0] - p[k][0], dx24 = e[prev][0] - e[k][0];
    const double dy13 = c[1] - p[k][1], dy24 = e[prev][1] - e[k][1];
    const double dz13 = c[2] - p[k][2], dz24 = e[prev][2] - e[k][2];
    areav[3 * k + 0] = half * (dz24 * dy13 - dz13 * dy24);
    areav[3 * k + 1] = half * (dx24 * dz13 - dx13 * dz24);
    areav[3 * k + 2] = half * (dy24 * dx13 - dy13 * dx24);
  }
}

// HexSCS::face_grad_op (Hex8CVFEM.C:668-684); intgExpFace_ (:348-373): the
// face node's parent location with the two in-plane coordinates halved;
// intgExpFaceShift_ (:424-440): the face node itself
int orc_hex_face_grad_op(int side, int shifted, const double* coords, double* gradop) {
  static const double loc[8][3] = {{-0.5, -0.5, -0.5}, {0.5, -0.5, -0.5}, {0.5, 0.5, -0.5}, {-0.5, 0.5, -0.5},
                                   {-0.5, -0.5, 0.5},  {0.5, -0.5, 0.5},  {0.5, 0.5, 0.5},  {-0.5, 0.5, 0.5}};
  static const int normal_axis[6] = {1, 0, 1, 0, 2, 2};
  double pts[12], deriv[96];
  for (int k = 0; k < 4; ++k)
    for (int d = 0; d < 3; ++d) {
      const double x = loc[kSide[side][k]][d];
      pts[3 * k + d] = (shifted || d == normal_axis[side]) ? x : 0.5 * x;
    }
  orc_hex8_derivative(4, pts, deriv);
  return orc_generic_grad_op(4, deriv, coords, gradop, nullptr);
}

void orc_skin(int64_t n_elems, const int32_t* conn, uint8_t* flags) {
  std::map<std::array<int32_t, 4>, int> count;
  auto key = [&](int64_t e, int s) {
    std::array<int32_t, 4> k;
    for (int i = 0; i < 4; ++i) k[i] = conn[8 * e + kSide[s][i]];
    std::sort(k.begin(), k.end());
    return k;
  };
  for (int64_t e = 0; e < n_elems; ++e)
    for (int s = 0; s < 6; ++s) ++count[key(e, s)];
  for (int64_t e = 0; e < n_elems; ++e)
    for (int s = 0; s < 6; ++s) flags[6 * e + s] = count[key(e, s)] == 1 ? 1 : 0;
}

// Quad3DSCS shape functions (quad3d_shape_fcn, MasterElementWork.F:3651-3700)
// at intgLoc_ (Quad43DCVFEM.C:37-41) or intgLocShift_ (:44-48)
static void quad_face_shape(int shifted, double shp[4][4]) {
  const double a = shifted ? 0.5 : 0.25;
  const double loc[4][2] = {{-a, -a}, {a, -a}, {a, a}, {-a, a}};
  const double one4th = 1.0 / 4.0, half = 1.0 / 2.0;
  for (int j = 0; j < 4; ++j) {
    const double s1 = loc[j][0], s2 = loc[j][1];
    shp[j][0] = one4th + half * (-s1 - s2) + s1 * s2;
    shp[j][1] = one4th + half * (s1 - s2) - s1 * s2;
    shp[j][2] = one4th + half * (s1 + s2) + s1 * s2;
    shp[j][3] = one4th + half * (-s1 + s2) - s1 * s2;
  }
}

static void face_area(int side, const double* coords, double* areav) {
  double fc[12];
  for (int k = 0; k < 4; ++k)
    for (int d = 0; d < 3; ++d) fc[3 * k + d] = coords[3 * kSide[side][k] + d];
  orc_quad3d_scs_areav(fc, areav);
}

void orc_nodal_grad_boundary(int64_t n_faces, const int32_t* face_elem, const int32_t* face_side,
                             const int32_t* conn, const double* coords, const double* q, int ncomp,
                             const double* dual_volume, int shifted, double* grad) {
  double shp[4][4];
  quad_face_shape(shifted, shp);
  for (int64_t f = 0; f < n_faces; ++f) {
    const int64_t e = face_elem[f];
    const int s = face_side[f];
    double c[24], a[12];
    for (int n = 0; n < 8; ++n)
      for (int d = 0; d < 3; ++d) c[3 * n + d] = coords[3 * (int64_t)conn[8 * e + n] + d];
    face_area(s, c, a);
    for (int ip = 0; ip < 4; ++ip) {
      const int64_t nn = conn[8 * e + kSide[s][ip]];
      const double inv_vol = 1.0 / dual_volume[nn];
      for (int k = 0; k < ncomp; ++k) {
        double qip = 0.0;
        for (int ic = 0; ic < 4; ++ic) qip += shp[ip][ic] * q[(int64_t)conn[8 * e + kSide[s][ic]] * ncomp + k];
        for (int j = 0; j < 3; ++j) grad[(nn * ncomp + k) * 3 + j] += qip * a[3 * ip + j] * inv_vol;
      }
    }
  }
}

void orc_continuity_inflow_face(int side, const double* coords, const double* rho, const double* ubc,
                                double proj_time_scale, int shifted, double* rhs) {
  double shp[4][4], a[12];
  quad_face_shape(shifted, shp);
  face_area(side, coords, a);
  for (int i = 0; i < 8; ++i) rhs[i] = 0.0;
  for (int ip = 0; ip < 4; ++ip) {
    const int nn = kSide[side][ip];
    double w[3] = {0.0, 0.0, 0.0};
    for (int ic = 0; ic < 4; ++ic) {
      const double r = shp[ip][ic];
      const double rhoIC = rho[kSide[side][ic]];
      for (int j = 0; j < 3; ++j) w[j] += r * rhoIC * ubc[3 * kSide[side][ic] + j];
    }
    double mDot = 0.0;
    for (int j = 0; j < 3; ++j) mDot += w[j] * a[3 * ip + j];
    rhs[nn] -= mDot / proj_time_scale;
  }
}

void orc_continuity_open_face(int side, const double* coords, const double* p, const double* pbc,
                              const double* rho, const double* u, const double* gpdx, const double* dynp,
                              double proj_time_scale, int shift_grad_op, int reduced_sens, int shift_mdot,
                              double* lhs, double* rhs) {
  const double penaltyFac = 2.0;
  double shp[4][4], a[12], g_std[96], g_sh[96];
  quad_face_shape(shift_mdot, shp);
  face_area(side, coords, a);
  orc_hex_face_grad_op(side, 0, coords, g_std);
  orc_hex_face_grad_op(side, 1, coords, g_sh);
  const double* dndx = shift_grad_op ? g_sh : g_std;
  const double* dndx_lhs = (shift_grad_op || reduced_sens) ? g_sh : g_std;
  for (int i = 0; i < 64; ++i) lhs[i] = 0.0;
  for (int i = 0; i < 8; ++i) rhs[i] = 0.0;
  const int* fn = kSide[side];
  for (int ip = 0; ip < 4; ++ip) {
    const int nn = fn[ip];
    double w_rho_u[3] = {0, 0, 0}, w_gp[3] = {0, 0, 0}, w_dpdx[3] = {0, 0, 0};
    double aMag = 0.0;
    for (int j = 0; j < 3; ++j) aMag += a[3 * ip + j] * a[3 * ip + j];
    aMag = std::sqrt(aMag);
    double invL = 0.0;
    for (int ic = 0; ic < 4; ++ic)
      for (int j = 0; j < 3; ++j) invL += dndx[ip * 24 + fn[ic] * 3 + j] * a[3 * ip + j];
    invL /= aMag;
    double pBip = 0.0, pbcBip = -(dynp ? dynp[ip] : 0.0);
    for (int ic = 0; ic < 4; ++ic) {
      const double r = shp[ip][ic];
      const double rhoIC = rho[fn[ic]];
      pBip += r * p[fn[ic]];
      pbcBip += r * pbc[fn[ic]];
      for (int j = 0; j < 3; ++j) {
        w_rho_u[j] += r * rhoIC * u[3 * fn[ic] + j];
        w_gp[j] += r * gpdx[3 * fn[ic] + j];
      }
    }
    for (int ic = 0; ic < 8; ++ic)
      for (int j = 0; j < 3; ++j) w_dpdx[j] += dndx[ip * 24 + ic * 3 + j] * p[ic];
    double mdot = penaltyFac * proj_time_scale * invL * (pBip - pbcBip) * aMag;
    for (int j = 0; j < 3; ++j)
      mdot += (w_rho_u[j] - proj_time_scale * (w_dpdx[j] - w_gp[j])) * a[3 * ip + j];
    for (int ic = 0; ic < 4; ++ic) lhs[nn * 8 + fn[ic]] += shp[ip][ic] * penaltyFac * invL * aMag;
    for (int ic = 0; ic < 8; ++ic) {
      double lhsFac = 0.0;
      for (int j = 0; j < 3; ++j) lhsFac += -dndx_lhs[ip * 24 + ic * 3 + j] * a[3 * ip + j];
      lhs[nn * 8 + ic] += lhsFac;
    }
    rhs[nn] -= mdot / proj_time_scale;
  }
}

int orc_assemble_faces(int kernel, int64_t n_faces, const int32_t* face_elem, const int32_t* face_side,
                       const int32_t* conn, const int32_t* node_lid, const double* coords, const double* p,
                       const double* pbc, const double* rho, const double* u, const double* gpdx,
                       const double* dynp, const double* opts, const int64_t* rowptr, const int32_t* colind,
                       double* values, double* rhs) {
  for (int64_t f = 0; f < n_faces; ++f) {
    const int64_t e = face_elem[f];
    const int s = face_side[f];
    double c[24], pe[8], pb[8], re[8], ue[24], ge[24], lhs[64], erhs[8];
    int32_t elid[8];
    for (int n = 0; n < 8; ++n) {
      const int64_t i = conn[8 * e + n];
      elid[n] = node_lid ? node_lid[i] : (int32_t)i;
      pe[n] = p ? p[i] : 0.0;
      pb[n] = pbc ? pbc[i] : 0.0;
      re[n] = rho[i];
      for (int d = 0; d < 3; ++d) {
        c[3 * n + d] = coords[3 * i + d];
        ue[3 * n + d] = u[3 * i + d];
        ge[3 * n + d] = gpdx ? gpdx[3 * i + d] : 0.0;
      }
    }
    if (kernel == 0) {
      for (int i = 0; i < 64; ++i) lhs[i] = 0.0;
      orc_continuity_inflow_face(s, c, re, ue, opts[0], opts[3] != 0.0, erhs);
    } else {
      orc_continuity_open_face(s, c, pe, pb, re, ue, ge, dynp ? dynp + 4 * f : nullptr, opts[0], opts[1] != 0.0,
                               opts[2] != 0.0, opts[3] != 0.0, lhs, erhs);
    }
    sum_into(1, elid, lhs, erhs, rowptr, colind, values, rhs);
  }
  return 0;
}

void orc_sum_into(int num_dof, const int32_t* elem_nodes_lid, const double* lhs, const double* rhs,
                  const int64_t* rowptr, const int32_t* colind, double* values, double* sysrhs) {
  sum_into(num_dof, elem_nodes_lid, lhs, rhs, rowptr, colind, values, sysrhs);
}

// TpetraLinearSystem::applyDirichletBCs: src/TpetraLinearSystem.C:1579-1653 (owned rows):
// row -> unit diagonal, other entries 0, rhs = bc - current.
void orc_apply_dirichlet(const int64_t* rowptr, const int32_t* colind, double* values, double* rhs,
                         int64_t n_bc, const int32_t* rows, const double* bc, const double* cur) {
  for (int64_t k = 0; k < n_bc; ++k) {
    const int32_t r = rows[k];
    for (int64_t j = rowptr[r]; j < rowptr[r + 1]; ++j) values[j] = (colind[j] == r) ? 1.0 : 0.0;
    rhs[r] = bc[k] - cur[k];
  }
}

// TpetraLinearSystem::resetRows: src/TpetraLinearSystem.C:1707-1755
void orc_reset_rows(const int64_t* rowptr, double* values, double* rhs, int64_t n, const int32_t* rows) {
  for (int64_t k = 0; k < n; ++k) {
    const int32_t r = rows[k];
    for (int64_t j = rowptr[r]; j < rowptr[r + 1]; ++j) values[j] = 0.0;
    rhs[r] = 0.0;
  }
}

// FixPressureAtNodeAlgorithm::execute after resetRows: src/FixPressureAtNodeAlgorithm.C:53-80
// (sumInto of a 1x1 system: diag += 1, rhs += p_ref - p)
void orc_sum_into_diag(const int64_t* rowptr, const int32_t* colind, double* values, double* rhs,
                       int32_t row, double diag, double rhs_value) {
  for (int64_t j = rowptr[row]; j < rowptr[row + 1]; ++j)
    if (colind[j] == row) values[j] += diag;
  rhs[row] += rhs_value;
}

void orc_spmv(int64_t n, const int64_t* rp, const int32_t* ci, const double* v, const double* x,
              double* y, int n_threads) {
  parallel_for(n, n_threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      double s = 0.0;
      for (int64_t j = rp[i]; j < rp[i + 1]; ++j) s += v[j] * x[ci[j]];
      y[i] = s;
    }
  });
}

static double dot(int64_t n, const double* a, const double* b) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

static double true_rel_res(int64_t n, const int64_t* rp, const int32_t* ci, const double* v,
                           const double* b, const double* x, int nt) {
  std::vector<double> r(n);
  orc_spmv(n, rp, ci, v, x, r.data(), nt);
  double rr = 0.0, bb = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double d = b[i] - r[i];
    rr += d * d;
    bb += b[i] * b[i];
  }
  return bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
}

// Jacobi-preconditioned CG (stand-in for Belos CG + Ifpack2 Jacobi,
// src/LinearSolver.C:183-232; stop on the unpreconditioned relative residual).
int orc_pcg_jacobi(int64_t n, const int64_t* rp, const int32_t* ci, const double* v,
                   const double* b, double* x, double tol, int max_it, double* res_out, int nt) {
  std::vector<double> dinv(n), r(n), z(n), p(n), q(n);
  for (int64_t i = 0; i < n; ++i) {
    double d = 0.0;
    for (int64_t j = rp[i]; j < rp[i + 1]; ++j)
      if (ci[j] == i) d = v[j];
    dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
  }
  orc_spmv(n, rp, ci, v, x, q.data(), nt);
  for (int64_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
  const double bn = std::sqrt(dot(n, b, b));
  const double stop = tol * (bn > 0 ? bn : 1.0);
  for (int64_t i = 0; i < n; ++i) z[i] = dinv[i] * r[i], p[i] = z[i];
  double rz = dot(n, r.data(), z.data());
  int it = 0;
  double rn = std::sqrt(dot(n, r.data(), r.data()));
  while (rn > stop && it < max_it) {
    orc_spmv(n, rp, ci, v, p.data(), q.data(), nt);
    const double alpha = rz / dot(n, p.data(), q.data());
    for (int64_t i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      z[i] = dinv[i] * r[i];
    }
    const double rz1 = dot(n, r.data(), z.data());
    const double beta = rz1 / rz;
    rz = rz1;
    for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    rn = std::sqrt(dot(n, r.data(), r.data()));
    ++it;
  }
  if (res_out) *res_out = true_rel_res(n, rp, ci, v, b, x, nt);
  return it;
}

// Right-preconditioned restarted GMRES(m) with Jacobi (stand-in for Belos
// GMRES + Ifpack2 Jacobi; Givens rotations, modified Gram-Schmidt).
int orc_gmres_jacobi(int64_t n, const int64_t* rp, const int32_t* ci, const double* v,
                     const double* b, double* x, int m, double tol, int max_it, double* res_out,
                     int nt) {
  std::vector<double> dinv(n), r(n), w(n), z(n);
  for (int64_t i = 0; i < n; ++i) {
    double d = 0.0;
    for (int64_t j = rp[i]; j < rp[i + 1]; ++j)
      if (ci[j] == i) d = v[j];
    dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
  }
  std::vector<double> V((size_t)(m + 1) * n), H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  const double bn = std::sqrt(dot(n, b, b));
  const double stop = tol * (bn > 0 ? bn : 1.0);
  int it = 0;
  while (it < max_it) {
    orc_spmv(n, rp, ci, v, x, w.data(), nt);
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - w[i];
    double beta = std::sqrt(dot(n, r.data(), r.data()));
    if (beta <= stop) break;
    for (int64_t i = 0; i < n; ++i) V[i] = r[i] / beta;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    for (; k < m && it < max_it; ++k, ++it) {
      for (int64_t i = 0; i < n; ++i) z[i] = dinv[i] * V[(size_t)k * n + i];
      orc_spmv(n, rp, ci, v, z.data(), w.data(), nt);
      for (int j = 0; j <= k; ++j) {
        const double h = dot(n, w.data(), &V[(size_t)j * n]);
        H[(size_t)j * m + k] = h;
        for (int64_t i = 0; i < n; ++i) w[i] -= h * V[(size_t)j * n + i];
      }
      const double hn = std::sqrt(dot(n, w.data(), w.data()));
      H[(size_t)(k + 1) * m + k] = hn;
      for (int64_t i = 0; i < n; ++i) V[(size_t)(k + 1) * n + i] = hn > 0 ? w[i] / hn : 0.0;
      for (int j = 0; j < k; ++j) {
        const double t = cs[j] * H[(size_t)j * m + k] + sn[j] * H[(size_t)(j + 1) * m + k];
        H[(size_t)(j + 1) * m + k] = -sn[j] * H[(size_t)j * m + k] + cs[j] * H[(size_t)(j + 1) * m + k];
        H[(size_t)j * m + k] = t;
      }
      const double a = H[(size_t)k * m + k], bb = H[(size_t)(k + 1) * m + k];
      const double den = std::sqrt(a * a + bb * bb);
      cs[k] = den > 0 ? a / den : 1.0;
      sn[k] = den > 0 ? bb / den : 0.0;
      H[(size_t)k * m + k] = den;
      H[(size_t)(k + 1) * m + k] = 0.0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      if (std::fabs(g[k + 1]) <= stop) {
        ++k;
        ++it;
        break;
      }
    }
    for (int j = k - 1; j >= 0; --j) {
      double s = g[j];
      for (int l = j + 1; l < k; ++l) s -= H[(size_t)j * m + l] * y[l];
      y[j] = s / H[(size_t)j * m + j];
    }
    std::fill(z.begin(), z.end(), 0.0);
    for (int j = 0; j < k; ++j)
      for (int64_t i = 0; i < n; ++i) z[i] += y[j] * V[(size_t)j * n + i];
    for (int64_t i = 0; i < n; ++i) x[i] += dinv[i] * z[i];
    if (true_rel_res(n, rp, ci, v, b, x, nt) <= tol) break;
  }
  if (res_out) *res_out = true_rel_res(n, rp, ci, v, b, x, nt);
  return it;
}

}  // extern "C"
