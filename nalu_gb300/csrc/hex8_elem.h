// hex8_elem.h -- Hex8 CVFEM element math, shared by the sm_103a kernels and a
// host-side check build.
//
// What the reference computes (src/master_element/Hex8CVFEM.C,
// include/master_element/{MasterElementFunctions,Hex8GeometryFunctions}.h)
// is reproduced here in a form with far fewer FP64 operations, because FP64
// issue rate, not HBM, bounds this assembly on GB300:
//
// * The Jacobian at an integration point is the bilinear interpolation of the
//   four element edges along each isoparametric axis (the exact derivative of
//   the trilinear map), instead of 8 nodes x 9 entries of multiply-adds.
// * The SCS area vector needs no sub-division and no triangle fan: for the
//   trilinear map, the fan-triangulated vector area of each SCS quad
//   (quad_area_by_triangulation over subdivide_hex_8 points) equals exactly
//   1/4 of the cofactor column of J that belongs to the face normal axis,
//   evaluated at the ip.  (The 27 sub-division points are the map at
//   {-1/2,0,1/2}^3; a quad fan's vector area is (p2-p0)x(p3-p1)/2; the midpoint
//   rule is exact for the bilinear cross product.)  The cofactors are needed
//   for the gradient operator anyway, so the areas cost 3 multiplies per ip.
// * The element Laplacian row factor  -k * sum_j dndx(ip,c,j) A_j  is
//   evaluated as  -k/det * sum_j dN_c/ds_j * G_j  with  G = adj(J)^T A,
//   so dndx itself is never formed.
//
// The tables below (L/R node pairs, ip locations, corner signs, shape
// functions and their derivatives) are the reference's HexSCS tables
// (Hex8CVFEM.C:265-276, 319-346, 380-396, 25-70, 487-517) written as
// compile-time functions so that the unrolled kernels fold them into
// immediates.
#pragma once

#ifdef __CUDACC__
#define NALU_HD __host__ __device__ __forceinline__
#else
#define NALU_HD inline
#endif

namespace nalu_gb300 {

// corner sign (+1/-1) of node n along isoparametric axis k
NALU_HD constexpr int corner_sign(int n, int k) {
  return k == 0 ? (((n & 3) == 1 || (n & 3) == 2) ? 1 : -1)
                : (k == 1 ? (((n & 3) >= 2) ? 1 : -1) : (n >= 4 ? 1 : -1));
}
// node index from its three corner signs
NALU_HD constexpr int node_of(int s0, int s1, int s2) {
  return (s2 > 0 ? 4 : 0) + (s1 > 0 ? (s0 > 0 ? 2 : 3) : (s0 > 0 ? 1 : 0));
}
// SCS integration point location (a = 1/4 standard, a = 1/2 shifted)
NALU_HD constexpr double ip_loc(int ip, int k, double a) {
  return ip < 8
             ? (k == 2 ? (ip < 4 ? -a : a)
                       : ((ip & 3) == 0 ? (k == 0 ? 0.0 : -a)
                                        : ((ip & 3) == 1 ? (k == 0 ? a : 0.0)
                                                         : ((ip & 3) == 2 ? (k == 0 ? 0.0 : a)
                                                                          : (k == 0 ? -a : 0.0)))))
             : (k == 2 ? 0.0 : corner_sign(ip - 8, k) * a);
}
// L/R nodes of an SCS ip (lrscv_)
NALU_HD constexpr int ip_left(int ip) { return ip < 8 ? ((ip & 3) == 3 ? (ip & 4) : ip) : ip - 8; }
NALU_HD constexpr int ip_right(int ip) { return ip < 8 ? ((ip & 3) == 3 ? (ip & 4) + 3 : ip + 1) : ip - 4; }
// isoparametric axis normal to the SCS of an ip, and the sign that orients
// the area vector from the left to the right node
NALU_HD constexpr int ip_dir(int ip) { return ip < 8 ? ((ip & 1) ? 1 : 0) : 2; }
NALU_HD constexpr double ip_sign(int ip) { return (ip < 8 && (ip & 3) == 2) ? -1.0 : 1.0; }

// trilinear shape function N_n at point s
NALU_HD constexpr double shape(int n, double s0, double s1, double s2) {
  return (0.5 + corner_sign(n, 0) * s0) * (0.5 + corner_sign(n, 1) * s1) * (0.5 + corner_sign(n, 2) * s2);
}
NALU_HD constexpr double shape_ip(int ip, int n, double a) {
  return shape(n, ip_loc(ip, 0, a), ip_loc(ip, 1, a), ip_loc(ip, 2, a));
}
// dN_n/ds_k at point s
NALU_HD constexpr double dshape(int n, int k, double s0, double s1, double s2) {
  return k == 0 ? corner_sign(n, 0) * (0.5 + corner_sign(n, 1) * s1) * (0.5 + corner_sign(n, 2) * s2)
                : (k == 1 ? corner_sign(n, 1) * (0.5 + corner_sign(n, 0) * s0) * (0.5 + corner_sign(n, 2) * s2)
                          : corner_sign(n, 2) * (0.5 + corner_sign(n, 0) * s0) * (0.5 + corner_sign(n, 1) * s1));
}
NALU_HD constexpr double dshape_ip(int ip, int n, int k, double a) {
  return dshape(n, k, ip_loc(ip, 0, a), ip_loc(ip, 1, a), ip_loc(ip, 2, a));
}

// Bilinear form of dx/ds_k over the two other axes (u < v):
//   dx/ds_k(s_u, s_v) = A + B s_u + C s_v + D s_u s_v  (per component)
struct EdgeForm {
  double A[3][3], B[3][3], C[3][3], D[3][3];  // [k][component]
};

NALU_HD void edge_form(const double x[8][3], EdgeForm& f) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int u = (k == 0) ? 1 : 0;
    const int v = (k == 2) ? 1 : 2;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double e[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int sg[3];
        sg[u] = (q & 1) ? 1 : -1;
        sg[v] = (q & 2) ? 1 : -1;
        sg[k] = -1;
        const int a = node_of(sg[0], sg[1], sg[2]);
        sg[k] = 1;
        const int b = node_of(sg[0], sg[1], sg[2]);
        e[q] = x[b][i] - x[a][i];
      }
      const double p01 = e[0] + e[1], m01 = e[1] - e[0];
      const double p23 = e[2] + e[3], m23 = e[3] - e[2];
      f.A[k][i] = 0.25 * (p01 + p23);
      f.B[k][i] = 0.5 * (m01 + m23);
      f.C[k][i] = 0.5 * (p23 - p01);
      f.D[k][i] = m23 - m01;
    }
  }
}

// Jacobian jact[i][j] = dx_i/ds_j at an ip (compile-time location)
template <int IP, bool SHIFT>
NALU_HD void jacobian_ip(const EdgeForm& f, double jact[3][3]) {
  constexpr double a = SHIFT ? 0.5 : 0.25;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int u = (k == 0) ? 1 : 0;
    const int v = (k == 2) ? 1 : 2;
    const double su = ip_loc(IP, u, a), sv = ip_loc(IP, v, a);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double r = f.A[k][i];
      if (su != 0.0) r = r + f.B[k][i] * su;
      if (sv != 0.0) r = r + f.C[k][i] * sv;
      if (su * sv != 0.0) r = r + f.D[k][i] * (su * sv);
      jact[i][k] = r;
    }
  }
}

// cofactor matrix (cofactorMatrix, MasterElementFunctions.h:31-43) and det
NALU_HD void cofactor(const double j[3][3], double adj[3][3], double& det) {
  adj[0][0] = j[1][1] * j[2][2] - j[2][1] * j[1][2];
  adj[0][1] = j[1][2] * j[2][0] - j[2][2] * j[1][0];
  adj[0][2] = j[1][0] * j[2][1] - j[2][0] * j[1][1];
  adj[1][0] = j[0][2] * j[2][1] - j[2][2] * j[0][1];
  adj[1][1] = j[0][0] * j[2][2] - j[2][0] * j[0][2];
  adj[1][2] = j[0][1] * j[2][0] - j[2][1] * j[0][0];
  adj[2][0] = j[0][1] * j[1][2] - j[1][1] * j[0][2];
  adj[2][1] = j[0][2] * j[1][0] - j[1][2] * j[0][0];
  adj[2][2] = j[0][0] * j[1][1] - j[1][0] * j[0][1];
  det = j[0][0] * adj[0][0] + j[1][0] * adj[1][0] + j[2][0] * adj[2][0];
}

// Per-ip geometry used by the scalar kernels.
struct IpGeom {
  double area[3];  // SCS area vector, oriented left -> right node
  double G[3];     // adj(J)^T * area
  double det;      // det(J)
};

// Geometry of one ip.  SHIFT selects the shifted (grad-op) location; the
// area vector always comes from the standard location.
template <int IP>
NALU_HD void ip_geometry(const EdgeForm& f, IpGeom& g) {
  double j[3][3], adj[3][3], det;
  jacobian_ip<IP, false>(f, j);
  cofactor(j, adj, det);
  constexpr int d = ip_dir(IP);
  constexpr double s = 0.25 * ip_sign(IP);
#pragma unroll
  for (int i = 0; i < 3; ++i) g.area[i] = s * adj[i][d];
#pragma unroll
  for (int jj = 0; jj < 3; ++jj) g.G[jj] = adj[0][jj] * g.area[0] + adj[1][jj] * g.area[1] + adj[2][jj] * g.area[2];
  g.det = det;
}

// G and det at the shifted location for a given area vector
template <int IP>
NALU_HD void ip_shifted_G(const EdgeForm& f, const double area[3], double G[3], double& det) {
  double j[3][3], adj[3][3];
  jacobian_ip<IP, true>(f, j);
  cofactor(j, adj, det);
#pragma unroll
  for (int jj = 0; jj < 3; ++jj) G[jj] = adj[0][jj] * area[0] + adj[1][jj] * area[1] + adj[2][jj] * area[2];
}

// lhsfac[c] = scale * sum_j dN_c/ds_j(ip) * G_j   (grad op at std or shifted ip)
template <int IP, bool SHIFT>
NALU_HD void lhs_factors(const double G[3], double scale, double fac[8]) {
  constexpr double a = SHIFT ? 0.5 : 0.25;
  const double g0 = G[0] * scale, g1 = G[1] * scale, g2 = G[2] * scale;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const double d0 = dshape_ip(IP, c, 0, a), d1 = dshape_ip(IP, c, 1, a), d2 = dshape_ip(IP, c, 2, a);
    double r = 0.0;
    bool first = true;
    if (d0 != 0.0) { r = g0 * d0; first = false; }
    if (d1 != 0.0) { r = first ? g1 * d1 : r + g1 * d1; first = false; }
    if (d2 != 0.0) { r = first ? g2 * d2 : r + g2 * d2; first = false; }
    fac[c] = r;
  }
}

// interpolate a nodal scalar to an ip with the (standard or shifted) shape functions
template <int IP, bool SHIFT>
NALU_HD double interp_ip(const double v[8]) {
  constexpr double a = SHIFT ? 0.5 : 0.25;
  double r = 0.0;
  bool first = true;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const double w = shape_ip(IP, c, a);
    if (w != 0.0) {
      r = first ? w * v[c] : r + w * v[c];
      first = false;
    }
  }
  return r;
}

// ---------------------------------------------------------------------------
// Element-matrix accumulator: first touch of a row stores, later ips add, in
// ascending ip order -- the same summation order as the reference's
// zero-initialised lhs(il,ic) += / lhs(ir,ic) -= over ip (the first add of
// 0.0 is exact).  Touch order is a compile-time property of the ip loop.
// ---------------------------------------------------------------------------
NALU_HD constexpr int first_ip_of_row(int r) {
  // smallest ip whose left or right node is r
  return r == 0 ? 0 : (r == 1 ? 0 : (r == 2 ? 1 : (r == 3 ? 2 : (r == 4 ? 4 : (r == 5 ? 4 : (r == 6 ? 5 : 6))))));
}

template <int IP, class Acc>
NALU_HD void accumulate_ip(Acc& acc, const double fac[8]) {
  constexpr int il = ip_left(IP), ir = ip_right(IP);
  constexpr bool fl = first_ip_of_row(il) == IP;
  constexpr bool fr = first_ip_of_row(ir) == IP;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    if (fl) acc.set(il, c, fac[c]); else acc.add(il, c, fac[c]);
    if (fr) acc.set(ir, c, -fac[c]); else acc.add(ir, c, -fac[c]);
  }
}

// compile-time ip loop
template <int IP, int N>
struct IpLoop {
  template <class F>
  NALU_HD static void run(F& f) {
    f.template apply<IP>();
    IpLoop<IP + 1, N>::run(f);
  }
};
template <int N>
struct IpLoop<N, N> {
  template <class F>
  NALU_HD static void run(F&) {}
};

// ---------------------------------------------------------------------------
// ScalarDiffElemKernel (src/kernel/ScalarDiffElemKernel.C:66-110):
//   lhs(il,c) += -k_ip dndx(ip,c).A ; lhs(ir,c) -= ... ; rhs = -lhs q
// ---------------------------------------------------------------------------
template <bool SHIFT, class Acc>
struct ScalarDiffBody {
  const EdgeForm& f;
  const double* k;
  Acc& acc;
  double mindet;  // smallest det(J) seen (negative-Jacobian check)
  template <int IP>
  NALU_HD void apply() {
    IpGeom g;
    ip_geometry<IP>(f, g);
    double G[3] = {g.G[0], g.G[1], g.G[2]};
    double det = g.det;
    if (SHIFT) ip_shifted_G<IP>(f, g.area, G, det);
    mindet = det < mindet ? det : mindet;
    const double kIp = interp_ip<IP, false>(k);  // kernel ctor uses shape_fcn (:46)
    double fac[8];
    lhs_factors<IP, SHIFT>(G, -kIp / det, fac);
    accumulate_ip<IP>(acc, fac);
  }
};

template <bool SHIFT, class Acc>
NALU_HD double scalar_diff_lhs(const double x[8][3], const double k[8], Acc& acc) {
  EdgeForm f;
  edge_form(x, f);
  ScalarDiffBody<SHIFT, Acc> body{f, k, acc, 1.0e300};
  IpLoop<0, 12>::run(body);
  return body.mindet;
}

// ---------------------------------------------------------------------------
// ContinuityAdvElemKernel (src/kernel/ContinuityAdvElemKernel.C:79-147).
// MODE 0: default (standard grad op on both sides)
// MODE 1: reduced sensitivities (lhs shifted, rhs standard)
// MODE 2: shifted Poisson (both shifted)
// SMDOT : shifted shape functions for the mass flux interpolation.
// The caller finishes rhs(r) += -sum_c lhs_rhsop(r,c) p_c (for MODE 0/2 the
// rhs operator is the lhs itself; MODE 1 keeps a separate operator in
// `rhs_p` accumulated here).
// ---------------------------------------------------------------------------
template <int MODE, bool SMDOT, class Acc>
struct ContinuityBody {
  const EdgeForm& f;
  const double (*w)[3];  // rho*u + tau*Gpdx at the nodes
  double inv_tau;
  const double* p;
  Acc& acc;
  double* rhs;  // [8]
  double mindet;
  template <int IP>
  NALU_HD void apply() {
    IpGeom g;
    ip_geometry<IP>(f, g);
    constexpr int il = ip_left(IP), ir = ip_right(IP);
    double fac[8];
    mindet = g.det < mindet ? g.det : mindet;
    if (MODE == 0) {
      lhs_factors<IP, false>(g.G, -1.0 / g.det, fac);
    } else {
      double Gs[3], dets;
      ip_shifted_G<IP>(f, g.area, Gs, dets);
      mindet = dets < mindet ? dets : mindet;
      lhs_factors<IP, true>(Gs, -1.0 / dets, fac);
    }
    accumulate_ip<IP>(acc, fac);
    // mdot/tau = (rho u + tau Gp).A / tau - dpdx.A ;  dpdx.A = sum_c p_c dndx(c).A
    double wx = 0.0, wy = 0.0, wz = 0.0;
    {
      double t0[8], t1[8], t2[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) { t0[c] = w[c][0]; t1[c] = w[c][1]; t2[c] = w[c][2]; }
      wx = interp_ip<IP, SMDOT>(t0);
      wy = interp_ip<IP, SMDOT>(t1);
      wz = interp_ip<IP, SMDOT>(t2);
    }
    double m = (wx * g.area[0] + wy * g.area[1] + wz * g.area[2]) * inv_tau;
    if (MODE == 1) {
      // rhs pressure gradient with the standard grad op
      double fs[8];
      lhs_factors<IP, false>(g.G, -1.0 / g.det, fs);  // = -dndx_std(c).A
      double dpa = 0.0;
#pragma unroll
      for (int c = 0; c < 8; ++c) dpa = dpa + fs[c] * p[c];
      m = m + dpa;  // -(dpdx.A) = sum_c p_c * fs_c
    }
    rhs[il] -= m;
    rhs[ir] += m;
  }
};

template <int MODE, bool SMDOT, class Acc>
NALU_HD double continuity_elem(const double x[8][3], const double w[8][3], double inv_tau, const double p[8],
                               Acc& acc, double rhs[8]) {
  EdgeForm f;
  edge_form(x, f);
#pragma unroll
  for (int r = 0; r < 8; ++r) rhs[r] = 0.0;
  ContinuityBody<MODE, SMDOT, Acc> body{f, w, inv_tau, p, acc, rhs, 1.0e300};
  IpLoop<0, 12>::run(body);
  return body.mindet;
}

// ---------------------------------------------------------------------------
// Mass flow rate at the SCS (ComputeMdotElemAlgorithm.C:200-245):
//   mdot = (rho u - tau (dpdx - Gp)).A
// ---------------------------------------------------------------------------
template <bool SMDOT, bool SPOIS>
struct MdotBody {
  const EdgeForm& f;
  const double (*w)[3];  // rho*u + tau*Gpdx
  const double* p;
  double tau;
  double* mdot;
  double mindet;
  template <int IP>
  NALU_HD void apply() {
    IpGeom g;
    ip_geometry<IP>(f, g);
    mindet = g.det < mindet ? g.det : mindet;
    double t0[8], t1[8], t2[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) { t0[c] = w[c][0]; t1[c] = w[c][1]; t2[c] = w[c][2]; }
    const double m0 = interp_ip<IP, SMDOT>(t0) * g.area[0] + interp_ip<IP, SMDOT>(t1) * g.area[1] +
                      interp_ip<IP, SMDOT>(t2) * g.area[2];
    double fs[8];
    if (SPOIS) {
      double Gs[3], dets;
      ip_shifted_G<IP>(f, g.area, Gs, dets);
      lhs_factors<IP, true>(Gs, 1.0 / dets, fs);  // = dndx(c).A
    } else {
      lhs_factors<IP, false>(g.G, 1.0 / g.det, fs);
    }
    double dpa = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) dpa = dpa + fs[c] * p[c];
    mdot[IP] = m0 - tau * dpa;
  }
};

template <bool SMDOT, bool SPOIS>
NALU_HD double mdot_elem(const double x[8][3], const double w[8][3], const double p[8], double tau,
                         double mdot[12]) {
  EdgeForm f;
  edge_form(x, f);
  MdotBody<SMDOT, SPOIS> body{f, w, p, tau, mdot, 1.0e300};
  IpLoop<0, 12>::run(body);
  return body.mindet;
}

// Plain array accumulator (host check and small paths)
struct ArrayAcc {
  double* m;  // [8][8]
  NALU_HD void set(int r, int c, double v) { m[r * 8 + c] = v; }
  NALU_HD void add(int r, int c, double v) { m[r * 8 + c] += v; }
};

}  // namespace nalu_gb300
