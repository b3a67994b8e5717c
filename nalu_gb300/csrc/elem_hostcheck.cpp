// elem_hostcheck.cpp -- host build of the element math in hex8_elem.h.
//
// The sm_103a kernels and this file include the same header, so the CPU test
// suite can check the restructured element math against the oracle on
// thousands of random elements without a GPU.  Exposes plain C entry points.
#include <cstdint>

#include "hex8_elem.h"

using namespace nalu_gb300;

namespace {
template <class F>
void with_x(const double* xin, F f) {
  double x[8][3];
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) x[n][d] = xin[n * 3 + d];
  f(x);
}
}  // namespace

extern "C" {

void hc_scalar_diff(const double* xin, const double* q, const double* k, int shift, double* lhs,
                    double* rhs) {
  with_x(xin, [&](double (&x)[8][3]) {
    ArrayAcc acc{lhs};
    if (shift) scalar_diff_lhs<true>(x, k, acc);
    else scalar_diff_lhs<false>(x, k, acc);
  });
  for (int r = 0; r < 8; ++r) {
    double s = 0.0;
    for (int c = 0; c < 8; ++c) s += lhs[r * 8 + c] * q[c];
    rhs[r] = -s;
  }
}

void hc_continuity(const double* xin, const double* u, const double* rho, const double* p,
                   const double* gp, double tau, int smdot, int spois, int reduced, double* lhs,
                   double* rhs) {
  double w[8][3];
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) w[n][d] = rho[n] * u[n * 3 + d] + tau * gp[n * 3 + d];
  const int mode = spois ? 2 : (reduced ? 1 : 0);
  with_x(xin, [&](double (&x)[8][3]) {
    ArrayAcc acc{lhs};
    const double it = 1.0 / tau;
    if (mode == 0) {
      if (smdot) continuity_elem<0, true>(x, w, it, p, acc, rhs);
      else continuity_elem<0, false>(x, w, it, p, acc, rhs);
    } else if (mode == 1) {
      if (smdot) continuity_elem<1, true>(x, w, it, p, acc, rhs);
      else continuity_elem<1, false>(x, w, it, p, acc, rhs);
    } else {
      if (smdot) continuity_elem<2, true>(x, w, it, p, acc, rhs);
      else continuity_elem<2, false>(x, w, it, p, acc, rhs);
    }
  });
  if (mode != 1) {
    for (int r = 0; r < 8; ++r) {
      double s = 0.0;
      for (int c = 0; c < 8; ++c) s += lhs[r * 8 + c] * p[c];
      rhs[r] -= s;
    }
  }
}

void hc_mdot(const double* xin, const double* rho, const double* u, const double* p,
             const double* gp, double tau, int smdot, int spois, double* mdot) {
  double w[8][3];
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) w[n][d] = rho[n] * u[n * 3 + d] + tau * gp[n * 3 + d];
  with_x(xin, [&](double (&x)[8][3]) {
    if (smdot) {
      if (spois) mdot_elem<true, true>(x, w, p, tau, mdot);
      else mdot_elem<true, false>(x, w, p, tau, mdot);
    } else {
      if (spois) mdot_elem<false, true>(x, w, p, tau, mdot);
      else mdot_elem<false, false>(x, w, p, tau, mdot);
    }
  });
}
}

// ---- double-float (df64) element math, as the df64 kernels run it ----
#include "hex8_elem_df.h"

extern "C" {

void hc_scalar_diff_df(const double* xin, const double* q, const double* k, int shift, double* lhs,
                       double* rhs) {
  df64 kd[8], m[64];
  int kexp = 0;
  for (int n = 0; n < 8; ++n) kd[n] = df_split_input(k[n]);
  with_x(xin, [&](double (&x)[8][3]) {
    df64 rr_acc[8];
    ArrayAccDF acc{m, rr_acc};
    if (shift) scalar_diff_lhs_df<true>(x, kd, acc, kexp);
    else scalar_diff_lhs_df<false>(x, kd, acc, kexp);
  });
  for (int i = 0; i < 64; ++i) lhs[i] = df_to_double_bits(m[i], kexp);
  for (int r = 0; r < 8; ++r) {
    double s = 0.0;
    for (int c = 0; c < 8; ++c) s += lhs[r * 8 + c] * q[c];
    rhs[r] = -s;
  }
}

void hc_mdot_df(const double* xin, const double* rho, const double* u, const double* p, const double* gp,
                double tau, int smdot, int spois, double* mdot) {
  df64 w[8][3], pd[8];
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) w[n][d] = df_nodal_w(df_split_input(rho[n]), u[n * 3 + d], df_split_input(tau), gp[n * 3 + d]);
  for (int n = 0; n < 8; ++n) pd[n] = df_split_bits(p[n]);
  const df64 t = df_from_double(tau);
  with_x(xin, [&](double (&x)[8][3]) {
    if (smdot) {
      if (spois) mdot_elem_df<true, true>(x, w, pd, t, mdot);
      else mdot_elem_df<true, false>(x, w, pd, t, mdot);
    } else {
      if (spois) mdot_elem_df<false, true>(x, w, pd, t, mdot);
      else mdot_elem_df<false, false>(x, w, pd, t, mdot);
    }
  });
}

// the per-node pass of the df64 continuity kernels on n values: w = rho u +
// tau gp as a pair (hi, lo) per value, and whether every input was inside the
// pairs' range (the condition the device pass flags)
int hc_nodal_w(int64_t n, const double* rho, const double* u, double tau, const double* gp, float* hi, float* lo) {
  int ok = 1;
  const df64 t = df_split_input(tau);
  for (int64_t i = 0; i < n; ++i) {
    const df64 w = df_nodal_w(df_split_input(rho[i]), u[i], t, gp[i]);
    hi[i] = w.hi;
    lo[i] = w.lo;
    ok &= df_split_in_range(rho[i]) && df_split_in_range(u[i]) && df_split_in_range(gp[i]) ? 1 : 0;
  }
  return ok && df_split_in_range(tau);
}

void hc_continuity_df(const double* xin, const double* u, const double* rho, const double* p,
                      const double* gp, double tau, int smdot, int spois, int reduced, double* lhs,
                      double* rhs) {
  df64 w[8][3], m[64], r8[8], pd[8];
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) w[n][d] = df_nodal_w(df_split_input(rho[n]), u[n * 3 + d], df_split_input(tau), gp[n * 3 + d]);
  for (int n = 0; n < 8; ++n) pd[n] = df_split_bits(p[n]);
  const int mode = spois ? 2 : (reduced ? 1 : 0);
  const df64 it = df_from_double(1.0 / tau);
  int kexp = 0;
  with_x(xin, [&](double (&x)[8][3]) {
    df64 rr_acc[8];
    ArrayAccDF acc{m, rr_acc};
    if (mode == 0) {
      if (smdot) continuity_elem_df<0, true>(x, w, it, pd, acc, r8, kexp);
      else continuity_elem_df<0, false>(x, w, it, pd, acc, r8, kexp);
    } else if (mode == 1) {
      if (smdot) continuity_elem_df<1, true>(x, w, it, pd, acc, r8, kexp);
      else continuity_elem_df<1, false>(x, w, it, pd, acc, r8, kexp);
    } else {
      if (smdot) continuity_elem_df<2, true>(x, w, it, pd, acc, r8, kexp);
      else continuity_elem_df<2, false>(x, w, it, pd, acc, r8, kexp);
    }
  });
  for (int i = 0; i < 64; ++i) lhs[i] = df_to_double_bits(m[i], kexp);
  for (int r = 0; r < 8; ++r) {
    double s = df_to_double_bits(r8[r], 2 * kexp);
    if (mode != 1)
      for (int c = 0; c < 8; ++c) s -= lhs[r * 8 + c] * p[c];
    rhs[r] = s;
  }
}
}
