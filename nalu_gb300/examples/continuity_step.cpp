// continuity_step.cpp -- C++ caller of the continuity path through
// include/nalu_gb300.hpp, in the order a Nalu low-Mach step drives it
// (LowMachEquationSystem / ContinuityEquationSystem, src/LowMachEquationSystem.C):
// geometry (HexSCV volumes, dual nodal volume, the skin's side set), the
// projected nodal gradient of the pressure with its boundary closure, the SCS
// mass flow (ComputeMdotElemAlgorithm), then the continuity system
// (ContinuityAdvElemKernel through AssembleElemSolverAlgorithm), the pressure
// pinned at node 0 (FixPressureAtNodeAlgorithm), and the solve.
//
// Mesh: N^3 elements on the unit cube, z spacing geometric with ratio 1.05
// (every element an axis-aligned box).  Fields: rho = 1, a divergence-free
// velocity, pressure p = 0.4 + 0.7 x - 1.3 y + 2.1 z (linear, so its
// projected nodal gradient with the closure is exact on this mesh).
// Prints one JSON line with the checks.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/nalu_gb300.hpp"

int main(int argc, char** argv) {
  const int N = argc > 1 ? std::atoi(argv[1]) : 20;
  const int n1 = N + 1;
  const int64_t nn = (int64_t)n1 * n1 * n1, ne = (int64_t)N * N * N;
  const double pi = 3.14159265358979323846;
  // z nodes: geometric spacing (ratio 1.05) normalised to [0, 1]
  std::vector<double> zs(n1, 0.0);
  {
    double h = 1.0, s = 0.0;
    for (int k = 1; k < n1; ++k, h *= 1.05) zs[k] = (s += h);
    for (int k = 1; k < n1; ++k) zs[k] /= s;
  }
  std::vector<double> x(3 * nn), u(3 * nn), rho(nn, 1.0), p(nn), gp(3 * nn, 0.0);
  const double g[3] = {0.7, -1.3, 2.1};
  for (int k = 0; k < n1; ++k)
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n1; ++i) {
        const int64_t a = i + (int64_t)n1 * (j + (int64_t)n1 * k);
        const double X = (double)i / N, Y = (double)j / N, Z = zs[k];
        x[3 * a] = X;
        x[3 * a + 1] = Y;
        x[3 * a + 2] = Z;
        u[3 * a] = std::sin(pi * X) * std::cos(pi * Y);
        u[3 * a + 1] = -std::cos(pi * X) * std::sin(pi * Y);
        u[3 * a + 2] = 0.1 * std::sin(pi * X);
        p[a] = 0.4 + g[0] * X + g[1] * Y + g[2] * Z;
      }
  std::vector<int32_t> conn(8 * ne);
  auto id = [&](int i, int j, int k) { return (int32_t)(i + n1 * (j + n1 * k)); };
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        int32_t* c = &conn[8 * (i + (int64_t)N * (j + (int64_t)N * k))];
        c[0] = id(i, j, k); c[1] = id(i + 1, j, k); c[2] = id(i + 1, j + 1, k); c[3] = id(i, j + 1, k);
        c[4] = id(i, j, k + 1); c[5] = id(i + 1, j, k + 1); c[6] = id(i + 1, j + 1, k + 1); c[7] = id(i, j + 1, k + 1);
      }
  try {
    using namespace nalu_gb300;
    Context ctx(0);
    ctx.mesh(nn, ne, conn.data(), nullptr, x.data());
    ctx.field(NALU_FIELD_VELOCITY, u.data(), 3 * nn);
    ctx.field(NALU_FIELD_VELOCITY_RTM, u.data(), 3 * nn);
    ctx.field(NALU_FIELD_DENSITY, rho.data(), nn);
    ctx.field(NALU_FIELD_PRESSURE, p.data(), nn);
    ctx.field(NALU_FIELD_DPDX, gp.data(), 3 * nn);

    // master elements, batched over every element: the SCV volumes add up to
    // the unit cube, and the eight shape-function gradients sum to zero at
    // every ip (the shape functions are a partition of unity)
    std::vector<double> ecoords(24 * ne);
    for (int64_t e = 0; e < ne; ++e)
      for (int n = 0; n < 8; ++n)
        for (int d = 0; d < 3; ++d) ecoords[24 * e + 3 * n + d] = x[3 * (int64_t)conn[8 * e + n] + d];
    HexSCV scv(ctx);
    std::vector<double> vol(8 * ne);
    scv.determinant(ne, ecoords.data(), vol.data());
    double vsum = 0.0;
    for (double v : vol) vsum += v;
    HexSCS scs(ctx);
    std::vector<double> areav(36 * ne), gradop(288 * ne);
    scs.determinant(ne, ecoords.data(), areav.data());
    const bool jac_ok = scs.grad_op(ne, ecoords.data(), gradop.data());
    double gsum = 0.0;
    for (int64_t e = 0; e < ne; ++e)
      for (int ip = 0; ip < 12; ++ip)
        for (int d = 0; d < 3; ++d) {
          double s = 0.0;
          for (int n = 0; n < 8; ++n) s += gradop[288 * e + 24 * ip + 3 * n + d];
          gsum = std::max(gsum, std::fabs(s));
        }
    const std::vector<int32_t> lr = HexSCS::adjacentNodes();
    const std::vector<double> shp = HexSCS::shape_fcn();

    // dual nodal volume and the projected nodal gradient with the skin closure
    ctx.computeDualNodalVolume();
    std::vector<double> dvol(nn);
    ctx.fieldGet(NALU_FIELD_DUAL_VOLUME, dvol.data(), nn);
    double dsum = 0.0;
    for (double v : dvol) dsum += v;
    const int64_t skin_faces = ctx.skin(0);
    AssembleNodalGradElemAlgorithm grad(ctx, NALU_FIELD_PRESSURE, NALU_FIELD_DPDX);
    grad.boundarySets_.push_back(0);
    grad.execute();
    std::vector<double> dpdx(3 * nn);
    ctx.fieldGet(NALU_FIELD_DPDX, dpdx.data(), 3 * nn);
    double gerr = 0.0;
    for (int64_t a = 0; a < nn; ++a)
      for (int d = 0; d < 3; ++d) gerr = std::max(gerr, std::fabs(dpdx[3 * a + d] - g[d]));

    // SCS mass flow with that gradient as Gpdx: for a linear p on boxes the
    // pressure terms cancel, so mdot = rho u_ip . A_ip with u_ip from the
    // SCS shape functions and A_ip from HexSCS::determinant
    TimeIntegrator ti;
    ComputeMdotElemAlgorithm mdot(ctx);
    mdot.execute(ti);
    std::vector<double> md(12 * ne);
    ctx.fieldGet(NALU_FIELD_MDOT_SCS, md.data(), 12 * ne);
    double merr = 0.0, mmax = 0.0;
    for (int64_t e = 0; e < ne; ++e)
      for (int ip = 0; ip < 12; ++ip) {
        double ref = 0.0;
        for (int d = 0; d < 3; ++d) {
          double ui = 0.0;
          for (int n = 0; n < 8; ++n) ui += shp[8 * ip + n] * u[3 * (int64_t)conn[8 * e + n] + d];
          ref += ui * areav[36 * e + 3 * ip + d];
        }
        merr = std::max(merr, std::fabs(md[12 * e + ip] - ref));
        mmax = std::max(mmax, std::fabs(ref));
      }

    // the continuity system, the pin at node 0, the solve
    LinearSystem linsys(ctx, 1);
    AssembleElemSolverAlgorithm alg(linsys);
    ContinuityAdvElemKernel cont;
    alg.activeKernels_.push_back(&cont);
    alg.initialize_connectivity();
    linsys.finalizeLinearSystem();
    linsys.zeroSystem();
    alg.execute(ti);
    linsys.resetRows({0}, 0, 1);
    linsys.sumIntoDiagonal(0, 0, 1.0, 0.0);
    linsys.loadComplete();
    int64_t rows = 0, nnz = 0;
    linsys.sizes(&rows, &nnz);
    linsys.solverOpts.tol = 1e-8;
    const int status = linsys.solve();
    std::printf(
        "{\"N\": %d, \"scv_volume_sum_err\": %.3e, \"dual_volume_sum_err\": %.3e, \"grad_op_row_sum\": %.3e, "
        "\"jacobians_positive\": %s, \"lrscv_0\": [%d, %d], \"skin_faces\": %lld, \"linear_gradient_err\": %.3e, "
        "\"mdot_rel_err\": %.3e, \"rows\": %lld, \"nnz\": %lld, \"status\": %d, "
        "\"iterations\": %d, \"true_rel_res\": %.3e}\n",
        N, std::fabs(vsum - 1.0), std::fabs(dsum - 1.0), gsum, jac_ok ? "true" : "false", lr[0], lr[1],
        (long long)skin_faces, gerr, merr / (mmax > 0.0 ? mmax : 1.0), (long long)rows, (long long)nnz, status,
        linsys.linearSolveIterations(), linsys.linearResidual());
    return status == 0 ? 0 : 2;
  } catch (const nalu_gb300::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
    return 1;
  }
}
