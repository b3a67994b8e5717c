// heat_conduction.cpp -- C++ caller of the library through include/nalu_gb300.hpp,
// written the way a Nalu equation system drives this path
// (EquationSystem::assemble_and_solve, src/EquationSystem.C:264-307):
// register a kernel, build the graph, zero, assemble, apply Dirichlet rows,
// load, solve.  Heat conduction on an N^3 unit-cube block mesh with +-10 %
// interior jitter, k = 1, T = 0 at x = 0 and T = 1 at x = 1.
// Prints one JSON line with the solve result.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "../../include/nalu_gb300.hpp"

int main(int argc, char** argv) {
  const int N = argc > 1 ? std::atoi(argv[1]) : 32;
  const int n1 = N + 1;
  const int64_t nn = (int64_t)n1 * n1 * n1, ne = (int64_t)N * N * N;
  std::vector<double> x(3 * nn), T(nn), k(nn, 1.0);
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0), U01(0.0, 1.0);
  const double h = 1.0 / N;
  for (int kk = 0; kk < n1; ++kk)
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n1; ++i) {
        const int64_t a = i + (int64_t)n1 * (j + (int64_t)n1 * kk);
        const bool interior = i > 0 && i < N && j > 0 && j < N && kk > 0 && kk < N;
        x[3 * a] = i * h + (interior ? 0.1 * h * U(rng) : 0.0);
        x[3 * a + 1] = j * h + (interior ? 0.1 * h * U(rng) : 0.0);
        x[3 * a + 2] = kk * h + (interior ? 0.1 * h * U(rng) : 0.0);
        T[a] = U01(rng);
      }
  std::vector<int32_t> conn(8 * ne);
  auto id = [&](int i, int j, int kk) { return (int32_t)(i + n1 * (j + n1 * kk)); };
  for (int kk = 0; kk < N; ++kk)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        int32_t* c = &conn[8 * (i + (int64_t)N * (j + (int64_t)N * kk))];
        c[0] = id(i, j, kk); c[1] = id(i + 1, j, kk); c[2] = id(i + 1, j + 1, kk); c[3] = id(i, j + 1, kk);
        c[4] = id(i, j, kk + 1); c[5] = id(i + 1, j, kk + 1); c[6] = id(i + 1, j + 1, kk + 1); c[7] = id(i, j + 1, kk + 1);
      }
  try {
    nalu_gb300::Context ctx(0);
    ctx.mesh(nn, ne, conn.data(), nullptr, x.data());
    ctx.field(NALU_FIELD_SCALAR_Q, T.data(), nn);
    ctx.field(NALU_FIELD_DIFF_COEFF, k.data(), nn);
    nalu_gb300::LinearSystem linsys(ctx, 1);
    nalu_gb300::AssembleElemSolverAlgorithm alg(linsys);
    nalu_gb300::ScalarDiffElemKernel diff;
    alg.activeKernels_.push_back(&diff);
    alg.initialize_connectivity();
    linsys.finalizeLinearSystem();
    linsys.zeroSystem();
    alg.execute();
    std::vector<int32_t> nodes;
    std::vector<double> bc, cur;
    for (int64_t a = 0; a < nn; ++a) {
      if (x[3 * a] == 0.0 || x[3 * a] == 1.0) {
        nodes.push_back((int32_t)a);
        bc.push_back(x[3 * a] == 0.0 ? 0.0 : 1.0);
        cur.push_back(T[a]);
      }
    }
    linsys.applyDirichletBCs(nodes, bc, cur, 0, 1);
    linsys.loadComplete();
    linsys.solverOpts.tol = 1e-8;
    const int status = linsys.solve();
    std::printf("{\"N\": %d, \"status\": %d, \"iterations\": %d, \"true_rel_res\": %.3e}\n", N, status,
                linsys.linearSolveIterations(), linsys.linearResidual());
    return status == 0 ? 0 : 2;
  } catch (const nalu_gb300::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
    return 1;
  }
}
