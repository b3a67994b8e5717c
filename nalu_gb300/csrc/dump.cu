// dump.cu -- MatrixMarket files of the linear system and its solution, the
// format TpetraLinearSystem::writeToFile / writeSolutionToFile
// (src/TpetraLinearSystem.C:1967-2117) hands to external tools:
//
//   <base>-O-<count>.mm.1    %%MatrixMarket matrix coordinate real general,
//                            1-based global row/column ids, dimension the
//                            largest row id
//                            GID_(gid, ndof, idof) = ndof (gid - 1) + idof + 1
//                            (:72), rows in LID (global id) order
//   <base>-O-<count>.rhs.1   %%MatrixMarket matrix array real general, n x 1
//   <base>-O-<count>.sln.1   the same for the solution; writing it advances
//                            count (the reference does both after a solve,
//                            :1813-1817)
//
// One rank, so the ".1" suffix is the reference's p_size.  Values carry 17
// significant digits (they read back bit for bit).  Host code only.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "internal.h"

using namespace nalu_gb300;

namespace {

std::string file_name(const nalu_ctx* ctx, const char* base, const char* kind) {
  return std::string(base) + "-O-" + std::to_string(ctx->write_counter) + "." + kind + ".1";
}

int64_t row_gid(const nalu_ctx* ctx, int64_t lid_row) {
  const int nd = ctx->num_dof;
  return (int64_t)nd * (ctx->h_gid[lid_row / nd] - 1) + lid_row % nd + 1;
}

int write_dense(nalu_ctx* ctx, const std::string& path, const double* d_vec) {
  std::vector<double> v((size_t)ctx->n_rows);
  NALU_CUDA(ctx, cudaMemcpyAsync(v.data(), d_vec, sizeof(double) * ctx->n_rows, cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return set_error(ctx, NALU_ERR_ARG, "cannot open " + path);
  std::fprintf(f, "%%%%MatrixMarket matrix array real general\n%lld 1\n", (long long)ctx->n_rows);
  for (double x : v) std::fprintf(f, "%.16e\n", x);
  const bool ok = std::fclose(f) == 0;
  return ok ? NALU_OK : set_error(ctx, NALU_ERR_ARG, "write failed: " + path);
}

}  // namespace

extern "C" {

int nalu_linsys_write_system(nalu_ctx* ctx, const char* base) {
  if (!ctx || !base) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  const int64_t n = ctx->n_rows, nnz = ctx->nnz;
  std::vector<int64_t> rp((size_t)n + 1);
  std::vector<int32_t> ci((size_t)nnz);
  std::vector<double> v((size_t)nnz);
  NALU_CUDA(ctx, cudaMemcpyAsync(rp.data(), ctx->d_rowptr.p, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost,
                                 ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(ci.data(), ctx->d_colind.p, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(v.data(), ctx->d_values.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const std::string mm = file_name(ctx, base, "mm");
  FILE* f = std::fopen(mm.c_str(), "w");
  if (!f) return set_error(ctx, NALU_ERR_ARG, "cannot open " + mm);
  // dimension: the largest global row id (n_rows when the global ids are 1..n)
  const long long dim = std::max((long long)n, (long long)row_gid(ctx, n - 1));
  std::fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n%%%s\n%%matrix for: %s\n%lld %lld %lld\n", base,
               base, dim, dim, (long long)nnz);
  for (int64_t r = 0; r < n; ++r) {
    const long long g = (long long)row_gid(ctx, r);
    for (int64_t k = rp[r]; k < rp[r + 1]; ++k)
      std::fprintf(f, "%lld %lld %.16e\n", g, (long long)row_gid(ctx, ci[k]), v[k]);
  }
  if (std::fclose(f) != 0) return set_error(ctx, NALU_ERR_ARG, "write failed: " + mm);
  return write_dense(ctx, file_name(ctx, base, "rhs"), ctx->d_rhs.p);
}

int nalu_linsys_write_solution(nalu_ctx* ctx, const char* base) {
  if (!ctx || !base) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  const int rc = write_dense(ctx, file_name(ctx, base, "sln"), ctx->d_x.p);
  if (rc == NALU_OK) ++ctx->write_counter;
  return rc;
}

}  // extern "C"
