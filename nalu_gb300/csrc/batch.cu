// batch.cu -- many independent continuity problems in one context.
//
// The meshes are one union mesh with disjoint node ranges, so the assembly is
// a single launch over all elements and the CRS graph is block diagonal.  The
// solve is Jacobi-preconditioned CG with separate alpha, beta and stop test
// per problem, run as ONE persistent cooperative kernel: every iteration of
// every problem happens inside that launch.  Rows are cut into tiles of at
// most 256 rows that never cross a problem boundary; partial sums are kept per
// tile and reduced per problem in a fixed order (deterministic).  Phases are
// separated by a grid barrier whose waits are bounded: a barrier that does not
// complete within its spin limit sets an error flag and the kernel returns,
// so a fault can never turn into a hang.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "internal.h"

namespace nalu_gb300 {
namespace {

constexpr int kBT = 256;
constexpr int kTileRows = 256;
constexpr int kTPR = 8;
constexpr long long kSpinLimit = 1ll << 25;

struct BatchArgs {
  int64_t n;
  int P, ntiles, max_it;
  const int64_t* __restrict__ rp;
  const int32_t* __restrict__ ci;
  const double* __restrict__ v;
  const double* __restrict__ dinv;
  const double* __restrict__ b;
  double* x;
  double* r;
  double* z;
  double* p;
  double* q;
  const int64_t* __restrict__ tile_row0;
  const int32_t* __restrict__ tile_rows;
  const int32_t* __restrict__ tile_prob;
  const int32_t* __restrict__ ptile0;
  const int32_t* __restrict__ ptile1;
  double* tpart;  // [3][ntiles]
  double* rz;     // [P]
  double* alpha;
  double* beta;
  double* rr;
  const double* stop2;
  int* done;   // 0 active, 1 converged, 2 breakdown
  int* iters;
  unsigned* bar_count;
  unsigned* bar_gen;
  int* err;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block sum broadcast to every thread (fixed order)
__device__ double block_sum_bcast(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) sh[32] = t;
  }
  __syncthreads();
  const double total = sh[32];
  __syncthreads();
  return total;
}

// Grid barrier with a bounded wait (sense by generation counter).
__device__ bool grid_barrier(const BatchArgs& a, int* sflag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = a.bar_gen;
    const unsigned g0 = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(a.bar_count, 1u) + 1u;
    int ok = 1;
    if (arrived == gridDim.x) {
      atomicExch(a.bar_count, 0u);
      __threadfence();
      atomicAdd(a.bar_gen, 1u);
    } else {
      long long spins = 0;
      while (*gen == g0) {
        if (++spins > kSpinLimit) {
          atomicExch(a.err, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (*(volatile int*)a.err) ok = 0;
    *sflag = ok;
  }
  __syncthreads();
  return *sflag != 0;
}

__global__ void __launch_bounds__(kBT) k_batched_cg(BatchArgs a) {
  __shared__ double sh[33];
  __shared__ int sflag;
  const int G = gridDim.x;
  for (int it = 0; it < a.max_it; ++it) {
    // A: p = z + beta p
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      const int pr = a.tile_prob[t];
      if (a.done[pr]) continue;
      const double beta = it == 0 ? 0.0 : a.beta[pr];
      const int64_t r0 = a.tile_row0[t];
      const int nr = a.tile_rows[t];
      for (int i = threadIdx.x; i < nr; i += blockDim.x) {
        const int64_t row = r0 + i;
        a.p[row] = it == 0 ? a.z[row] : a.z[row] + beta * a.p[row];
      }
    }
    if (!grid_barrier(a, &sflag)) return;
    // B: q = A p ; per-tile p.q
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      const int pr = a.tile_prob[t];
      if (a.done[pr]) {
        if (threadIdx.x == 0) a.tpart[t] = 0.0;
        continue;
      }
      const int64_t r0 = a.tile_row0[t];
      const int nr = a.tile_rows[t];
      const int sub = threadIdx.x % kTPR;
      double dot = 0.0;
      for (int base = 0; base < nr; base += kBT / kTPR) {
        const int i = base + threadIdx.x / kTPR;
        const bool valid = i < nr;
        double s = 0.0;
        int64_t row = r0 + i;
        if (valid) {
          const int64_t jb = a.rp[row], je = a.rp[row + 1];
          for (int64_t j = jb + sub; j < je; j += kTPR) s += a.v[j] * a.p[a.ci[j]];
        }
#pragma unroll
        for (int o = kTPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kTPR);
        if (valid && sub == 0) {
          a.q[row] = s;
          dot += a.p[row] * s;
        }
      }
      const double tot = block_sum_bcast(dot, sh);
      if (threadIdx.x == 0) a.tpart[t] = tot;
    }
    if (!grid_barrier(a, &sflag)) return;
    // C: alpha per problem
    for (int pr = blockIdx.x; pr < a.P; pr += G) {
      if (a.done[pr]) continue;
      double s = 0.0;
      for (int t = a.ptile0[pr] + threadIdx.x; t < a.ptile1[pr]; t += blockDim.x) s += a.tpart[t];
      const double pq = block_sum_bcast(s, sh);
      if (threadIdx.x == 0) {
        const double al = a.rz[pr] / pq;
        if (isfinite(al)) a.alpha[pr] = al;
        else {
          a.alpha[pr] = 0.0;
          a.done[pr] = 2;
        }
      }
    }
    if (!grid_barrier(a, &sflag)) return;
    // D: x += alpha p ; r -= alpha q ; z = D^-1 r ; per-tile r.z and r.r
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      const int pr = a.tile_prob[t];
      double rz = 0.0, rr = 0.0;
      if (!a.done[pr]) {
        const double al = a.alpha[pr];
        const int64_t r0 = a.tile_row0[t];
        const int nr = a.tile_rows[t];
        for (int i = threadIdx.x; i < nr; i += blockDim.x) {
          const int64_t row = r0 + i;
          a.x[row] += al * a.p[row];
          const double ri = a.r[row] - al * a.q[row];
          a.r[row] = ri;
          const double zi = a.dinv[row] * ri;
          a.z[row] = zi;
          rz += ri * zi;
          rr += ri * ri;
        }
      }
      const double trz = block_sum_bcast(rz, sh);
      const double trr = block_sum_bcast(rr, sh);
      if (threadIdx.x == 0) {
        a.tpart[a.ntiles + t] = trz;
        a.tpart[2 * a.ntiles + t] = trr;
      }
    }
    if (!grid_barrier(a, &sflag)) return;
    // E: beta, residual and stop test per problem
    for (int pr = blockIdx.x; pr < a.P; pr += G) {
      if (a.done[pr]) continue;
      double s1 = 0.0, s2 = 0.0;
      for (int t = a.ptile0[pr] + threadIdx.x; t < a.ptile1[pr]; t += blockDim.x) {
        s1 += a.tpart[a.ntiles + t];
        s2 += a.tpart[2 * a.ntiles + t];
      }
      const double rzn = block_sum_bcast(s1, sh);
      const double rrn = block_sum_bcast(s2, sh);
      if (threadIdx.x == 0) {
        const double be = rzn / a.rz[pr];
        a.beta[pr] = isfinite(be) ? be : 0.0;
        a.rz[pr] = rzn;
        a.rr[pr] = rrn;
        a.iters[pr] += 1;
        if (!isfinite(rrn) || !isfinite(be)) a.done[pr] = 2;
        else if (rrn <= a.stop2[pr]) a.done[pr] = 1;
      }
    }
    if (!grid_barrier(a, &sflag)) return;
    int active = 0;
    for (int pr = threadIdx.x; pr < a.P; pr += blockDim.x) active |= (a.done[pr] == 0);
    if (!__syncthreads_or(active)) break;
  }
}

// x = 0 except identity rows (x = b there); D^-1 and identity detection
__global__ void k_batch_prep(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                             const double* __restrict__ v, const double* __restrict__ b, double* __restrict__ dinv,
                             double* __restrict__ x, int zero) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  bool off_zero = true;
  for (int64_t j = rp[i]; j < rp[i + 1]; ++j) {
    if (ci[j] == i) d = v[j];
    else if (v[j] != 0.0) off_zero = false;
  }
  dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
  double xi = zero ? 0.0 : x[i];
  if (off_zero && d == 1.0) xi = b[i];
  x[i] = xi;
}

// r = b - A x ; z = D^-1 r ; per-tile r.z, r.r, b.b
__global__ void __launch_bounds__(kBT) k_batch_resid(BatchArgs a) {
  __shared__ double sh[33];
  for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
    const int64_t r0 = a.tile_row0[t];
    const int nr = a.tile_rows[t];
    const int sub = threadIdx.x % kTPR;
    double rz = 0.0, rr = 0.0, bb = 0.0;
    for (int base = 0; base < nr; base += kBT / kTPR) {
      const int i = base + threadIdx.x / kTPR;
      const bool valid = i < nr;
      const int64_t row = r0 + i;
      double s = 0.0;
      if (valid) {
        for (int64_t j = a.rp[row] + sub; j < a.rp[row + 1]; j += kTPR) s += a.v[j] * a.x[a.ci[j]];
      }
#pragma unroll
      for (int o = kTPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kTPR);
      if (valid && sub == 0) {
        const double ri = a.b[row] - s;
        a.r[row] = ri;
        const double zi = a.dinv[row] * ri;
        a.z[row] = zi;
        rz += ri * zi;
        rr += ri * ri;
        bb += a.b[row] * a.b[row];
      }
    }
    const double t1 = block_sum_bcast(rz, sh), t2 = block_sum_bcast(rr, sh), t3 = block_sum_bcast(bb, sh);
    if (threadIdx.x == 0) {
      a.tpart[t] = t1;
      a.tpart[a.ntiles + t] = t2;
      a.tpart[2 * a.ntiles + t] = t3;
    }
  }
}

// per-problem sums of the three tile partial arrays: out[3][P]
__global__ void k_batch_sums(const double* __restrict__ tpart, int ntiles, const int32_t* __restrict__ ptile0,
                             const int32_t* __restrict__ ptile1, int P, double* __restrict__ out) {
  __shared__ double sh[33];
  for (int pr = blockIdx.x; pr < P; pr += gridDim.x) {
    for (int k = 0; k < 3; ++k) {
      double s = 0.0;
      for (int t = ptile0[pr] + threadIdx.x; t < ptile1[pr]; t += blockDim.x) s += tpart[k * ntiles + t];
      const double tot = block_sum_bcast(s, sh);
      if (threadIdx.x == 0) out[k * P + pr] = tot;
    }
  }
}

}  // namespace

int solve_batched(nalu_ctx* ctx, const nalu_solver_opts& o, nalu_solve_info* infos) {
  const auto t0 = std::chrono::steady_clock::now();
  const int P = (int)ctx->problem_offsets.size() - 1;
  if (P < 1) return set_error(ctx, NALU_ERR_STATE, "no problem partition (nalu_set_problems)");
  const int64_t n = ctx->n_rows;
  const int nd = ctx->num_dof;
  // tiles of <= 256 rows inside each problem
  std::vector<int64_t> trow0;
  std::vector<int32_t> trows, tprob, pt0(P), pt1(P);
  for (int pr = 0; pr < P; ++pr) {
    const int64_t rb = ctx->problem_offsets[pr] * nd, re = ctx->problem_offsets[pr + 1] * nd;
    pt0[pr] = (int32_t)trow0.size();
    for (int64_t r = rb; r < re; r += kTileRows) {
      trow0.push_back(r);
      trows.push_back((int32_t)std::min<int64_t>(kTileRows, re - r));
      tprob.push_back(pr);
    }
    pt1[pr] = (int32_t)trow0.size();
  }
  const int ntiles = (int)trow0.size();
  SolverWork& s = ctx->sw;
  DBuf<int64_t> d_trow0;
  DBuf<int32_t> d_ints;   // trows | tprob | pt0 | pt1 | done | iters | err
  DBuf<double> d_dbl;     // tpart[3 ntiles] | rz alpha beta rr stop2 [P each] | sums [3P]
  DBuf<unsigned> d_bar;
  NALU_CUDA(ctx, d_trow0.alloc(ntiles));
  NALU_CUDA(ctx, d_ints.alloc(2 * (int64_t)ntiles + 4 * (int64_t)P + 1));
  NALU_CUDA(ctx, d_dbl.alloc(3 * (int64_t)ntiles + 8 * (int64_t)P));
  NALU_CUDA(ctx, d_bar.alloc(2));
  for (auto* b : {&s.r, &s.z, &s.p, &s.q, &s.dinv})
    if (b->n < n) NALU_CUDA(ctx, b->alloc(n));
  int32_t* trows_d = d_ints.p;
  int32_t* tprob_d = trows_d + ntiles;
  int32_t* pt0_d = tprob_d + ntiles;
  int32_t* pt1_d = pt0_d + P;
  int32_t* done_d = pt1_d + P;
  int32_t* iters_d = done_d + P;
  int32_t* err_d = iters_d + P;
  double* tpart = d_dbl.p;
  double* rz_d = tpart + 3 * (int64_t)ntiles;
  double* alpha_d = rz_d + P;
  double* beta_d = alpha_d + P;
  double* rr_d = beta_d + P;
  double* stop2_d = rr_d + P;
  double* sums_d = stop2_d + P;  // [3][P]
  cudaStream_t st = ctx->stream;
  NALU_CUDA(ctx, cudaMemcpyAsync(d_trow0.p, trow0.data(), sizeof(int64_t) * ntiles, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemcpyAsync(trows_d, trows.data(), sizeof(int32_t) * ntiles, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemcpyAsync(tprob_d, tprob.data(), sizeof(int32_t) * ntiles, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemcpyAsync(pt0_d, pt0.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemcpyAsync(pt1_d, pt1.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemsetAsync(done_d, 0, sizeof(int32_t) * (2 * P + 1), st));
  NALU_CUDA(ctx, cudaMemsetAsync(d_bar.p, 0, sizeof(unsigned) * 2, st));

  BatchArgs a{};
  a.n = n;
  a.P = P;
  a.ntiles = ntiles;
  a.rp = ctx->d_rowptr.p;
  a.ci = ctx->d_colind.p;
  a.v = ctx->d_values.p;
  a.dinv = s.dinv.p;
  a.b = ctx->d_rhs.p;
  a.x = ctx->d_x.p;
  a.r = s.r.p;
  a.z = s.z.p;
  a.p = s.p.p;
  a.q = s.q.p;
  a.tile_row0 = d_trow0.p;
  a.tile_rows = trows_d;
  a.tile_prob = tprob_d;
  a.ptile0 = pt0_d;
  a.ptile1 = pt1_d;
  a.tpart = tpart;
  a.rz = rz_d;
  a.alpha = alpha_d;
  a.beta = beta_d;
  a.rr = rr_d;
  a.stop2 = stop2_d;
  a.done = done_d;
  a.iters = iters_d;
  a.bar_count = d_bar.p;
  a.bar_gen = d_bar.p + 1;
  a.err = err_d;

  k_batch_prep<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, a.rp, a.ci, a.v, a.b, s.dinv.p, a.x, o.x0_zero ? 1 : 0);
  ctx->launches++;
  int blocks_per_sm = 0;
  NALU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_batched_cg, kBT, 0));
  const int grid = std::max(1, std::min(ntiles, blocks_per_sm * ctx->sm_count));
  std::vector<double> sums(3 * P);
  std::vector<int32_t> done(P), iters(P);
  std::vector<double> true_res(P, 0.0), bnorm(P, 0.0);
  int rc = NALU_OK;
  for (int outer = 0; outer < 6; ++outer) {
    // true residual, z, r.z per problem; stop when every problem is within tol
    k_batch_resid<<<std::min(ntiles, 4 * ctx->sm_count), kBT, 0, st>>>(a);
    k_batch_sums<<<std::min(P, 1024), kBT, 0, st>>>(tpart, ntiles, pt0_d, pt1_d, P, sums_d);
    ctx->launches += 2;
    NALU_CUDA(ctx, cudaMemcpyAsync(sums.data(), sums_d, sizeof(double) * 3 * P, cudaMemcpyDeviceToHost, st));
    NALU_CUDA(ctx, cudaStreamSynchronize(st));
    bool all = true;
    std::vector<double> stop2(P), rz0(P);
    for (int pr = 0; pr < P; ++pr) {
      bnorm[pr] = std::sqrt(sums[2 * P + pr]);
      const double bref = bnorm[pr] > 0 ? bnorm[pr] : 1.0;
      true_res[pr] = std::sqrt(sums[P + pr]) / bref;
      done[pr] = true_res[pr] <= o.tol ? 1 : 0;
      all = all && done[pr];
      stop2[pr] = std::pow(0.5 * o.tol * bref, 2);
      rz0[pr] = sums[pr];
    }
    if (all) break;
    NALU_CUDA(ctx, cudaMemcpyAsync(stop2_d, stop2.data(), sizeof(double) * P, cudaMemcpyHostToDevice, st));
    NALU_CUDA(ctx, cudaMemcpyAsync(rz_d, rz0.data(), sizeof(double) * P, cudaMemcpyHostToDevice, st));
    NALU_CUDA(ctx, cudaMemcpyAsync(done_d, done.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
    a.max_it = o.max_iters;
    void* args[] = {&a};
    cudaError_t ce = cudaLaunchCooperativeKernel((const void*)k_batched_cg, grid, kBT, args, 0, st);
    if (ce != cudaSuccess) return cuda_check(ctx, ce, "cooperative batched CG launch");
    ctx->launches++;
    int32_t err = 0;
    NALU_CUDA(ctx, cudaMemcpyAsync(&err, err_d, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    NALU_CUDA(ctx, cudaMemcpyAsync(done.data(), done_d, sizeof(int32_t) * P, cudaMemcpyDeviceToHost, st));
    NALU_CUDA(ctx, cudaStreamSynchronize(st));
    if (err) {
      rc = set_error(ctx, NALU_ERR_CUDA, "batched CG grid barrier timed out");
      break;
    }
  }
  NALU_CUDA(ctx, cudaMemcpyAsync(iters.data(), iters_d, sizeof(int32_t) * P, cudaMemcpyDeviceToHost, st));
  NALU_CUDA(ctx, cudaStreamSynchronize(st));
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  bool all_ok = true;
  for (int pr = 0; pr < P; ++pr) {
    infos[pr].iterations = iters[pr];
    infos[pr].outer_iterations = 1;
    infos[pr].true_rel_res = true_res[pr];
    infos[pr].seconds = secs;
    infos[pr].status = true_res[pr] <= o.tol ? NALU_OK : NALU_ERR_NOT_CONVERGED;
    all_ok = all_ok && infos[pr].status == NALU_OK;
  }
  d_trow0.free();
  d_ints.free();
  d_dbl.free();
  d_bar.free();
  if (rc) return rc;
  return all_ok ? NALU_OK : set_error(ctx, NALU_ERR_NOT_CONVERGED, "some problems did not reach the tolerance");
}

}  // namespace nalu_gb300

extern "C" {

int nalu_set_problems(nalu_ctx* ctx, int n, const int64_t* node_offsets) {
  using namespace nalu_gb300;
  if (!ctx || n < 1 || !node_offsets) return NALU_ERR_ARG;
  if (ctx->n_nodes == 0) return set_error(ctx, NALU_ERR_STATE, "no mesh");
  if (node_offsets[0] != 0 || node_offsets[n] != ctx->n_nodes)
    return set_error(ctx, NALU_ERR_ARG, "problem offsets must span [0, n_nodes]");
  for (int k = 0; k < n; ++k)
    if (node_offsets[k + 1] <= node_offsets[k]) return set_error(ctx, NALU_ERR_ARG, "empty or unordered problem");
  // every problem's nodes must occupy a contiguous LID range
  for (int k = 0; k < n; ++k)
    for (int64_t i = node_offsets[k]; i < node_offsets[k + 1]; ++i)
      if (ctx->h_lid[i] < node_offsets[k] || ctx->h_lid[i] >= node_offsets[k + 1])
        return set_error(ctx, NALU_ERR_ARG, "problem nodes must have ascending global ids problem by problem");
  // no element may couple two problems
  for (int64_t e = 0; e < ctx->n_elems; ++e) {
    const int32_t* c = &ctx->h_conn_lid[8 * e];
    const int64_t* k0 = std::upper_bound(node_offsets, node_offsets + n + 1, (int64_t)c[0]);
    for (int m = 1; m < 8; ++m)
      if (std::upper_bound(node_offsets, node_offsets + n + 1, (int64_t)c[m]) != k0)
        return set_error(ctx, NALU_ERR_ARG, "an element couples two problems");
  }
  ctx->problem_offsets.assign(node_offsets, node_offsets + n + 1);
  return NALU_OK;
}

int nalu_solve_batched(nalu_ctx* ctx, const nalu_solver_opts* opts, nalu_solve_info* infos) {
  using namespace nalu_gb300;
  if (!ctx || !opts || !infos) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  return solve_batched(ctx, *opts, infos);
}

}  // extern "C"
