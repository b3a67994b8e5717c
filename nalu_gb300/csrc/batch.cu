// batch.cu -- many independent continuity problems in one context.
//
// The meshes are one union mesh with disjoint node ranges, so the assembly is
// a single launch over all elements and the CRS graph is block diagonal.  The
// solve is Jacobi-preconditioned CG with a separate alpha, beta and stop test
// per problem, on the same arithmetic as the single-system CG (cg_fast.cu):
// df64 SELL-32 SpMV, search direction as FP32 pairs, dot products as FP32
// pairs, x and r in FP64.
//
// Rows are cut into tiles of at most 1024 rows that never cross a problem
// boundary; one block owns one tile and one thread four of its rows.  An iteration is
// three kernels over the tiles:
//   pupdate  p = D^-1 r + beta_p p
//   spmv     q = A p, tile sums of p.q; the last tile of a problem to finish
//            (per-problem atomic ticket after a fence) sums that problem's
//            tile partials in a fixed order and writes alpha_p
//   axpy     x += alpha_p p, r -= alpha_p q, tile sums of r.D^-1 r and r.r;
//            the last tile of a problem writes beta_p, and marks the problem
//            done when its recursive residual is below its stop value
// Tiles of finished problems return at once, so the work shrinks as problems
// converge.  With the learned preconditioner every problem runs flexible CG
// (a fourth kernel applies the learned stencil, z = M r, and the last tile
// forms beta from z . q_old); a problem whose step turns non-positive
// continues with Jacobi-CG after the next restart.  A chunk of iterations is
// captured into a CUDA graph; the host reads the done flags between chunks and
// ends the solve with the true FP64 residual of every problem.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "internal.h"
#include "reduce.cuh"
#include "spmv_df.cuh"

namespace nalu_gb300 {
namespace {

constexpr int kBT = 256;                  // threads per block (one block per tile)
constexpr int kRowsPerThread = 4;         // default: a tile's fixed costs (block sums, ticket) over 4 rows a thread
constexpr int kTileRows = kRowsPerThread * kBT;
constexpr int kTileCandidates[4] = {256, 512, 1024, 2048};  // rows per tile the autotuner times
constexpr int kSliceB = 32;

struct GraphExecs {
  cudaGraphExec_t e[2] = {nullptr, nullptr};
  ~GraphExecs() {
    for (auto x : e)
      if (x) cudaGraphExecDestroy(x);
  }
};

struct TileArgs {
  int64_t n;
  int P, ntiles;
  const int64_t* __restrict__ tile_row0;
  const int32_t* __restrict__ tile_rows;
  const int32_t* __restrict__ tile_prob;
  const int32_t* __restrict__ ptile0;
  const int32_t* __restrict__ ptile1;
  // SELL-32 copy of the union matrix
  const int64_t* __restrict__ sptr;
  const int32_t* __restrict__ slen;
  const int32_t* __restrict__ scol;
  const uint16_t* __restrict__ col16;  // 16-bit column offsets (see cg_fast.cu)
  const int32_t* __restrict__ cbase;
  const uint8_t* __restrict__ wide;
  const float2* __restrict__ sval;
  const float* __restrict__ dinvf;
  double* x;    // FP64 solution, accumulated over rounds
  double* r;    // FP64 residual at the start of a round
  float2* x2;   // this round's increment, FP32 pairs (folded into x after the round)
  float2* r2;   // residual, FP32 pairs
  float2* q2;   // A p, FP32 pairs
  float2* p;
  double* tpart;        // [2][ntiles]
  unsigned* pcnt;       // [P] arrival tickets
  double* alpha;        // [P]
  double* beta;         // [P]
  double* rz;           // [P]
  double* rr;           // [P]
  const double* stop2;  // [P]
  int* done;            // [P] 0 active, 1 converged, 2 breakdown, 3 flexible-CG step not positive
  int* iters;           // [P] iterations in total
  // flexible CG: z = M r with the learned stencil values (mode 1) or from the
  // multigrid V-cycle on the union system (mode 2, zf)
  const float* wsell;   // preconditioner values on the SELL pattern (or null)
  double* z;            // [n]
  const int* mode;      // [P] 0 Jacobi-CG, 1 learned FCG, 2 multigrid FCG
  float* rf;            // [n] FP32 residual, the V-cycle's input (mode 2)
  const float* zf;      // [n] the V-cycle's output (mode 2)
  double* pq;           // [P] p.Ap of the previous iteration
  int* kiter;           // [P] iterations since the last restart
  int* liters;          // [P] iterations in flexible CG (learned or multigrid)
};

// The last tile of problem pr to arrive returns true (after a fence), with
// the problem's tile partials summed in a fixed order into tot[].
template <int K>
__device__ bool problem_reduce(const TileArgs& a, int t, int pr, const double (&v)[K], double (&tot)[K],
                               double* sh) {
  __shared__ unsigned ticket;
  for (int k = 0; k < K; ++k) {
    const double s = red::block_sum(v[k], sh);
    if (threadIdx.x == 0) a.tpart[k * a.ntiles + t] = s;
  }
  const int t0 = a.ptile0[pr], t1 = a.ptile1[pr];
  if (threadIdx.x == 0) {
    __threadfence();
    ticket = atomicAdd(a.pcnt + pr, 1u);
  }
  __syncthreads();
  if (ticket != (unsigned)(t1 - t0 - 1)) return false;
  __threadfence();
  for (int k = 0; k < K; ++k) {
    double s = 0.0;
    for (int i = t0 + threadIdx.x; i < t1; i += blockDim.x) s += __ldcg(a.tpart + k * a.ntiles + i);
    tot[k] = red::block_sum(s, sh);
  }
  if (threadIdx.x == 0) a.pcnt[pr] = 0u;
  return true;
}

// multigrid problems: the V-cycle's FP32 input, the high part of r
__global__ void __launch_bounds__(kBT) k_bt_hi(TileArgs a) {
  const int t = blockIdx.x;
  const int pr = a.tile_prob[t];
  if (a.done[pr] || a.mode[pr] != 2) return;
  for (int i = threadIdx.x; i < a.tile_rows[t]; i += kBT) {
    const int64_t row = a.tile_row0[t] + i;
    a.rf[row] = a.r2[row].x;
  }
}

// flexible-CG problems: z = M r (learned: FP32 stencil values; multigrid: the
// V-cycle's output); beta = -(z . q_old) / (p . q)_old
__global__ void __launch_bounds__(kBT) k_bt_prec(TileArgs a) {
  __shared__ double sh[33];
  const int t = blockIdx.x;
  const int pr = a.tile_prob[t];
  const int m = a.mode[pr];
  if (a.done[pr] || m == 0) return;
  double dot = 0.0;
  for (int i = threadIdx.x; i < a.tile_rows[t]; i += kBT) {
    const int64_t row = a.tile_row0[t] + i;
    if (m == 2) {
      const double zi = widen_f(a.zf[row]);
      a.z[row] = zi;
      dot += zi * join_df(a.q2[row]);
      continue;
    }
    const int64_t sl = row / kSliceB;
    const int64_t b0 = __ldg(a.sptr + sl);
    const int64_t base = b0 + (row % kSliceB);
    const int len = __ldg(a.slen + sl);
    float acc = 0.0f;
    if (__ldg(a.wide + sl)) {
      for (int k = 0; k < len; ++k) {
        const int64_t e = base + (int64_t)k * kSliceB;
        acc = fmaf(__ldg(a.wsell + e), __ldg(a.r2 + __ldg(a.scol + e)).x, acc);
      }
    } else {
      const int32_t* cb = a.cbase + b0 / kSliceB;
      for (int k = 0; k < len; ++k) {
        const int64_t e = base + (int64_t)k * kSliceB;
        acc = fmaf(__ldg(a.wsell + e), __ldg(a.r2 + __ldg(cb + k) + (int32_t)__ldg(a.col16 + e)).x, acc);
      }
    }
    const double zi = widen_f(acc);
    a.z[row] = zi;
    dot += zi * join_df(a.q2[row]);
  }
  const double v[1] = {dot};
  double tot[1];
  if (problem_reduce<1>(a, t, pr, v, tot, sh) && threadIdx.x == 0)
    a.beta[pr] = a.kiter[pr] == 0 ? 0.0 : -tot[0] / a.pq[pr];
}

__global__ void __launch_bounds__(kBT) k_bt_pupdate(TileArgs a) {
  const int t = blockIdx.x;
  const int pr = a.tile_prob[t];
  if (a.done[pr]) return;
  const float2 beta = split_df(a.beta[pr]);
  const bool learned = a.mode[pr] != 0;  // flexible CG: p = z + beta p
  for (int i = threadIdx.x; i < a.tile_rows[t]; i += kBT) {
    const int64_t row = a.tile_row0[t] + i;
    const float2 z = learned ? split_df(a.z[row])
                             : fma_df(a.r2[row], make_float2(a.dinvf[row], 0.0f), make_float2(0.0f, 0.0f));
    a.p[row] = fma_df(beta, a.p[row], z);
  }
}

__global__ void __launch_bounds__(kBT) k_bt_spmv(TileArgs a) {
  __shared__ double sh[33];
  const int t = blockIdx.x;
  const int pr = a.tile_prob[t];
  if (a.done[pr]) return;
  float dh = 0.0f, dl = 0.0f, rh = 0.0f, rl = 0.0f;
  for (int i = threadIdx.x; i < a.tile_rows[t]; i += kBT) {
    const int64_t row = a.tile_row0[t] + i;
    const int64_t s = row / kSliceB;
    const int64_t b0 = __ldg(a.sptr + s);
    const int len = __ldg(a.slen + s);
    const float2 qi = __ldg(a.wide + s) ? sell_row_df2(b0 + (row % kSliceB), len, a.scol, a.sval, a.p)
                                        : sell_row_df2_c16(b0 + (row % kSliceB), len, a.col16,
                                                           a.cbase + b0 / kSliceB, a.sval, a.p);
    a.q2[row] = qi;
    const float2 pi = a.p[row];
    acc_mul_df(dh, dl, pi, qi);
    acc_mul_df(rh, rl, pi, a.r2[row]);
  }
  const double v[2] = {join_df(make_float2(dh, dl)), join_df(make_float2(rh, rl))};
  double tot[2];
  if (problem_reduce<2>(a, t, pr, v, tot, sh) && threadIdx.x == 0) {
    if (a.mode[pr] != 0) {  // flexible CG: alpha = (p . r) / (p . A p)
      const double al = tot[1] / tot[0];
      a.pq[pr] = tot[0];
      a.alpha[pr] = al;
      if (!(al > 0.0)) {  // the preconditioner is not positive on this residual
        a.alpha[pr] = 0.0;
        a.done[pr] = 3;
      }
    } else {
      a.alpha[pr] = a.rz[pr] / tot[0];
    }
  }
}

__global__ void __launch_bounds__(kBT) k_bt_axpy(TileArgs a) {
  __shared__ double sh[33];
  const int t = blockIdx.x;
  const int pr = a.tile_prob[t];
  if (a.done[pr]) return;
  float zh = 0.0f, zl = 0.0f, rh = 0.0f, rl = 0.0f;
  const float2 al = split_df(a.alpha[pr]);
  for (int i = threadIdx.x; i < a.tile_rows[t]; i += kBT) {
    const int64_t row = a.tile_row0[t] + i;
    a.x2[row] = fma_df(al, a.p[row], a.x2[row]);
    const float2 rs = fma_df(make_float2(-al.x, -al.y), a.q2[row], a.r2[row]);
    a.r2[row] = rs;
    acc_sq_df(zh, zl, rs, a.dinvf[row]);
    acc_sq_df(rh, rl, rs, 1.0f);
  }
  const double v[2] = {join_df(make_float2(zh, zl)), join_df(make_float2(rh, rl))};
  double tot[2];
  if (problem_reduce<2>(a, t, pr, v, tot, sh) && threadIdx.x == 0) {
    const bool learned = a.mode[pr] != 0;  // flexible CG: beta comes from k_bt_prec
    const double be = learned ? 0.0 : tot[0] / a.rz[pr];
    if (!learned) a.beta[pr] = be;
    a.rz[pr] = tot[0];  // kept in flexible CG too: a problem may change to Jacobi-CG in place
    a.rr[pr] = tot[1];
    a.iters[pr] += 1;
    a.kiter[pr] += 1;
    if (learned) a.liters[pr] += 1;
    if (!isfinite(tot[1]) || !isfinite(be)) a.done[pr] = 2;
    else if (tot[1] <= a.stop2[pr]) a.done[pr] = 1;
  }
}

// x = 0 (or kept) except identity rows (x = b there)
__global__ void k_batch_prep(int64_t n, const uint8_t* __restrict__ idmask, const double* __restrict__ b,
                             double* __restrict__ x, int zero) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xi = zero ? 0.0 : x[i];
  if (idmask[i]) xi = b[i];
  x[i] = xi;
}

// x += this round's FP32-pair increment; the increment restarts from 0
__global__ void k_batch_fold(int64_t n, float2* __restrict__ x2, double* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] += join_df(x2[i]);
  x2[i] = make_float2(0.0f, 0.0f);
}

// r = b - A x (FP64 CRS), p = 0; per-tile r.D^-1 r, r.r, b.b
__global__ void __launch_bounds__(kBT) k_batch_resid(TileArgs a, const int64_t* __restrict__ rp,
                                                     const int32_t* __restrict__ ci, const double* __restrict__ v,
                                                     const double* __restrict__ b, double* __restrict__ tb) {
  __shared__ double sh[33];
  const int t = blockIdx.x;
  double rz = 0.0, rr = 0.0, bb = 0.0;
  for (int i = threadIdx.x; i < a.tile_rows[t]; i += kBT) {
    const int64_t row = a.tile_row0[t] + i;
    double s = 0.0;
    for (int64_t j = rp[row]; j < rp[row + 1]; ++j) s += v[j] * a.x[ci[j]];
    const double ri = b[row] - s;
    a.r[row] = ri;
    a.r2[row] = split_df(ri);
    a.x2[row] = make_float2(0.0f, 0.0f);
    a.p[row] = make_float2(0.0f, 0.0f);
    a.q2[row] = make_float2(0.0f, 0.0f);
    rz += ri * (widen_f(a.dinvf[row]) * ri);
    rr += ri * ri;
    bb += b[row] * b[row];
  }
  const double t1 = red::block_sum(rz, sh), t2 = red::block_sum(rr, sh), t3 = red::block_sum(bb, sh);
  if (threadIdx.x == 0) {
    a.tpart[t] = t1;
    a.tpart[a.ntiles + t] = t2;
    tb[t] = t3;
  }
}

// per-problem sums of three tile arrays: out[3][P]
__global__ void k_batch_sums(const double* __restrict__ t0p, const double* __restrict__ t1p,
                             const double* __restrict__ t2p, const int32_t* __restrict__ ptile0,
                             const int32_t* __restrict__ ptile1, int P, double* __restrict__ out) {
  __shared__ double sh[33];
  for (int pr = blockIdx.x; pr < P; pr += gridDim.x) {
    const double* src[3] = {t0p, t1p, t2p};
    for (int k = 0; k < 3; ++k) {
      double s = 0.0;
      for (int t = ptile0[pr] + threadIdx.x; t < ptile1[pr]; t += blockDim.x) s += src[k][t];
      const double tot = red::block_sum(s, sh);
      if (threadIdx.x == 0) out[k * P + pr] = tot;
    }
  }
}

__global__ void k_to_float(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

}  // namespace

int solve_batched(nalu_ctx* ctx, const nalu_solver_opts& o, nalu_solve_info* infos) {
  const auto t0 = std::chrono::steady_clock::now();
  const int P = (int)ctx->problem_offsets.size() - 1;
  if (P < 1) return set_error(ctx, NALU_ERR_STATE, "no problem partition (nalu_set_problems)");
  const int64_t n = ctx->n_rows;
  const int nd = ctx->num_dof;
  // tiles of <= tile_rows rows inside each problem
  const int tile_rows = ctx->batch_tile_rows > 0 ? ctx->batch_tile_rows : kTileRows;
  std::vector<int64_t> trow0;
  std::vector<int32_t> trows, tprob, pt0(P), pt1(P);
  for (int pr = 0; pr < P; ++pr) {
    const int64_t rb = ctx->problem_offsets[pr] * nd, re = ctx->problem_offsets[pr + 1] * nd;
    pt0[pr] = (int32_t)trow0.size();
    for (int64_t r = rb; r < re; r += tile_rows) {
      trow0.push_back(r);
      trows.push_back((int32_t)std::min<int64_t>(tile_rows, re - r));
      tprob.push_back(pr);
    }
    pt1[pr] = (int32_t)trow0.size();
  }
  const int ntiles = (int)trow0.size();
  SolverWork& s = ctx->sw;
  int rc = compute_dinv(ctx);
  if (rc) return rc;
  const float2* sv2 = nullptr;
  if ((rc = sell_build<float2>(ctx, s.sell, &sv2))) return rc;
  DBuf<int64_t> d_trow0;
  const bool learned = o.precond == NALU_PRECOND_LEARNED;
  const bool multilevel = o.precond == NALU_PRECOND_MULTILEVEL;
  const bool flexible = learned || multilevel;
  if (flexible && (o.method != NALU_SOLVER_CG || o.precision != NALU_PRECISION_FP64))
    return set_error(ctx, NALU_ERR_ARG, "the learned and multigrid preconditioners run in FP64 flexible CG only");
  if (!(o.precond == NALU_PRECOND_JACOBI || flexible))
    return set_error(ctx, NALU_ERR_ARG, "batched solve: Jacobi, learned or multigrid preconditioner");
  double setup_s = 0.0;
  if (learned) {
    LearnedState& L = ctx->learned;
    if (!L.has_weights) return set_error(ctx, NALU_ERR_STATE, "learned preconditioner has no weights");
    if (L.wsell.n < s.sell.stored) NALU_CUDA(ctx, L.wsell.alloc(s.sell.stored));
  }
  DBuf<float> rfb, zfb;
  if (multilevel) {
    // one hierarchy for the union: aggregation follows couplings, so no
    // aggregate spans two problems, every coarse operator is block diagonal and
    // the V-cycle applies each problem's own preconditioner; each problem
    // coarsens down to the coarsest size on its own and keeps a dense block
    // of its own there
    if (nd != 1) return set_error(ctx, NALU_ERR_ARG, "the multigrid preconditioner needs a scalar system");
    const auto ts = std::chrono::steady_clock::now();
    std::vector<int64_t> roff(P + 1);
    for (int pr = 0; pr <= P; ++pr) roff[pr] = ctx->problem_offsets[pr] * nd;
    if ((rc = sell_c16_ensure(ctx, s.sell)) || (rc = ml_setup(ctx, false, &roff))) return rc;
    NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count();
    NALU_CUDA(ctx, rfb.alloc(n));
    NALU_CUDA(ctx, zfb.alloc(n));
    NALU_CUDA(ctx, cudaMemsetAsync(rfb.p, 0, sizeof(float) * n, ctx->stream));
  }
  DBuf<int32_t> d_ints;  // trows | tprob | pt0 | pt1 | done | iters | mode | kiter | liters
  DBuf<double> d_dbl;    // tpart[2 ntiles] | tb[ntiles] | alpha beta rz rr stop2 [P] | sums [3P]
  DBuf<unsigned> d_cnt;
  DBuf<float> dinvf;
  DBuf<float2> p2;
  NALU_CUDA(ctx, d_trow0.alloc(ntiles));
  NALU_CUDA(ctx, d_ints.alloc(2 * (int64_t)ntiles + 7 * (int64_t)P));
  NALU_CUDA(ctx, d_dbl.alloc(3 * (int64_t)ntiles + 9 * (int64_t)P));
  DBuf<double> zbuf;
  if (flexible) NALU_CUDA(ctx, zbuf.alloc(n));
  NALU_CUDA(ctx, d_cnt.alloc(P));
  NALU_CUDA(ctx, dinvf.alloc(n));
  NALU_CUDA(ctx, p2.alloc(n));
  for (auto* b : {&s.r, &s.q})
    if (b->n < n) NALU_CUDA(ctx, b->alloc(n));
  int32_t* trows_d = d_ints.p;
  int32_t* tprob_d = trows_d + ntiles;
  int32_t* pt0_d = tprob_d + ntiles;
  int32_t* pt1_d = pt0_d + P;
  int32_t* done_d = pt1_d + P;
  int32_t* iters_d = done_d + P;
  int32_t* mode_d = iters_d + P;
  int32_t* kiter_d = mode_d + P;
  int32_t* liters_d = kiter_d + P;
  double* tpart = d_dbl.p;
  double* tb = tpart + 2 * (int64_t)ntiles;
  double* alpha_d = tb + ntiles;
  double* beta_d = alpha_d + P;
  double* rz_d = beta_d + P;
  double* rr_d = rz_d + P;
  double* stop2_d = rr_d + P;
  double* sums_d = stop2_d + P;  // [3][P]
  double* pq_d = sums_d + 3 * P;
  cudaStream_t st = ctx->stream;
  NALU_CUDA(ctx, cudaMemcpyAsync(d_trow0.p, trow0.data(), sizeof(int64_t) * ntiles, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemcpyAsync(trows_d, trows.data(), sizeof(int32_t) * ntiles, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemcpyAsync(tprob_d, tprob.data(), sizeof(int32_t) * ntiles, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemcpyAsync(pt0_d, pt0.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemcpyAsync(pt1_d, pt1.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
  NALU_CUDA(ctx, cudaMemsetAsync(iters_d, 0, sizeof(int32_t) * P, st));
  NALU_CUDA(ctx, cudaMemsetAsync(liters_d, 0, sizeof(int32_t) * P, st));
  std::vector<int32_t> mode(P, multilevel ? 2 : 0), fallback(P, learned ? 2 : 0);
  NALU_CUDA(ctx, cudaMemsetAsync(d_cnt.p, 0, sizeof(unsigned) * P, st));
  k_to_float<<<1024, 256, 0, st>>>(n, s.dinv.p, dinvf.p);
  k_batch_prep<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, ctx->d_bcmask.p, ctx->d_rhs.p, ctx->d_x.p,
                                                           o.x0_zero ? 1 : 0);
  ctx->launches += 2;

  TileArgs a{};
  a.n = n;
  a.P = P;
  a.ntiles = ntiles;
  a.tile_row0 = d_trow0.p;
  a.tile_rows = trows_d;
  a.tile_prob = tprob_d;
  a.ptile0 = pt0_d;
  a.ptile1 = pt1_d;
  a.sptr = s.sell.ptr.p;
  a.slen = s.sell.len.p;
  a.scol = s.sell.col.p;
  if ((rc = sell_c16_ensure(ctx, s.sell))) return rc;
  a.col16 = s.sell.col16.p;
  a.cbase = s.sell.cbase.p;
  a.wide = s.sell.wide.p;
  a.sval = s.sell.val2.p;
  a.dinvf = dinvf.p;
  a.x = ctx->d_x.p;
  a.r = s.r.p;
  if (s.x2.n < n) NALU_CUDA(ctx, s.x2.alloc(n));
  if (s.r2.n < n) NALU_CUDA(ctx, s.r2.alloc(n));
  if (s.q2.n < n) NALU_CUDA(ctx, s.q2.alloc(n));
  a.x2 = s.x2.p;
  a.r2 = s.r2.p;
  a.q2 = s.q2.p;
  a.p = p2.p;
  a.tpart = tpart;
  a.pcnt = d_cnt.p;
  a.alpha = alpha_d;
  a.beta = beta_d;
  a.rz = rz_d;
  a.rr = rr_d;
  a.stop2 = stop2_d;
  a.done = done_d;
  a.iters = iters_d;
  a.wsell = learned ? ctx->learned.wsell.p : nullptr;  // rows set up problem by problem
  a.z = zbuf.p;
  a.rf = rfb.p;
  a.zf = zfb.p;
  a.mode = mode_d;
  a.pq = pq_d;
  a.kiter = kiter_d;
  a.liters = liters_d;

  const int chunk = o.check_every > 0 ? o.check_every : 25;
  // two graphs of `chunk` iterations: Jacobi-CG only (three kernels an
  // iteration) and flexible CG (the learned stencil apply, or the union
  // V-cycle, first); the second runs only while some unfinished problem is
  // in flexible CG
  GraphExecs gx;
  auto capture = [&](bool with_prec, cudaGraphExec_t* out) -> int {
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (ce != cudaSuccess) return cuda_check(ctx, ce, "begin capture");
    for (int k = 0; k < chunk; ++k) {
      if (with_prec && multilevel) {
        k_bt_hi<<<ntiles, kBT, 0, st>>>(a);
        ml_apply(ctx, a.rf, zfb.p);
      }
      if (with_prec) k_bt_prec<<<ntiles, kBT, 0, st>>>(a);
      k_bt_pupdate<<<ntiles, kBT, 0, st>>>(a);
      k_bt_spmv<<<ntiles, kBT, 0, st>>>(a);
      k_bt_axpy<<<ntiles, kBT, 0, st>>>(a);
    }
    ce = cudaStreamEndCapture(st, &graph);
    if (ce != cudaSuccess) return cuda_check(ctx, ce, "end capture");
    ce = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    return ce == cudaSuccess ? NALU_OK : cuda_check(ctx, ce, "instantiate");
  };
  if ((rc = capture(false, &gx.e[0]))) return rc;
  if (flexible && (rc = capture(true, &gx.e[1]))) return rc;

  std::vector<double> sums(3 * P);
  std::vector<int32_t> done(P), iters(P);
  std::vector<double> true_res(P, 0.0), r0(P, 0.0);
  const int window = o.stall_window > 0 ? o.stall_window : 20;
  // one round: true residual r = b - A x (FP64), Jacobi r.z and ||b|| per
  // problem, then the per-problem start of CG (or flexible CG, per mode);
  // returns 1 when every problem already meets the tolerance
  auto start_round = [&]() -> int {
    k_batch_resid<<<ntiles, kBT, 0, st>>>(a, ctx->d_rowptr.p, ctx->d_colind.p, ctx->d_values.p, ctx->d_rhs.p, tb);
    k_batch_sums<<<std::min(P, 1024), kBT, 0, st>>>(tpart, tpart + ntiles, tb, pt0_d, pt1_d, P, sums_d);
    ctx->launches += 2;
    NALU_CUDA(ctx, cudaMemcpyAsync(sums.data(), sums_d, sizeof(double) * 3 * P, cudaMemcpyDeviceToHost, st));
    NALU_CUDA(ctx, cudaStreamSynchronize(st));
    bool all = true;
    std::vector<double> stop2(P), rz0(P);
    for (int pr = 0; pr < P; ++pr) {
      const double bnorm = std::sqrt(sums[2 * P + pr]);
      const double bref = bnorm > 0 ? bnorm : 1.0;
      r0[pr] = std::sqrt(sums[P + pr]);
      true_res[pr] = r0[pr] / bref;
      done[pr] = true_res[pr] <= o.tol ? 1 : 0;
      all = all && done[pr];
      stop2[pr] = std::pow(0.5 * o.tol * bref, 2);
      rz0[pr] = sums[pr];
    }
    if (all) return 1;
    NALU_CUDA(ctx, cudaMemcpyAsync(stop2_d, stop2.data(), sizeof(double) * P, cudaMemcpyHostToDevice, st));
    NALU_CUDA(ctx, cudaMemcpyAsync(rz_d, rz0.data(), sizeof(double) * P, cudaMemcpyHostToDevice, st));
    NALU_CUDA(ctx, cudaMemcpyAsync(done_d, done.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
    NALU_CUDA(ctx, cudaMemsetAsync(beta_d, 0, sizeof(double) * P, st));
    NALU_CUDA(ctx, cudaMemsetAsync(kiter_d, 0, sizeof(int32_t) * P, st));
    NALU_CUDA(ctx, cudaMemcpyAsync(mode_d, mode.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
    return 0;
  };

  // ---- the learned preconditioner, problem by problem --------------------
  // A problem changes method in place between chunks (no restart of the
  // others, no iteration discarded): to learned FCG with kiter = 0 (its next
  // step is p = M r), to Jacobi-CG with beta = 0 (p = D^-1 r; r.D^-1 r is kept
  // by every iteration).  With the probe on, the round opens with `probe`
  // iterations of Jacobi-CG for all problems; their rates predict each
  // problem's remaining Jacobi-CG iterations.  Only problems with at least
  // kLearnedMinRemaining x probe of them left are candidates (the learned
  // set-up and probe cannot pay off on the rest), and the candidate with the
  // most remaining row-iterations alone is set up and run `probe` iterations
  // in learned mode while the others continue Jacobi-CG.  From the two phases'
  // device times, the cost of a learned row-iteration over a Jacobi one
  // (kappa) follows; the learned FCG wins when its residual reduction per
  // unit of time beats the problem's own Jacobi-CG rate.  If it loses, the
  // problem changes back and no other problem is set up.  If it wins, every
  // other candidate is set up and changes; each is judged the same way after
  // its own `probe` learned iterations.  A learned problem also changes back
  // when its residual stalls (no new minimum for max(window, 10 x the
  // iterations taken to reach it)), when its learned iterations pass twice the
  // predicted Jacobi-CG count, or when its step breaks down.
  constexpr int kLearnedMinRemaining = 4;
  const int probe = chunk * std::max(1, (std::max(40, 2 * window) + chunk - 1) / chunk);
  std::vector<int64_t> prow0(P), prow1(P);
  for (int pr = 0; pr < P; ++pr) {
    prow0[pr] = ctx->problem_offsets[pr] * nd;
    prow1[pr] = ctx->problem_offsets[pr + 1] * nd;
  }
  std::vector<double> rrh(P), lres0(P, 0.0), best(P, INFINITY), rate_j(P, 0.0), rate_l(P, 0.0), remain_j(P, 0.0);
  std::vector<int> lit(P, 0), best_it(P, 0), pace(P, 0);
  std::vector<char> prepared(P, 0), judged(P, 0), candidate(P, 0);
  double kappa = 1.0, u_j = 0.0;  // learned / Jacobi cost per row-iteration; ms per Jacobi row-iteration
  auto set_mode = [&](int pr, int m) -> int {
    mode[pr] = m;
    const int32_t zi = 0;
    const double zd = 0.0;
    NALU_CUDA(ctx, cudaMemcpyAsync(mode_d + pr, &mode[pr], sizeof(int32_t), cudaMemcpyHostToDevice, st));
    NALU_CUDA(ctx, cudaMemcpyAsync(kiter_d + pr, &zi, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    NALU_CUDA(ctx, cudaMemcpyAsync(beta_d + pr, &zd, sizeof(double), cudaMemcpyHostToDevice, st));
    if (done[pr] == 3) {
      done[pr] = 0;
      NALU_CUDA(ctx, cudaMemcpyAsync(done_d + pr, &done[pr], sizeof(int32_t), cudaMemcpyHostToDevice, st));
    }
    return NALU_OK;
  };
  auto to_learned = [&](int pr) -> int {
    if (!prepared[pr]) {
      const auto ts = std::chrono::steady_clock::now();
      int r = learned_prepare_rows(ctx, prow0[pr], prow1[pr]);
      if (r) return r;
      NALU_CUDA(ctx, cudaStreamSynchronize(st));
      setup_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count();
      prepared[pr] = 1;
    }
    lit[pr] = 0;
    lres0[pr] = std::sqrt(std::max(rrh[pr], 0.0));
    best[pr] = lres0[pr];
    best_it[pr] = 0;
    fallback[pr] = 0;
    return set_mode(pr, 1);
  };
  auto to_jacobi = [&](int pr, int why) -> int {
    fallback[pr] = why;
    return set_mode(pr, 0);
  };
  // learned rate (ln residual reduction per iteration) since the change
  auto learned_rate = [&](int pr) {
    return std::log(std::max(std::sqrt(std::max(rrh[pr], 0.0)), 1e-300) / std::max(lres0[pr], 1e-300)) /
           std::max(lit[pr], 1);
  };
  auto learned_wins = [&](int pr) { return done[pr] != 3 && rate_l[pr] < kappa * rate_j[pr]; };
  auto rows_active = [&](int m) {  // m < 0: every mode; m = 3: flexible CG (modes 1 and 2)
    int64_t s0 = 0;
    for (int pr = 0; pr < P; ++pr)
      if (!done[pr] && (m < 0 || mode[pr] == m || (m == 3 && mode[pr] != 0))) s0 += prow1[pr] - prow0[pr];
    return s0;
  };
  cudaEvent_t pe[2];
  for (auto& e : pe) NALU_CUDA(ctx, cudaEventCreate(&e));
  struct EvFree {
    cudaEvent_t* e;
    ~EvFree() { cudaEventDestroy(e[0]); cudaEventDestroy(e[1]); }
  } evfree{pe};
  enum Phase { kJacobiProbe, kLearnedProbe, kDecided };
  Phase phase = (learned && o.learned_probe) ? kJacobiProbe : kDecided;
  int rep = -1;
  double rows_a = 0.0, rows_bj = 0.0, rows_bl = 0.0;  // row-iterations of the two timed phases

  // device time of the first round's chunks (the tile-size autotuner's measure)
  cudaEvent_t rt[2];
  for (auto& e : rt) NALU_CUDA(ctx, cudaEventCreate(&e));
  struct EvFree2 {
    cudaEvent_t* e;
    ~EvFree2() { cudaEventDestroy(e[0]); cudaEventDestroy(e[1]); }
  } rtfree{rt};
  ctx->batch_round_ms = 0.0;
  ctx->batch_round_its = 0;
  bool first_round = true;
  int its_used = 0;  // iterations launched over all rounds (max_iters bounds the total)
  // one round of at most max_its iterations; x is updated in place
  auto run_round = [&](int max_its) -> int {
    int phase_it = 0, round_its = 0;
    if (first_round) NALU_CUDA(ctx, cudaEventRecord(rt[0], st));
    if (phase != kDecided) NALU_CUDA(ctx, cudaEventRecord(pe[0], st));
    for (int it = 0; it < max_its; it += chunk) {
      const bool any_learned = flexible && rows_active(3) > 0;
      if (phase == kJacobiProbe) rows_a += (double)rows_active(-1) * chunk;
      if (phase == kLearnedProbe) {
        rows_bj += (double)rows_active(0) * chunk;
        rows_bl += (double)rows_active(1) * chunk;
      }
      cudaGraphLaunch(gx.e[any_learned ? 1 : 0], st);
      ctx->launches += (any_learned ? 4 : 3) * chunk;
      round_its += chunk;
      its_used += chunk;
      if (first_round) NALU_CUDA(ctx, cudaEventRecord(rt[1], st));
      NALU_CUDA(ctx, cudaMemcpyAsync(done.data(), done_d, sizeof(int32_t) * P, cudaMemcpyDeviceToHost, st));
      NALU_CUDA(ctx, cudaMemcpyAsync(rrh.data(), rr_d, sizeof(double) * P, cudaMemcpyDeviceToHost, st));
      if (phase != kDecided) NALU_CUDA(ctx, cudaEventRecord(pe[1], st));
      NALU_CUDA(ctx, cudaStreamSynchronize(st));
      phase_it += chunk;
      for (int pr = 0; pr < P; ++pr)
        if (mode[pr] == 1 && (done[pr] == 0 || done[pr] == 3)) lit[pr] += chunk;
      const bool all_done = std::all_of(done.begin(), done.end(), [](int d) { return d == 1 || d == 2; });
      if (phase == kJacobiProbe && (phase_it >= probe || all_done)) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, pe[0], pe[1]);
        u_j = rows_a > 0 ? ms / rows_a : 0.0;
        double best_work = -1.0;
        for (int pr = 0; pr < P; ++pr) {
          if (done[pr]) continue;
          const double res = std::sqrt(std::max(rrh[pr], 0.0));
          const double stop = 0.5 * o.tol * std::sqrt(std::max(sums[2 * P + pr], 0.0));
          rate_j[pr] = std::log(std::max(res, 1e-300) / std::max(r0[pr], 1e-300)) / phase_it;
          remain_j[pr] = rate_j[pr] < 0.0 ? std::log(std::max(stop, 1e-300) / std::max(res, 1e-300)) / rate_j[pr]
                                          : INFINITY;
          if (remain_j[pr] < (double)kLearnedMinRemaining * probe) continue;
          candidate[pr] = 1;
          pace[pr] = (int)std::min(2.0 * remain_j[pr], 2.0e9);
          const double work = std::min(remain_j[pr], 1e12) * (double)(prow1[pr] - prow0[pr]);
          if (work > best_work) {
            best_work = work;
            rep = pr;
          }
        }
        phase = kDecided;
        if (rep >= 0) {
          if ((rc = to_learned(rep))) return rc;
          phase = kLearnedProbe;
          phase_it = 0;
          NALU_CUDA(ctx, cudaEventRecord(pe[0], st));
        }
      } else if (phase == kLearnedProbe && (phase_it >= probe || done[rep] != 0 || all_done)) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, pe[0], pe[1]);
        if (rows_bl > 0 && u_j > 0)
          kappa = std::min(10.0, std::max(1.0, 1.0 + (ms - u_j * (rows_bj + rows_bl)) / (u_j * rows_bl)));
        rate_l[rep] = learned_rate(rep);
        judged[rep] = 1;
        phase = kDecided;
        if (!learned_wins(rep)) {
          if (done[rep] == 0 || done[rep] == 3) {
            if ((rc = to_jacobi(rep, 2))) return rc;
          } else {
            fallback[rep] = 2;
          }
        } else {
          for (int pr = 0; pr < P; ++pr)
            if (candidate[pr] && pr != rep && !done[pr] && (rc = to_learned(pr))) return rc;
        }
      } else if (phase == kDecided && multilevel) {
        for (int pr = 0; pr < P; ++pr)
          if (mode[pr] == 2 && done[pr] == 3 && (rc = to_jacobi(pr, 1))) return rc;  // not positive: Jacobi-CG
      } else if (phase == kDecided && learned) {
        for (int pr = 0; pr < P; ++pr) {
          if (mode[pr] != 1 || done[pr] == 1 || done[pr] == 2) continue;
          if (done[pr] == 3) {  // the learned step was not positive: Jacobi-CG from here
            if ((rc = to_jacobi(pr, 1))) return rc;
            continue;
          }
          const double res = std::sqrt(std::max(rrh[pr], 0.0));
          if (o.learned_probe && !judged[pr] && lit[pr] >= probe) {
            rate_l[pr] = learned_rate(pr);
            judged[pr] = 1;
            if (!learned_wins(pr)) {
              if ((rc = to_jacobi(pr, 2))) return rc;
              continue;
            }
          }
          const bool behind = pace[pr] > 0 && lit[pr] > pace[pr];  // behind Jacobi-CG's pace
          bool stalled = false;
          if (res < 0.999 * best[pr]) {
            best[pr] = res;
            best_it[pr] = lit[pr];
          } else if (lit[pr] - best_it[pr] > std::max(window, 10 * best_it[pr])) {
            stalled = true;
          }
          if ((behind || stalled) && (rc = to_jacobi(pr, behind ? 2 : 1))) return rc;
        }
      }
      if (all_done) break;
    }
    if (first_round && round_its > 0) {
      float ms = 0.f;
      NALU_CUDA(ctx, cudaEventSynchronize(rt[1]));
      cudaEventElapsedTime(&ms, rt[0], rt[1]);
      ctx->batch_round_ms = ms;
      ctx->batch_round_its = round_its;
    }
    first_round = false;
    // the round's increment into the FP64 solution
    k_batch_fold<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, a.x2, a.x);
    ctx->launches++;
    return cuda_check(ctx, cudaGetLastError(), "batch fold");
  };

  if (learned && !o.learned_probe) {  // every problem in learned mode from the start
    if ((rc = learned_prepare_rows(ctx, 0, n))) return rc;
    std::fill(prepared.begin(), prepared.end(), 1);
    std::fill(mode.begin(), mode.end(), 1);
    std::fill(fallback.begin(), fallback.end(), 0);
  }
  for (int outer = 0; outer < 6; ++outer) {
    if (start_round()) break;
    if (its_used >= o.max_iters) break;  // the budget is spent: the true residual above is the result
    if (outer == 0 && learned && !o.learned_probe)
      for (int pr = 0; pr < P; ++pr) lres0[pr] = best[pr] = r0[pr];
    int rcr = run_round(o.max_iters - its_used);
    if (rcr) return rcr;
    if (std::any_of(done.begin(), done.end(), [](int d) { return d == 2; })) break;
  }
  std::vector<int32_t> liters(P, 0);
  NALU_CUDA(ctx, cudaMemcpyAsync(liters.data(), liters_d, sizeof(int32_t) * P, cudaMemcpyDeviceToHost, st));
  NALU_CUDA(ctx, cudaMemcpyAsync(iters.data(), iters_d, sizeof(int32_t) * P, cudaMemcpyDeviceToHost, st));
  NALU_CUDA(ctx, cudaStreamSynchronize(st));
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  bool all_ok = true;
  for (int pr = 0; pr < P; ++pr) {
    infos[pr] = nalu_solve_info{};
    infos[pr].iterations = iters[pr];
    infos[pr].outer_iterations = 1;
    infos[pr].true_rel_res = true_res[pr];
    infos[pr].seconds = secs;
    infos[pr].fallback = fallback[pr];
    infos[pr].learned_iterations = liters[pr];
    infos[pr].setup_seconds = setup_s;
    // probe rates as ln(residual reduction) per ms of this problem's iterations
    const double ms_it = u_j * (double)(prow1[pr] - prow0[pr]);
    if (ms_it > 0.0 && rate_j[pr] != 0.0) infos[pr].probe_rate_jacobi = rate_j[pr] / ms_it;
    if (ms_it > 0.0 && judged[pr]) infos[pr].probe_rate_learned = rate_l[pr] / (kappa * ms_it);
    infos[pr].status = true_res[pr] <= o.tol ? NALU_OK : (done[pr] == 2 ? NALU_ERR_NONFINITE : NALU_ERR_NOT_CONVERGED);
    all_ok = all_ok && infos[pr].status == NALU_OK;
  }
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

int nalu_batch_autotune(nalu_ctx* ctx, int iterations, int* tile_rows, double* ms_per_iteration) {
  using namespace nalu_gb300;
  if (!ctx) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  const int P = (int)ctx->problem_offsets.size() - 1;
  if (P < 1) return set_error(ctx, NALU_ERR_STATE, "no problem partition (nalu_set_problems)");
  cudaSetDevice(ctx->device);
  // each candidate runs `iterations` of the batched Jacobi-CG from zero (at
  // full load while no problem has converged) and is timed on the device
  nalu_solver_opts o;
  nalu_solver_opts_default(&o);
  o.max_iters = iterations > 0 ? iterations : 100;
  o.tol = 1e-300;
  std::vector<nalu_solve_info> infos(P);
  int best = -1;
  double best_ms = 0.0;
  for (int k = 0; k < 4; ++k) {
    ctx->batch_tile_rows = kTileCandidates[k];
    const int rc = solve_batched(ctx, o, infos.data());
    if (rc != NALU_OK && rc != NALU_ERR_NOT_CONVERGED) {
      ctx->batch_tile_rows = 0;
      return rc;
    }
    const double ms = ctx->batch_round_its > 0 ? ctx->batch_round_ms / ctx->batch_round_its : -1.0;
    ctx->batch_tune_ms[k] = ms;
    if (ms > 0.0 && (best < 0 || ms < best_ms)) best = k, best_ms = ms;
  }
  ctx->batch_tile_rows = best >= 0 ? kTileCandidates[best] : 0;
  ctx->last_error.clear();
  if (tile_rows) *tile_rows = ctx->batch_tile_rows > 0 ? ctx->batch_tile_rows : kTileRows;
  if (ms_per_iteration)
    for (int k = 0; k < 4; ++k) ms_per_iteration[k] = ctx->batch_tune_ms[k];
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
