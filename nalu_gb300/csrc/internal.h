// internal.h -- context layout and helpers shared by the library's
// translation units (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <string>
#include <utility>
#include <vector>

#include "../../include/nalu_gb300.h"

namespace nalu_gb300 {

// Device buffer (freed by its destructor; movable, not copyable).
template <class T>
struct DBuf {
  T* p = nullptr;
  int64_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      free();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DBuf() { free(); }
  cudaError_t alloc(int64_t count) {
    free();
    if (count <= 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)&p, sizeof(T) * (size_t)count);
    if (e == cudaSuccess) n = count;
    else p = nullptr;
    return e;
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// Field storage: node fields in Tpetra row order (LID), element fields in
// element order.
struct Field {
  DBuf<double> d;
  int comps = 0;
  bool set = false;
  // nalu_field_set_async: the next contents, uploaded on the upload stream,
  // swapped into d by the next call that reads fields (stream order)
  DBuf<double> back, stage;
  bool pending = false;
  void swap_back() {
    std::swap(d.p, back.p);
    std::swap(d.n, back.n);
  }
};

// SELL-32 copy of the CRS matrix for the fast CG (cg_fast.cu)
struct SellMatrix {
  DBuf<int64_t> ptr;   // [nslices+1] start of each slice
  DBuf<int32_t> len;   // [nslices] entries per row in the slice
  DBuf<int32_t> col;
  DBuf<double> vald;
  DBuf<float> valf;
  DBuf<float2> val2;   // FP32 pairs (hi, lo) for the df64 SpMV
  int64_t nslices = 0, stored = 0;
  // compressed column indices: col = cbase[ptr[s] / 32 + k] + col16[entry] for
  // the k-th entry of slice s, unless wide[s] (then col holds them)
  DBuf<uint16_t> col16;
  DBuf<int32_t> cbase;
  DBuf<uint8_t> wide;
  bool c16_valid = false;
  // device pointers of the pattern, passed to kernels by value
  struct View {
    const int64_t* ptr;
    const int32_t* len;
    const int32_t* col;
    const uint16_t* col16;
    const int32_t* cbase;
    const uint8_t* wide;
  };
  View view() const { return View{ptr.p, len.p, col.p, col16.p, cbase.p, wide.p}; }
};

// Learned preconditioner state (learned.cu).  The MLP parameters are FP32
// master copies; the stencil and its SELL values are rebuilt per solve.
struct LearnedState {
  DBuf<float> params, adam_m, adam_v, grad;  // [kLearnedParams]
  DBuf<uint16_t> wbf;                         // BF16 W2/W3 in the padded kernel layout
  DBuf<int32_t> nbr;                          // [n][27] neighbour LID per topological slot, -1 if none
  DBuf<float> stencil;                        // [n][27] MLP output per slot
  DBuf<float> wsell;                          // preconditioner values on the SELL pattern of A
  DBuf<float> srow;                           // [n] row factors of the SPD safeguard (set-up scratch)
  DBuf<uint16_t> wsell16;                     // the same as BF16 (wide slices of the stencil apply)
  DBuf<uint32_t> wpack;                       // BF16 value << 16 | 16-bit column offset, per SELL entry
  int64_t nbr_nodes = 0;                      // mesh size the slot map was built for
  bool has_weights = false;
};

// Solver workspace (device vectors are allocated lazily per system size).
struct SolverWork {
  SellMatrix sell;
  DBuf<double> r, z, p, q, ap, dinv, w, tmp;
  DBuf<float> fvals, fr, fz, fp, fq, fdinv, fx;
  DBuf<double> V, Hbuf;  // GMRES basis (restart+1 vectors)
  DBuf<float> fV;
  DBuf<double> scal;     // device scalars
  DBuf<double> partial;  // block partial sums
  DBuf<float2> p2;       // search direction as FP32 pairs (df64 SpMV)
  DBuf<float2> x2, r2, q2;  // Jacobi-CG iterate, residual and A p as FP32 pairs
  DBuf<float> zf;           // learned-FCG preconditioned residual (FP32 stencil output)
  DBuf<double> cscal;    // CG scalars written by the last block of each kernel
  DBuf<unsigned> ccount; // arrival counter of the single-block reductions
  // FP32 3x3-block copy of a 3-dof matrix (node rows, node columns, nine
  // value planes of b3_nblk floats), rebuilt by each mixed-precision solve
  DBuf<int64_t> b3rp;
  DBuf<int32_t> b3col;
  DBuf<float> b3val;
  DBuf<int> b3flag;
  int64_t b3_nblk = 0;
  int64_t n = 0;
};

// one side set: face k is side side[k] (0..5) of element elem[k]
struct FaceSet {
  DBuf<int32_t> elem;
  DBuf<uint8_t> side;
  DBuf<double> dynp;                  // [n][4] dynamic_pressure at the face ips, or empty (0)
  std::vector<int32_t> h_elem;
  std::vector<uint8_t> h_side;
  int64_t n = 0;
  bool defined = false;
  void clear();
};

}  // namespace nalu_gb300

namespace nalu_gb300 {
struct MlState;  // multilevel preconditioner hierarchy (multilevel.cu)
}

struct nalu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  int64_t launches = 0;
  int sm_count = 0;

  // mesh
  int64_t n_nodes = 0, n_elems = 0;
  bool identity_order = true;            // gid == index+1 for all nodes
  std::vector<int32_t> h_lid;            // caller node index -> LID
  std::vector<int64_t> h_gid;            // LID -> node global id
  int write_counter = 0;                 // TpetraLinearSystem::writeCounter_
  std::vector<int32_t> h_conn_lid;       // [E][8] in LID space (host copy)
  nalu_gb300::DBuf<int32_t> d_conn;      // [E][8] LIDs
  nalu_gb300::DBuf<int32_t> d_lid;       // caller index -> LID (device)
  nalu_gb300::Field fields[NALU_FIELD_COUNT];

  // linear system
  int num_dof = 0;
  int64_t n_rows = 0, nnz = 0, node_nnz = 0;
  nalu_gb300::DBuf<int64_t> d_nrowptr;   // node-level graph
  nalu_gb300::DBuf<int32_t> d_ncolind;
  nalu_gb300::DBuf<int64_t> d_rowptr;    // dof-level CRS (Tpetra layout)
  nalu_gb300::DBuf<int32_t> d_colind;
  nalu_gb300::DBuf<double> d_values, d_rhs, d_x;
  nalu_gb300::DBuf<uint8_t> d_slots;     // [E][64] column offset in the node row
  nalu_gb300::DBuf<uint8_t> d_bcmask;    // 1 where the row was made an identity row
  nalu_gb300::DBuf<int32_t> d_colour_elems;  // element ids grouped by colour
  nalu_gb300::DBuf<double> d_node_df;    // df64 split of nodal kernel inputs (8 B each)
  std::vector<int64_t> colour_offsets;   // [n_colours+1]
  int scatter_choice[6][2] = {};  // autotuned scatter per kernel and arithmetic (FP64, df64; 0 = not tuned)
  // autotuned schedule x scatter of the double-float scalar kernels, per kernel,
  // with the device time of every candidate [schedule - 1][scatter - 1]
  int df_schedule[2] = {0, 0}, df_scatter[2] = {0, 0};
  double df_tune_ms[2][3][2] = {};

  // independent problems in one context (node offsets in LID order)
  std::vector<int64_t> problem_offsets;
  // batched solve: rows per tile (0: the default 1024; set by the autotuner),
  // and the device time and iterations of the last solve's first round
  int batch_tile_rows = 0;
  double batch_round_ms = 0.0;
  int batch_round_its = 0;
  double batch_tune_ms[4] = {-1.0, -1.0, -1.0, -1.0};  // ms per iteration of tiles of 256 .. 2048 rows

  // errors raised by kernels (negative Jacobian count, graph misses, ...)
  nalu_gb300::DBuf<int32_t> d_flags;     // [4]

  // asynchronous result download (nalu_linsys_copy_async): two staging
  // copies of values/rhs used in turn (a snapshot waits only for the
  // download two calls back, so downloads run back to back), a second
  // stream for the device-to-host transfers, events
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_snap = nullptr, ev_copied[2] = {nullptr, nullptr};
  bool copy_pending[2] = {false, false};
  int copy_slot = 0;
  nalu_gb300::DBuf<double> stage_values[2], stage_rhs[2];

  // timing
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t user_ev[64] = {};
  double last_assemble_ms = 0.0;
  nalu_gb300::DBuf<uint8_t> flush_buf;

  nalu_gb300::SolverWork sw;
  nalu_gb300::LearnedState learned;
  nalu_gb300::MlState* ml = nullptr;  // aggregation multigrid of the last multilevel solve

  // boundary side sets (nalu_faceset_define / nalu_faceset_skin)
  nalu_gb300::FaceSet face_sets[NALU_MAX_FACE_SETS];

  // staged field uploads (nalu_field_set_async): a third stream, the event of
  // the latest upload, and the event after which the retired buffers are free
  cudaStream_t upload_stream = nullptr;
  cudaEvent_t ev_uploaded = nullptr, ev_released = nullptr;
  bool any_pending = false, released_recorded = false;

  // HexSCV volumes [E][8], kept while the coordinates do not change
  // (coords_version counts coordinate uploads)
  nalu_gb300::DBuf<double> d_scv;
  int64_t coords_version = 0, scv_version = -1;
};

namespace nalu_gb300 {

enum FlagSlot { FLAG_NEG_JAC = 0, FLAG_GRAPH_MISS = 1, FLAG_CAPACITY = 2, FLAG_NONFINITE = 3 };

int set_error(nalu_ctx* ctx, int status, const std::string& msg);
int field_comps(int field);
// swap in the fields staged by nalu_field_set_async (the main stream waits
// for their upload); every call that reads fields starts with it
int resolve_uploads(nalu_ctx* ctx);
#define NALU_RESOLVE_UPLOADS(ctx)                  \
  do {                                             \
    const int rc_res_ = resolve_uploads(ctx);      \
    if (rc_res_ != NALU_OK) return rc_res_;        \
  } while (0)
int launch_permute_in_on(nalu_ctx* ctx, cudaStream_t st, const double* src, double* dst, int comps, int64_t n);
int cuda_check(nalu_ctx* ctx, cudaError_t e, const char* what);
#define NALU_CUDA(ctx, call)                                      \
  do {                                                            \
    cudaError_t e_ = (call);                                      \
    if (e_ != cudaSuccess) return nalu_gb300::cuda_check(ctx, e_, #call); \
  } while (0)

// launchers implemented in assemble.cu
int launch_assemble(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int scatter);
int launch_capture(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int64_t elem, double* d_lhs,
                   double* d_rhs);
int launch_mdot(nalu_ctx* ctx, const nalu_assemble_opts& o);
// assemble_df.cu (double-float element math for the scalar kernels)
int launch_assemble_df(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int scatter);
int launch_mdot_df(nalu_ctx* ctx, const nalu_assemble_opts& o);  // ComputeMdot, df64 element math
int launch_capture_df(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int64_t elem, double* d_lhs,
                      double* d_rhs);
int launch_slot_table(nalu_ctx* ctx);
// geometry.cu
int launch_mass(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int scatter, int64_t cap_elem,
                double* cap_lhs, double* cap_rhs);
int launch_dual_volume(nalu_ctx* ctx, double* vol, int64_t cap_elem, double* cap);
// make d_scv hold the current coordinates' SCV volumes
int ensure_scv_cache(nalu_ctx* ctx);
int launch_nodal_grad(nalu_ctx* ctx, const double* q, int ncomp, const double* dvol, double* grad, bool shifted,
                      int arith);
int launch_expand_graph(nalu_ctx* ctx);
int launch_sum_into(nalu_ctx* ctx, int64_t n, const int64_t* d_elems, const double* d_lhs,
                    const double* d_rhs);
int launch_bc_rows(nalu_ctx* ctx, int64_t n, const int32_t* d_rows, const double* d_vals, int mode);
int launch_permute_in(nalu_ctx* ctx, const double* src, double* dst, int comps, int64_t n);
int launch_permute_out(nalu_ctx* ctx, const double* src, double* dst, int comps, int64_t n);
int launch_fill(nalu_ctx* ctx, double* p, int64_t n, double v);
int check_flags(nalu_ctx* ctx);
int probe_fp64(nalu_ctx* ctx, double* tflops);

// krylov.cu
int solve(nalu_ctx* ctx, const nalu_solver_opts& o, nalu_solve_info* info);
int spmv_fp64(nalu_ctx* ctx, const double* x, double* y);
int compute_dinv(nalu_ctx* ctx);  // sw.dinv and d_bcmask for the current matrix
// cg_fast.cu
template <class VT>
int sell_build(nalu_ctx* ctx, SellMatrix& S, const VT** vals_out);
// learned.cu
int learned_prepare(nalu_ctx* ctx);
// train_tc.cu: the fused BF16 tensor-core training step (device arrays)
struct TrainData {
  const float* st;      // [n][81] static features
  const float* rf;      // [n][27] residual features
  const float* tg;      // [n] targets
  const int32_t* idx;   // [epochs * steps_per_epoch][B] training order
  const int32_t* vidx;  // [n_val] held-out samples
  int B, steps_per_epoch, epochs;
  int64_t n_val;
  float lr;
};
int train_tc(nalu_ctx* ctx, const TrainData& d, float* history);
// gradient (into grad_dev, [NALU_LEARNED_PARAMS]) and mean squared error
// (loss_dev[0]) of the samples idx[0..n) at the current weights
int gradient_tc(nalu_ctx* ctx, const float* st, const float* rf, const float* tg, const int32_t* idx, int n,
                float* grad_dev, float* loss_dev);
// the learned preconditioner's FP32 values (wsell) of rows [row0, row1) only;
// the rows' neighbours in A must lie in the same range (a problem of a batch)
int learned_prepare_rows(nalu_ctx* ctx, int64_t row0, int64_t row1);
// aggregation multigrid (multilevel.cu): the hierarchy for the current scalar
// matrix; flexible CG with it on the residual r (in place) for the correction
// x; the hierarchy's level sizes; its release
// row_off: row ranges of independent problems (a block-diagonal union), each
// coarsened on its own down to the coarsest size (null: one problem)
int ml_setup(nalu_ctx* ctx, bool learned_smoother, const std::vector<int64_t>* row_off = nullptr);
// flexible CG on FP32-pair vectors (learned.cu) preconditioned by prec(rf, zf),
// which launches kernels computing zf ~ A^-1 rf on the context stream
int fcg_df_external(nalu_ctx* ctx, double* x, double* r, double rtol, double r0norm, int max_it, int check_every,
                    const std::function<void(const float*, float*)>& prec, int* iters_out);
int fcg_multilevel(nalu_ctx* ctx, double* x, double* r, double rtol, double r0norm, int max_it, int check_every,
                   int klevels, int learned_sweeps, int* iters);
// one multigrid cycle z = M r (FP32, on the context's stream; graph-capturable)
int ml_apply(nalu_ctx* ctx, const float* rf, float* zf);
int ml_levels(const nalu_ctx* ctx, int max_levels, int64_t* rows, int64_t* nnz);
void ml_free(nalu_ctx* ctx);  // slot map, stencil and SELL preconditioner for the current matrix
// flexible CG with the learned preconditioner on A x = r (x from 0); returns
// NALU_ERR_NOT_CONVERGED with *stalled = 1 when the residual made no progress
// for `stall_window` iterations
int fcg_learned(nalu_ctx* ctx, double* x, double* r, double rtol, double r0norm, int max_it, int check_every,
                int stall_window, int* iters_out, int* stalled, float* iter_ms = nullptr);
// 16-bit column offsets of the SELL copy (built once per SELL build)
int sell_c16_ensure(nalu_ctx* ctx, SellMatrix& S);  // cg_fast.cu
unsigned wave_grid(nalu_ctx* ctx, const void* kernel, int threads);  // cg_fast.cu
// *iter_ms (optional): device time of the iterations alone (set-up excluded)
int pcg_df(nalu_ctx* ctx, const SellMatrix& S, double* x, double* r, double* z, double* q, const double* dinv,
           double rtol, double r0norm, int max_it, int check_every, int* iters_out, float* iter_ms = nullptr);
template <class T, class VT>
int pcg_fast(nalu_ctx* ctx, const VT* sval, const SellMatrix& S, T* x, T* r, T* z, T* p0, T* p1, T* q,
             const T* dinv, double rtol, double r0norm, int max_it, int check_every, int* iters_out);

}  // namespace nalu_gb300
