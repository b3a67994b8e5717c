// api.cu -- C ABI entry points: context, mesh, fields, linear-system graph and
// row operations.  Assembly/solve launchers live in assemble.cu, momentum.cu
// and krylov.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include "internal.h"

using namespace nalu_gb300;

namespace nalu_gb300 {

int set_error(nalu_ctx* ctx, int status, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return status;
}

int cuda_check(nalu_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return NALU_OK;
  cudaGetLastError();  // clear a pending launch error so that it does not resurface in a later call
  return set_error(ctx, NALU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int check_flags(nalu_ctx* ctx) {
  int32_t f[4] = {0, 0, 0, 0};
  NALU_CUDA(ctx, cudaMemcpyAsync(f, ctx->d_flags.p, sizeof(f), cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (f[0] || f[1] || f[2] || f[3]) {
    NALU_CUDA(ctx, cudaMemsetAsync(ctx->d_flags.p, 0, sizeof(f), ctx->stream));
  }
  if (f[FLAG_NEG_JAC])
    return set_error(ctx, NALU_ERR_NEG_JACOBIAN,
                     "det(J) <= 0 at " + std::to_string(f[FLAG_NEG_JAC]) + " element integration point set(s)");
  if (f[FLAG_GRAPH_MISS])
    return set_error(ctx, NALU_ERR_GRAPH, std::to_string(f[FLAG_GRAPH_MISS]) + " element entries missing from graph");
  if (f[FLAG_CAPACITY])
    return set_error(ctx, NALU_ERR_CAPACITY, "a node-graph row is longer than 256 entries");
  if (f[FLAG_NONFINITE]) return set_error(ctx, NALU_ERR_NONFINITE, "non-finite value detected");
  return NALU_OK;
}

int field_comps(int f) {
  switch (f) {
    case NALU_FIELD_COORDINATES:
    case NALU_FIELD_VELOCITY:
    case NALU_FIELD_VELOCITY_RTM:
    case NALU_FIELD_DPDX:
    case NALU_FIELD_VELOCITY_N:
    case NALU_FIELD_VELOCITY_NM1:
    case NALU_FIELD_VELOCITY_BC:
      return 3;
    case NALU_FIELD_DUDX:
      return 9;
    case NALU_FIELD_MDOT_SCS:
      return 12;
    case NALU_FIELD_DUAL_VOLUME:
      return 1;
    default:
      return 1;
  }
}

int resolve_uploads(nalu_ctx* ctx) {
  if (!ctx->any_pending) return NALU_OK;
  cudaSetDevice(ctx->device);
  NALU_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_uploaded, 0));
  for (int fi = 0; fi < NALU_FIELD_COUNT; ++fi) {
    Field& f = ctx->fields[fi];
    if (!f.pending) continue;
    f.swap_back();
    f.pending = false;
    f.set = true;
    if (fi == NALU_FIELD_COORDINATES) ++ctx->coords_version;
  }
  // the retired buffers were read by the work queued so far; the next upload
  // into them waits for this point
  NALU_CUDA(ctx, cudaEventRecord(ctx->ev_released, ctx->stream));
  ctx->released_recorded = true;
  ctx->any_pending = false;
  return NALU_OK;
}

}  // namespace nalu_gb300

namespace {


template <class F>
void parallel_ranges(int64_t n, F f) {
  int nt = (int)std::max(1u, std::thread::hardware_concurrency());
  nt = std::min(nt, 64);
  if (n < 4096) nt = 1;
  if (nt == 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  const int64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const int64_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([=]() { f(b, e); });
  }
  for (auto& x : th) x.join();
}

struct Pinned {
  void* p = nullptr;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

// copy host or device data to a device buffer
int to_device(nalu_ctx* ctx, void* dst, const void* src, size_t bytes, int src_is_device) {
  NALU_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, src_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 ctx->stream));
  return NALU_OK;
}

}  // namespace

extern "C" {

const char* nalu_status_string(int s) {
  switch (s) {
    case NALU_OK: return "ok";
    case NALU_ERR_ARG: return "invalid argument";
    case NALU_ERR_CUDA: return "CUDA error";
    case NALU_ERR_STATE: return "call out of order";
    case NALU_ERR_NEG_JACOBIAN: return "negative or zero Jacobian determinant";
    case NALU_ERR_NONFINITE: return "non-finite value";
    case NALU_ERR_CAPACITY: return "capacity exceeded";
    case NALU_ERR_NOT_CONVERGED: return "solver did not converge";
    case NALU_ERR_GRAPH: return "entry missing from graph";
    case NALU_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

int nalu_create(int device, nalu_ctx** out) {
  if (!out) return NALU_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) return NALU_ERR_NO_DEVICE;
  nalu_ctx* ctx = new nalu_ctx();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete ctx;
    return NALU_ERR_NO_DEVICE;
  }
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
      ctx->d_flags.alloc(4) != cudaSuccess || cudaMemset(ctx->d_flags.p, 0, 16) != cudaSuccess) {
    delete ctx;
    return NALU_ERR_CUDA;
  }
  *out = ctx;
  return NALU_OK;
}

int nalu_destroy(nalu_ctx* ctx) {
  if (!ctx) return NALU_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  nalu_gb300::ml_free(ctx);
  ctx->d_conn.free();
  ctx->d_lid.free();
  for (auto& f : ctx->fields) f.d.free();
  ctx->d_nrowptr.free();
  ctx->d_ncolind.free();
  ctx->d_rowptr.free();
  ctx->d_colind.free();
  ctx->d_values.free();
  ctx->d_rhs.free();
  ctx->d_x.free();
  ctx->d_slots.free();
  ctx->d_bcmask.free();
  ctx->d_colour_elems.free();
  ctx->d_node_df.free();
  ctx->d_flags.free();
  ctx->flush_buf.free();
  for (auto& ev : ctx->user_ev)
    if (ev) cudaEventDestroy(ev);
  auto& s = ctx->sw;
  for (auto* b : {&s.r, &s.z, &s.p, &s.q, &s.ap, &s.dinv, &s.w, &s.tmp, &s.V, &s.Hbuf, &s.scal, &s.partial}) b->free();
  for (auto* b : {&s.fvals, &s.fr, &s.fz, &s.fp, &s.fq, &s.fdinv, &s.fx, &s.fV}) b->free();
  s.sell.ptr.free();
  s.sell.len.free();
  s.sell.col.free();
  s.sell.vald.free();
  s.sell.valf.free();
  s.b3rp.free();
  s.b3col.free();
  s.b3val.free();
  if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
  if (ctx->upload_stream) {
    cudaStreamSynchronize(ctx->upload_stream);
    cudaEventDestroy(ctx->ev_uploaded);
    cudaEventDestroy(ctx->ev_released);
    cudaStreamDestroy(ctx->upload_stream);
  }
  if (ctx->ev_snap) cudaEventDestroy(ctx->ev_snap);
  for (cudaEvent_t e : ctx->ev_copied)
    if (e) cudaEventDestroy(e);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return NALU_OK;
}

const char* nalu_last_error(const nalu_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int nalu_get_stream(nalu_ctx* ctx, void** stream) {
  if (!ctx || !stream) return NALU_ERR_ARG;
  *stream = (void*)ctx->stream;
  return NALU_OK;
}

int nalu_synchronize(nalu_ctx* ctx) {
  if (!ctx) return NALU_ERR_ARG;
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->copy_stream) NALU_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
  if (ctx->upload_stream) NALU_CUDA(ctx, cudaStreamSynchronize(ctx->upload_stream));
  ctx->copy_pending[0] = ctx->copy_pending[1] = false;
  return NALU_OK;
}

int64_t nalu_kernel_launch_count(const nalu_ctx* ctx) { return ctx ? ctx->launches : -1; }
double nalu_last_assemble_ms(const nalu_ctx* ctx) {
  if (!ctx) return -1.0;
  nalu_ctx* c = const_cast<nalu_ctx*>(ctx);
  if (cudaEventSynchronize(c->ev1) != cudaSuccess) return -1.0;
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) != cudaSuccess) return -1.0;
  c->last_assemble_ms = ms;
  return ms;
}

int nalu_probe_fp64_tflops(nalu_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return NALU_ERR_ARG;
  cudaSetDevice(ctx->device);
  return probe_fp64(ctx, tflops);
}

int nalu_event_record(nalu_ctx* ctx, int slot) {
  if (!ctx || slot < 0 || slot >= 64) return NALU_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (!ctx->user_ev[slot]) NALU_CUDA(ctx, cudaEventCreate(&ctx->user_ev[slot]));
  NALU_CUDA(ctx, cudaEventRecord(ctx->user_ev[slot], ctx->stream));
  return NALU_OK;
}

int nalu_event_elapsed_ms(nalu_ctx* ctx, int a, int b, double* ms) {
  if (!ctx || !ms || a < 0 || a >= 64 || b < 0 || b >= 64) return NALU_ERR_ARG;
  if (!ctx->user_ev[a] || !ctx->user_ev[b]) return set_error(ctx, NALU_ERR_STATE, "event slot not recorded");
  cudaSetDevice(ctx->device);
  NALU_CUDA(ctx, cudaEventSynchronize(ctx->user_ev[b]));
  float f = 0.0f;
  NALU_CUDA(ctx, cudaEventElapsedTime(&f, ctx->user_ev[a], ctx->user_ev[b]));
  *ms = f;
  return NALU_OK;
}

int nalu_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return NALU_ERR_ARG;
  *ptr = nullptr;
  if (cudaMallocHost(ptr, bytes) != cudaSuccess) return NALU_ERR_CUDA;
  return NALU_OK;
}

int nalu_host_free(void* ptr) {
  if (ptr && cudaFreeHost(ptr) != cudaSuccess) return NALU_ERR_CUDA;
  return NALU_OK;
}

int nalu_flush_l2(nalu_ctx* ctx, size_t bytes) {
  if (!ctx) return NALU_ERR_ARG;
  cudaSetDevice(ctx->device);
  if ((size_t)ctx->flush_buf.n < bytes) NALU_CUDA(ctx, ctx->flush_buf.alloc((int64_t)bytes));
  NALU_CUDA(ctx, cudaMemsetAsync(ctx->flush_buf.p, 0, bytes, ctx->stream));
  return NALU_OK;
}

// ---- mesh -------------------------------------------------------------------
int nalu_mesh_create(nalu_ctx* ctx, int64_t n_nodes, int64_t n_elems, const int32_t* conn, const int64_t* gid,
                     const double* coords) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || n_nodes <= 0 || n_elems <= 0 || !conn || !coords) return set_error(ctx, NALU_ERR_ARG, "mesh args");
  if (n_nodes >= (int64_t)INT32_MAX / 3) return set_error(ctx, NALU_ERR_CAPACITY, "too many nodes for int32 LIDs");
  cudaSetDevice(ctx->device);
  ctx->n_nodes = n_nodes;
  ctx->n_elems = n_elems;
  ctx->num_dof = 0;
  ctx->learned.nbr_nodes = 0;  // the slot map belongs to the previous mesh
  ctx->problem_offsets.clear();
  for (auto& fs : ctx->face_sets) fs.clear();  // side sets refer to the previous mesh's elements
  ++ctx->coords_version;
  // LIDs: nodes sorted by global id (beginLinearSystemConstruction, :262-275)
  ctx->h_lid.assign(n_nodes, 0);
  ctx->h_gid.resize(n_nodes);
  ctx->identity_order = true;
  if (gid) {
    std::vector<int64_t> order(n_nodes);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return gid[a] < gid[b]; });
    for (int64_t k = 0; k < n_nodes; ++k) {
      ctx->h_lid[order[k]] = (int32_t)k;
      ctx->h_gid[k] = gid[order[k]];
      if (order[k] != k) ctx->identity_order = false;
    }
    for (int64_t k = 1; k < n_nodes; ++k)
      if (gid[order[k]] == gid[order[k - 1]]) return set_error(ctx, NALU_ERR_ARG, "duplicate node global id");
  } else {
    std::iota(ctx->h_lid.begin(), ctx->h_lid.end(), 0);
    std::iota(ctx->h_gid.begin(), ctx->h_gid.end(), (int64_t)1);
  }
  ctx->h_conn_lid.resize((size_t)n_elems * 8);
  for (int64_t i = 0; i < n_elems * 8; ++i) {
    const int32_t n = conn[i];
    if (n < 0 || n >= n_nodes) return set_error(ctx, NALU_ERR_ARG, "connectivity index out of range");
    ctx->h_conn_lid[i] = ctx->h_lid[n];
  }
  NALU_CUDA(ctx, ctx->d_conn.alloc(n_elems * 8));
  NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_conn.p, ctx->h_conn_lid.data(), sizeof(int32_t) * n_elems * 8,
                                 cudaMemcpyHostToDevice, ctx->stream));
  NALU_CUDA(ctx, ctx->d_lid.alloc(n_nodes));
  NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_lid.p, ctx->h_lid.data(), sizeof(int32_t) * n_nodes, cudaMemcpyHostToDevice,
                                 ctx->stream));
  for (auto& f : ctx->fields) {
    f.d.free();
    f.set = false;
  }
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return nalu_field_set(ctx, NALU_FIELD_COORDINATES, coords, n_nodes * 3, 0);
}

int nalu_field_set(nalu_ctx* ctx, int field, const double* src, int64_t count, int src_is_device) {
  if (!ctx || field < 0 || field >= NALU_FIELD_COUNT || !src) return set_error(ctx, NALU_ERR_ARG, "field args");
  if (ctx->n_nodes == 0) return set_error(ctx, NALU_ERR_STATE, "no mesh");
  cudaSetDevice(ctx->device);
  int rc0 = resolve_uploads(ctx);  // an earlier staged upload must not land after this one
  if (rc0) return rc0;
  const int comps = field_comps(field);
  const bool elem = field == NALU_FIELD_MDOT_SCS;
  const int64_t n = elem ? ctx->n_elems : ctx->n_nodes;
  if (count != n * comps) return set_error(ctx, NALU_ERR_ARG, "field size mismatch");
  Field& f = ctx->fields[field];
  if (f.d.n != count) NALU_CUDA(ctx, f.d.alloc(count));
  f.comps = comps;
  if (elem || ctx->identity_order) {
    int rc = to_device(ctx, f.d.p, src, sizeof(double) * count, src_is_device);
    if (rc) return rc;
  } else {
    DBuf<double> tmp;
    NALU_CUDA(ctx, tmp.alloc(count));
    int rc = to_device(ctx, tmp.p, src, sizeof(double) * count, src_is_device);
    if (rc == NALU_OK) rc = launch_permute_in(ctx, tmp.p, f.d.p, comps, n);
    cudaStreamSynchronize(ctx->stream);
    tmp.free();
    if (rc) return rc;
  }
  f.set = true;
  if (field == NALU_FIELD_COORDINATES) ++ctx->coords_version;
  return NALU_OK;
}

int nalu_field_set_async(nalu_ctx* ctx, int field, const double* src, int64_t count) {
  if (!ctx || field < 0 || field >= NALU_FIELD_COUNT || !src) return set_error(ctx, NALU_ERR_ARG, "field args");
  if (ctx->n_nodes == 0) return set_error(ctx, NALU_ERR_STATE, "no mesh");
  const int comps = field_comps(field);
  const bool elem = field == NALU_FIELD_MDOT_SCS;
  const int64_t n = elem ? ctx->n_elems : ctx->n_nodes;
  if (count != n * comps) return set_error(ctx, NALU_ERR_ARG, "field size mismatch");
  cudaSetDevice(ctx->device);
  if (!ctx->upload_stream) {
    NALU_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->upload_stream, cudaStreamNonBlocking));
    NALU_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_uploaded, cudaEventDisableTiming));
    NALU_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_released, cudaEventDisableTiming));
  }
  Field& f = ctx->fields[field];
  // buffers are (re)sized only when the field is new or changes size
  if (f.d.n != count) NALU_CUDA(ctx, f.d.alloc(count));
  if (f.back.n != count) NALU_CUDA(ctx, f.back.alloc(count));
  if (ctx->released_recorded) NALU_CUDA(ctx, cudaStreamWaitEvent(ctx->upload_stream, ctx->ev_released, 0));
  if (elem || ctx->identity_order) {
    NALU_CUDA(ctx, cudaMemcpyAsync(f.back.p, src, sizeof(double) * count, cudaMemcpyHostToDevice, ctx->upload_stream));
  } else {
    if (f.stage.n != count) NALU_CUDA(ctx, f.stage.alloc(count));
    NALU_CUDA(ctx, cudaMemcpyAsync(f.stage.p, src, sizeof(double) * count, cudaMemcpyHostToDevice, ctx->upload_stream));
    int rc = launch_permute_in_on(ctx, ctx->upload_stream, f.stage.p, f.back.p, comps, n);
    if (rc) return rc;
  }
  NALU_CUDA(ctx, cudaEventRecord(ctx->ev_uploaded, ctx->upload_stream));
  f.comps = comps;
  f.pending = true;
  ctx->any_pending = true;
  return NALU_OK;
}

int nalu_field_get(nalu_ctx* ctx, int field, double* dst, int64_t count, int dst_is_device) {
  if (!ctx || field < 0 || field >= NALU_FIELD_COUNT || !dst) return set_error(ctx, NALU_ERR_ARG, "field args");
  {
    const int rc0 = resolve_uploads(ctx);
    if (rc0) return rc0;
  }
  Field& f = ctx->fields[field];
  if (!f.set) return set_error(ctx, NALU_ERR_STATE, "field not set");
  if (count != f.d.n) return set_error(ctx, NALU_ERR_ARG, "field size mismatch");
  cudaSetDevice(ctx->device);
  const bool elem = field == NALU_FIELD_MDOT_SCS;
  if (elem || ctx->identity_order) {
    NALU_CUDA(ctx, cudaMemcpyAsync(dst, f.d.p, sizeof(double) * count,
                                   dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    DBuf<double> tmp;
    NALU_CUDA(ctx, tmp.alloc(count));
    int rc = launch_permute_out(ctx, f.d.p, tmp.p, f.comps, ctx->n_nodes);
    if (rc == NALU_OK)
      rc = cuda_check(ctx, cudaMemcpyAsync(dst, tmp.p, sizeof(double) * count,
                                           dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                           ctx->stream), "copy");
    cudaStreamSynchronize(ctx->stream);
    tmp.free();
    if (rc) return rc;
  }
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

// ---- graph --------------------------------------------------------------------
// Node graph of the Hex8 mesh in Tpetra order: row a lists the LIDs of every
// node that shares an element with a (itself included), ascending and unique --
// the finished result of addConnections + insertIndices on one rank.
int nalu_linsys_build_elem_graph(nalu_ctx* ctx, int num_dof) {
  if (!ctx || num_dof < 1 || num_dof > 8) return set_error(ctx, NALU_ERR_ARG, "num_dof");
  if (ctx->n_nodes == 0) return set_error(ctx, NALU_ERR_STATE, "no mesh");
  cudaSetDevice(ctx->device);
  const int64_t N = ctx->n_nodes, E = ctx->n_elems;
  const int32_t* cl = ctx->h_conn_lid.data();
  // node -> element incidence (CSR)
  std::vector<int64_t> ne(N + 1, 0);
  for (int64_t i = 0; i < E * 8; ++i) ne[cl[i] + 1]++;
  for (int64_t a = 0; a < N; ++a) ne[a + 1] += ne[a];
  std::vector<int32_t> inc(E * 8);
  {
    std::vector<int64_t> pos(ne.begin(), ne.end() - 1);
    for (int64_t e = 0; e < E; ++e)
      for (int k = 0; k < 8; ++k) inc[pos[cl[8 * e + k]]++] = (int32_t)e;
  }
  std::vector<int64_t> nrow(N + 1, 0);
  auto row_nodes = [&](int64_t a, std::vector<int32_t>& buf) {
    buf.clear();
    for (int64_t k = ne[a]; k < ne[a + 1]; ++k) {
      const int32_t* en = cl + 8 * (int64_t)inc[k];
      buf.insert(buf.end(), en, en + 8);
    }
    if (buf.empty()) buf.push_back((int32_t)a);  // isolated node: diagonal only
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
  };
  parallel_ranges(N, [&](int64_t b, int64_t e) {
    std::vector<int32_t> buf;
    for (int64_t a = b; a < e; ++a) {
      row_nodes(a, buf);
      nrow[a + 1] = (int64_t)buf.size();
    }
  });
  for (int64_t a = 0; a < N; ++a) nrow[a + 1] += nrow[a];
  const int64_t nnz_node = nrow[N];
  std::vector<int32_t> ncol(nnz_node);
  parallel_ranges(N, [&](int64_t b, int64_t e) {
    std::vector<int32_t> buf;
    for (int64_t a = b; a < e; ++a) {
      row_nodes(a, buf);
      std::copy(buf.begin(), buf.end(), ncol.begin() + nrow[a]);
    }
  });
  // element colouring (greedy in element order): elements of one colour share no node
  std::vector<uint64_t> mask(N, 0);
  std::vector<uint8_t> colour(E);
  int ncolours = 0;
  for (int64_t e = 0; e < E; ++e) {
    uint64_t used = 0;
    for (int k = 0; k < 8; ++k) used |= mask[cl[8 * e + k]];
    int c = 0;
    while (c < 64 && ((used >> c) & 1)) ++c;
    if (c >= 64) return set_error(ctx, NALU_ERR_CAPACITY, "element colouring needs more than 64 colours");
    colour[e] = (uint8_t)c;
    ncolours = std::max(ncolours, c + 1);
    for (int k = 0; k < 8; ++k) mask[cl[8 * e + k]] |= (1ull << c);
  }
  std::vector<int64_t> coff(ncolours + 1, 0);
  for (int64_t e = 0; e < E; ++e) coff[colour[e] + 1]++;
  for (int c = 0; c < ncolours; ++c) coff[c + 1] += coff[c];
  std::vector<int32_t> celems(E);
  {
    std::vector<int64_t> pos(coff.begin(), coff.end() - 1);
    for (int64_t e = 0; e < E; ++e) celems[pos[colour[e]]++] = (int32_t)e;
  }
  ctx->colour_offsets = coff;

  ctx->num_dof = num_dof;
  ctx->node_nnz = nnz_node;
  ctx->n_rows = N * num_dof;
  ctx->nnz = nnz_node * num_dof * num_dof;
  NALU_CUDA(ctx, ctx->d_nrowptr.alloc(N + 1));
  NALU_CUDA(ctx, ctx->d_ncolind.alloc(nnz_node));
  NALU_CUDA(ctx, ctx->d_rowptr.alloc(ctx->n_rows + 1));
  NALU_CUDA(ctx, ctx->d_colind.alloc(ctx->nnz));
  NALU_CUDA(ctx, ctx->d_values.alloc(ctx->nnz));
  NALU_CUDA(ctx, ctx->d_rhs.alloc(ctx->n_rows));
  NALU_CUDA(ctx, ctx->d_x.alloc(ctx->n_rows));
  NALU_CUDA(ctx, ctx->d_slots.alloc(E * 64));
  NALU_CUDA(ctx, ctx->d_colour_elems.alloc(E));
  NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_nrowptr.p, nrow.data(), sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice,
                                 ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_ncolind.p, ncol.data(), sizeof(int32_t) * nnz_node, cudaMemcpyHostToDevice,
                                 ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_colour_elems.p, celems.data(), sizeof(int32_t) * E, cudaMemcpyHostToDevice,
                                 ctx->stream));
  if (num_dof == 1) {
    NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_rowptr.p, ctx->d_nrowptr.p, sizeof(int64_t) * (N + 1),
                                   cudaMemcpyDeviceToDevice, ctx->stream));
    NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_colind.p, ctx->d_ncolind.p, sizeof(int32_t) * nnz_node,
                                   cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    int rc = launch_expand_graph(ctx);
    if (rc) return rc;
  }
  int rc = launch_slot_table(ctx);
  if (rc) return rc;
  NALU_CUDA(ctx, cudaMemsetAsync(ctx->d_values.p, 0, sizeof(double) * ctx->nnz, ctx->stream));
  NALU_CUDA(ctx, cudaMemsetAsync(ctx->d_rhs.p, 0, sizeof(double) * ctx->n_rows, ctx->stream));
  NALU_CUDA(ctx, cudaMemsetAsync(ctx->d_x.p, 0, sizeof(double) * ctx->n_rows, ctx->stream));
  for (auto& k : ctx->scatter_choice) k[0] = k[1] = 0;
  for (int k = 0; k < 2; ++k) ctx->df_schedule[k] = ctx->df_scatter[k] = 0;
  // the host build (sorting, colouring) is synchronous; the uploads finish here
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return check_flags(ctx);
}

int nalu_linsys_sizes(nalu_ctx* ctx, int64_t* n_rows, int64_t* nnz, int* num_dof) {
  if (!ctx) return NALU_ERR_ARG;
  if (n_rows) *n_rows = ctx->n_rows;
  if (nnz) *nnz = ctx->nnz;
  if (num_dof) *num_dof = ctx->num_dof;
  return NALU_OK;
}

int nalu_linsys_graph(nalu_ctx* ctx, int64_t* rowptr, int32_t* colind) {
  if (!ctx) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  if (rowptr)
    NALU_CUDA(ctx, cudaMemcpyAsync(rowptr, ctx->d_rowptr.p, sizeof(int64_t) * (ctx->n_rows + 1),
                                   cudaMemcpyDeviceToHost, ctx->stream));
  if (colind)
    NALU_CUDA(ctx, cudaMemcpyAsync(colind, ctx->d_colind.p, sizeof(int32_t) * ctx->nnz, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

int nalu_linsys_device_arrays(nalu_ctx* ctx, const int64_t** rowptr, const int32_t** colind, double** values,
                              double** rhs, double** solution) {
  if (!ctx) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  if (rowptr) *rowptr = ctx->d_rowptr.p;
  if (colind) *colind = ctx->d_colind.p;
  if (values) *values = ctx->d_values.p;
  if (rhs) *rhs = ctx->d_rhs.p;
  if (solution) *solution = ctx->d_x.p;
  return NALU_OK;
}

int nalu_linsys_zero(nalu_ctx* ctx) {
  if (!ctx) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  NALU_CUDA(ctx, cudaMemsetAsync(ctx->d_values.p, 0, sizeof(double) * ctx->nnz, ctx->stream));
  NALU_CUDA(ctx, cudaMemsetAsync(ctx->d_rhs.p, 0, sizeof(double) * ctx->n_rows, ctx->stream));
  NALU_CUDA(ctx, cudaMemsetAsync(ctx->d_x.p, 0, sizeof(double) * ctx->n_rows, ctx->stream));
  return NALU_OK;
}

int nalu_linsys_sum_into(nalu_ctx* ctx, int64_t n, const int64_t* elem_ids, const double* lhs, const double* rhs) {
  if (!ctx || n < 0 || (n > 0 && (!elem_ids || !lhs || !rhs))) return set_error(ctx, NALU_ERR_ARG, "sum_into args");
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  if (n == 0) return NALU_OK;
  cudaSetDevice(ctx->device);
  const int ne = 8 * ctx->num_dof;
  DBuf<int64_t> de;
  DBuf<double> dl, dr;
  NALU_CUDA(ctx, de.alloc(n));
  NALU_CUDA(ctx, dl.alloc(n * ne * ne));
  NALU_CUDA(ctx, dr.alloc(n * ne));
  NALU_CUDA(ctx, cudaMemcpyAsync(de.p, elem_ids, sizeof(int64_t) * n, cudaMemcpyHostToDevice, ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(dl.p, lhs, sizeof(double) * n * ne * ne, cudaMemcpyHostToDevice, ctx->stream));
  NALU_CUDA(ctx, cudaMemcpyAsync(dr.p, rhs, sizeof(double) * n * ne, cudaMemcpyHostToDevice, ctx->stream));
  int rc = launch_sum_into(ctx, n, de.p, dl.p, dr.p);
  cudaStreamSynchronize(ctx->stream);
  de.free();
  dl.free();
  dr.free();
  if (rc) return rc;
  return check_flags(ctx);
}

namespace {
// rows for node indices (caller order) and dof range
int bc_rows(nalu_ctx* ctx, int64_t n, const int32_t* node_idx, int begin_dof, int end_dof,
            std::vector<int32_t>& rows) {
  if (begin_dof < 0 || end_dof > ctx->num_dof || begin_dof >= end_dof) return set_error(ctx, NALU_ERR_ARG, "dof range");
  rows.clear();
  for (int64_t k = 0; k < n; ++k) {
    const int32_t ni = node_idx[k];
    if (ni < 0 || ni >= ctx->n_nodes) return set_error(ctx, NALU_ERR_ARG, "node index out of range");
    for (int d = begin_dof; d < end_dof; ++d) rows.push_back(ctx->h_lid[ni] * ctx->num_dof + d);
  }
  return NALU_OK;
}
int run_bc(nalu_ctx* ctx, const std::vector<int32_t>& rows, const std::vector<double>& vals, int mode) {
  if (rows.empty()) return NALU_OK;
  DBuf<int32_t> dr;
  DBuf<double> dv;
  NALU_CUDA(ctx, dr.alloc((int64_t)rows.size()));
  NALU_CUDA(ctx, cudaMemcpyAsync(dr.p, rows.data(), sizeof(int32_t) * rows.size(), cudaMemcpyHostToDevice, ctx->stream));
  if (!vals.empty()) {
    NALU_CUDA(ctx, dv.alloc((int64_t)vals.size()));
    NALU_CUDA(ctx, cudaMemcpyAsync(dv.p, vals.data(), sizeof(double) * vals.size(), cudaMemcpyHostToDevice, ctx->stream));
  }
  int rc = launch_bc_rows(ctx, (int64_t)rows.size(), dr.p, dv.p, mode);
  cudaStreamSynchronize(ctx->stream);
  dr.free();
  dv.free();
  return rc;
}
}  // namespace

int nalu_linsys_apply_dirichlet(nalu_ctx* ctx, int64_t n, const int32_t* node_idx, int begin_dof, int end_dof,
                                const double* bc, const double* solution) {
  if (!ctx || n < 0 || (n > 0 && (!node_idx || !bc || !solution))) return set_error(ctx, NALU_ERR_ARG, "dirichlet args");
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  std::vector<int32_t> rows;
  int rc = bc_rows(ctx, n, node_idx, begin_dof, end_dof, rows);
  if (rc) return rc;
  std::vector<double> vals;
  vals.reserve(rows.size());
  for (int64_t k = 0; k < n; ++k)
    for (int d = begin_dof; d < end_dof; ++d)
      vals.push_back(bc[k * ctx->num_dof + d] - solution[k * ctx->num_dof + d]);
  return run_bc(ctx, rows, vals, 0);
}

int nalu_linsys_reset_rows(nalu_ctx* ctx, int64_t n, const int32_t* node_idx, int begin_dof, int end_dof) {
  if (!ctx || n < 0 || (n > 0 && !node_idx)) return set_error(ctx, NALU_ERR_ARG, "reset args");
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  std::vector<int32_t> rows;
  int rc = bc_rows(ctx, n, node_idx, begin_dof, end_dof, rows);
  if (rc) return rc;
  return run_bc(ctx, rows, {}, 1);
}

int nalu_linsys_sum_into_diag(nalu_ctx* ctx, int32_t node_idx, int dof, double diag, double rhs) {
  if (!ctx) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  std::vector<int32_t> rows;
  int rc = bc_rows(ctx, 1, &node_idx, dof, dof + 1, rows);
  if (rc) return rc;
  return run_bc(ctx, rows, {diag, rhs}, 2);
}

int nalu_linsys_load_complete(nalu_ctx* ctx) {
  if (!ctx) return NALU_ERR_ARG;
  cudaSetDevice(ctx->device);
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return check_flags(ctx);
}

int nalu_linsys_copy_async(nalu_ctx* ctx, double* values, double* rhs) {
  if (!ctx || (!values && !rhs)) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  if (!ctx->copy_stream) {
    NALU_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    NALU_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_snap, cudaEventDisableTiming));
    NALU_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_copied[0], cudaEventDisableTiming));
    NALU_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_copied[1], cudaEventDisableTiming));
  }
  const int k = ctx->copy_slot;
  nalu_gb300::DBuf<double>& sv = ctx->stage_values[k];
  nalu_gb300::DBuf<double>& sr = ctx->stage_rhs[k];
  if (sv.n < ctx->nnz) NALU_CUDA(ctx, sv.alloc(ctx->nnz));
  if (sr.n < ctx->n_rows) NALU_CUDA(ctx, sr.alloc(ctx->n_rows));
  // this staging copy may be overwritten only after its previous download ended
  if (ctx->copy_pending[k]) NALU_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_copied[k], 0));
  if (values)
    NALU_CUDA(ctx, cudaMemcpyAsync(sv.p, ctx->d_values.p, sizeof(double) * ctx->nnz, cudaMemcpyDeviceToDevice,
                                   ctx->stream));
  if (rhs)
    NALU_CUDA(ctx, cudaMemcpyAsync(sr.p, ctx->d_rhs.p, sizeof(double) * ctx->n_rows, cudaMemcpyDeviceToDevice,
                                   ctx->stream));
  NALU_CUDA(ctx, cudaEventRecord(ctx->ev_snap, ctx->stream));
  NALU_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_snap, 0));
  if (values)
    NALU_CUDA(ctx, cudaMemcpyAsync(values, sv.p, sizeof(double) * ctx->nnz, cudaMemcpyDeviceToHost, ctx->copy_stream));
  if (rhs)
    NALU_CUDA(ctx, cudaMemcpyAsync(rhs, sr.p, sizeof(double) * ctx->n_rows, cudaMemcpyDeviceToHost, ctx->copy_stream));
  NALU_CUDA(ctx, cudaEventRecord(ctx->ev_copied[k], ctx->copy_stream));
  ctx->copy_pending[k] = true;
  ctx->copy_slot = k ^ 1;
  return NALU_OK;
}

int nalu_linsys_copy_wait(nalu_ctx* ctx) {
  if (!ctx) return NALU_ERR_ARG;
  cudaSetDevice(ctx->device);
  for (int k = 0; k < 2; ++k) {
    if (!ctx->copy_pending[k]) continue;
    NALU_CUDA(ctx, cudaEventSynchronize(ctx->ev_copied[k]));
    ctx->copy_pending[k] = false;
  }
  return NALU_OK;
}

int nalu_linsys_copy(nalu_ctx* ctx, double* values, double* rhs, int dst_is_device) {
  if (!ctx) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  const cudaMemcpyKind k = dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (values) NALU_CUDA(ctx, cudaMemcpyAsync(values, ctx->d_values.p, sizeof(double) * ctx->nnz, k, ctx->stream));
  if (rhs) NALU_CUDA(ctx, cudaMemcpyAsync(rhs, ctx->d_rhs.p, sizeof(double) * ctx->n_rows, k, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

// ---- assembly -------------------------------------------------------------------
void nalu_assemble_opts_default(nalu_assemble_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->proj_time_scale = 1.0;
  o->alpha = 0.0;       // SolutionOptions defaults (src/SolutionOptions.C:31-49)
  o->alpha_upw = 1.0;
  o->upw_factor = 1.0;
  o->hybrid_factor = 0.0;
  o->include_divu = 0.0;
  o->scatter = NALU_SCATTER_AUTO;
  o->gamma1 = 1.0;      // BDF1 (TimeIntegrator, src/TimeIntegrator.C)
  o->gamma2 = -1.0;
  o->gamma3 = 0.0;
}

namespace {
int kernel_dof(int kernel) {
  return (kernel == NALU_KERNEL_MOMENTUM_ADV_DIFF || kernel == NALU_KERNEL_MOMENTUM_UPW_ADV_DIFF ||
          kernel == NALU_KERNEL_MOMENTUM_MASS) ? 3 : 1;
}

int check_time_opts(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o) {
  if (kernel < NALU_KERNEL_CONTINUITY_MASS) return NALU_OK;
  if (!(o.dt > 0.0) || !std::isfinite(o.dt)) return set_error(ctx, NALU_ERR_ARG, "mass kernels need dt > 0");
  if (!(o.gamma1 != 0.0) || !std::isfinite(o.gamma1) || !std::isfinite(o.gamma2) || !std::isfinite(o.gamma3))
    return set_error(ctx, NALU_ERR_ARG, "mass kernels need finite gammas, gamma1 != 0");
  return NALU_OK;
}

int check_kernel_inputs(nalu_ctx* ctx, int kernel) {
  auto need = [&](int f, const char* name) -> int {
    if (!ctx->fields[f].set) return set_error(ctx, NALU_ERR_STATE, std::string("field not set: ") + name);
    return NALU_OK;
  };
  int rc = need(NALU_FIELD_COORDINATES, "coordinates");
  if (rc) return rc;
  switch (kernel) {
    case NALU_KERNEL_SCALAR_DIFF:
      if ((rc = need(NALU_FIELD_SCALAR_Q, "scalarQ"))) return rc;
      return need(NALU_FIELD_DIFF_COEFF, "diffFluxCoeff");
    case NALU_KERNEL_CONTINUITY_ADV:
      if ((rc = need(NALU_FIELD_VELOCITY, "velocity"))) return rc;
      if ((rc = need(NALU_FIELD_DENSITY, "density"))) return rc;
      if ((rc = need(NALU_FIELD_PRESSURE, "pressure"))) return rc;
      return need(NALU_FIELD_DPDX, "dpdx");
    case NALU_KERNEL_MOMENTUM_ADV_DIFF:
      if ((rc = need(NALU_FIELD_VELOCITY, "velocity"))) return rc;
      if ((rc = need(NALU_FIELD_VISCOSITY, "viscosity"))) return rc;
      return need(NALU_FIELD_MDOT_SCS, "mass_flow_rate_scs");
    case NALU_KERNEL_MOMENTUM_UPW_ADV_DIFF:
      if ((rc = need(NALU_FIELD_VELOCITY, "velocity"))) return rc;
      if ((rc = need(NALU_FIELD_VELOCITY_RTM, "velocity_rtm"))) return rc;
      if ((rc = need(NALU_FIELD_DENSITY, "density"))) return rc;
      if ((rc = need(NALU_FIELD_VISCOSITY, "viscosity"))) return rc;
      if ((rc = need(NALU_FIELD_DUDX, "dudx"))) return rc;
      return need(NALU_FIELD_MDOT_SCS, "mass_flow_rate_scs");
    case NALU_KERNEL_CONTINUITY_MASS:
      if ((rc = need(NALU_FIELD_DENSITY, "density"))) return rc;
      return need(NALU_FIELD_DENSITY_N, "density (state N)");
    case NALU_KERNEL_MOMENTUM_MASS:
      if ((rc = need(NALU_FIELD_DENSITY, "density"))) return rc;
      if ((rc = need(NALU_FIELD_DENSITY_N, "density (state N)"))) return rc;
      if ((rc = need(NALU_FIELD_VELOCITY, "velocity"))) return rc;
      if ((rc = need(NALU_FIELD_VELOCITY_N, "velocity (state N)"))) return rc;
      return need(NALU_FIELD_DPDX, "dpdx");
    default:
      return set_error(ctx, NALU_ERR_ARG, "unknown kernel");
  }
}

double time_assemble(nalu_ctx* ctx, int kernel, const nalu_assemble_opts& o, int scatter, int* rc) {
  cudaEventRecord(ctx->ev0, ctx->stream);
  *rc = launch_assemble(ctx, kernel, o, scatter);
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaEventSynchronize(ctx->ev1);
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  return ms;
}

// Autotuner of the double-float scalar kernels: on the first call of a
// context and kernel whose schedule or scatter is AUTO, time every schedule
// (element per thread, ip per thread with 8 or 16 elements per block) with
// both scatters on scratch copies of the system (two rounds, the second
// counts), keep the fastest pair and its table.  Resolves o.schedule and
// scatter for this call.
int tune_df(nalu_ctx* ctx, int kernel, nalu_assemble_opts& o, int& scatter) {
  const int k = kernel == NALU_KERNEL_SCALAR_DIFF ? 0 : 1;
  const bool auto_sched = !(o.schedule >= NALU_SCHEDULE_ELEMENT && o.schedule <= NALU_SCHEDULE_IP16);
  const bool auto_scatter = scatter == NALU_SCATTER_AUTO;
  int rc = NALU_OK;
  if ((auto_sched || auto_scatter) && ctx->df_schedule[k] == 0) {
    DBuf<double> sv, sr;
    NALU_CUDA(ctx, sv.alloc(ctx->nnz));
    NALU_CUDA(ctx, sr.alloc(ctx->n_rows));
    NALU_CUDA(ctx, cudaMemcpyAsync(sv.p, ctx->d_values.p, sizeof(double) * ctx->nnz, cudaMemcpyDeviceToDevice, ctx->stream));
    NALU_CUDA(ctx, cudaMemcpyAsync(sr.p, ctx->d_rhs.p, sizeof(double) * ctx->n_rows, cudaMemcpyDeviceToDevice, ctx->stream));
    double best = 1e30;
    int best_sched = NALU_SCHEDULE_IP8, best_sc = NALU_SCATTER_ATOMIC;
    for (int rep = 0; rep < 2; ++rep)
      for (int sch = NALU_SCHEDULE_ELEMENT; sch <= NALU_SCHEDULE_IP16; ++sch)
        for (int sc : {NALU_SCATTER_ATOMIC, NALU_SCATTER_COLOURED}) {
          nalu_assemble_opts t = o;
          t.schedule = sch;
          const double ms = time_assemble(ctx, kernel, t, sc, &rc);
          if (rc) return rc;
          if (rep == 1) {
            ctx->df_tune_ms[k][sch - 1][sc - 1] = ms;
            if (ms < best) best = ms, best_sched = sch, best_sc = sc;
          }
        }
    NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_values.p, sv.p, sizeof(double) * ctx->nnz, cudaMemcpyDeviceToDevice, ctx->stream));
    NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_rhs.p, sr.p, sizeof(double) * ctx->n_rows, cudaMemcpyDeviceToDevice, ctx->stream));
    NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->df_schedule[k] = best_sched;
    ctx->df_scatter[k] = best_sc;
    rc = check_flags(ctx);
    if (rc) return rc;
  }
  if (auto_sched) o.schedule = ctx->df_schedule[k] ? ctx->df_schedule[k] : NALU_SCHEDULE_IP8;
  if (auto_scatter) scatter = ctx->df_scatter[k] ? ctx->df_scatter[k] : NALU_SCATTER_ATOMIC;
  return NALU_OK;
}
}  // namespace

int nalu_assemble_tuning(const nalu_ctx* ctx, int kernel, int* schedule, int* scatter, double* ms) {
  if (!ctx || kernel < NALU_KERNEL_SCALAR_DIFF || kernel > NALU_KERNEL_CONTINUITY_ADV) return NALU_ERR_ARG;
  const int k = kernel == NALU_KERNEL_SCALAR_DIFF ? 0 : 1;
  if (ctx->df_schedule[k] == 0) return NALU_ERR_STATE;
  if (schedule) *schedule = ctx->df_schedule[k];
  if (scatter) *scatter = ctx->df_scatter[k];
  if (ms)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 2; ++j) ms[2 * i + j] = ctx->df_tune_ms[k][i][j] > 0 ? ctx->df_tune_ms[k][i][j] : -1.0;
  return NALU_OK;
}

int nalu_assemble(nalu_ctx* ctx, int kernel, const nalu_assemble_opts* opts) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || !opts || kernel < 0 || kernel > NALU_KERNEL_MOMENTUM_MASS)
    return set_error(ctx, NALU_ERR_ARG, "assemble args");
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  if (ctx->num_dof != kernel_dof(kernel)) return set_error(ctx, NALU_ERR_STATE, "graph numDof does not match the kernel");
  if (!(opts->proj_time_scale != 0.0)) return set_error(ctx, NALU_ERR_ARG, "proj_time_scale must be non-zero");
  int rc = check_time_opts(ctx, kernel, *opts);
  if (rc) return rc;
  rc = check_kernel_inputs(ctx, kernel);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  int scatter = opts->scatter;
  // the mass kernels scatter a few entries per row: atomics, no autotuning
  if (scatter == NALU_SCATTER_AUTO && kernel >= NALU_KERNEL_CONTINUITY_MASS) scatter = NALU_SCATTER_ATOMIC;
  if (opts->arith == NALU_ARITH_DF64 && kernel <= NALU_KERNEL_CONTINUITY_ADV) {
    // double-float scalar kernels: schedule x scatter, tuned together
    nalu_assemble_opts o = *opts;
    rc = tune_df(ctx, kernel, o, scatter);
    if (rc) return rc;
    cudaEventRecord(ctx->ev0, ctx->stream);
    rc = launch_assemble(ctx, kernel, o, scatter);
    cudaEventRecord(ctx->ev1, ctx->stream);
    return rc;
  }
  if (scatter == NALU_SCATTER_AUTO) {
    const int ar = opts->arith == NALU_ARITH_DF64 ? 1 : 0;
    scatter = ctx->scatter_choice[kernel][ar];
    if (scatter == 0) {
      // autotune: time both strategies on scratch copies of values/rhs
      DBuf<double> sv, sr;
      NALU_CUDA(ctx, sv.alloc(ctx->nnz));
      NALU_CUDA(ctx, sr.alloc(ctx->n_rows));
      NALU_CUDA(ctx, cudaMemcpyAsync(sv.p, ctx->d_values.p, sizeof(double) * ctx->nnz, cudaMemcpyDeviceToDevice, ctx->stream));
      NALU_CUDA(ctx, cudaMemcpyAsync(sr.p, ctx->d_rhs.p, sizeof(double) * ctx->n_rows, cudaMemcpyDeviceToDevice, ctx->stream));
      double best = 1e30;
      int pick = NALU_SCATTER_ATOMIC;
      for (int rep = 0; rep < 2; ++rep)
        for (int s : {NALU_SCATTER_ATOMIC, NALU_SCATTER_COLOURED}) {
          const double ms = time_assemble(ctx, kernel, *opts, s, &rc);
          if (rc) return rc;
          if (rep == 1 && ms < best) best = ms, pick = s;
        }
      NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_values.p, sv.p, sizeof(double) * ctx->nnz, cudaMemcpyDeviceToDevice, ctx->stream));
      NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_rhs.p, sr.p, sizeof(double) * ctx->n_rows, cudaMemcpyDeviceToDevice, ctx->stream));
      NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      sv.free();
      sr.free();
      ctx->scatter_choice[kernel][ar] = pick;
      scatter = pick;
      rc = check_flags(ctx);
      if (rc) return rc;
    }
  }
  cudaEventRecord(ctx->ev0, ctx->stream);
  rc = launch_assemble(ctx, kernel, *opts, scatter);
  cudaEventRecord(ctx->ev1, ctx->stream);
  return rc;
}

int nalu_capture_element(nalu_ctx* ctx, int kernel, const nalu_assemble_opts* opts, int64_t elem, double* lhs,
                         double* rhs) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || !opts || !lhs || !rhs || kernel < 0 || kernel > NALU_KERNEL_MOMENTUM_MASS)
    return set_error(ctx, NALU_ERR_ARG, "capture args");
  if (elem < 0 || elem >= ctx->n_elems) return set_error(ctx, NALU_ERR_ARG, "element out of range");
  int rc = check_time_opts(ctx, kernel, *opts);
  if (rc) return rc;
  rc = check_kernel_inputs(ctx, kernel);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  const int ne = 8 * kernel_dof(kernel);
  DBuf<double> dl, dr;
  NALU_CUDA(ctx, dl.alloc(ne * ne));
  NALU_CUDA(ctx, dr.alloc(ne));
  rc = launch_capture(ctx, kernel, *opts, elem, dl.p, dr.p);
  if (rc == NALU_OK) {
    rc = cuda_check(ctx, cudaMemcpyAsync(lhs, dl.p, sizeof(double) * ne * ne, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (rc == NALU_OK)
      rc = cuda_check(ctx, cudaMemcpyAsync(rhs, dr.p, sizeof(double) * ne, cudaMemcpyDeviceToHost, ctx->stream), "copy");
  }
  cudaStreamSynchronize(ctx->stream);
  dl.free();
  dr.free();
  if (rc) return rc;
  return check_flags(ctx);
}

int nalu_compute_mdot(nalu_ctx* ctx, const nalu_assemble_opts* opts) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || !opts) return NALU_ERR_ARG;
  for (int f : {NALU_FIELD_COORDINATES, NALU_FIELD_DENSITY, NALU_FIELD_VELOCITY_RTM, NALU_FIELD_PRESSURE, NALU_FIELD_DPDX})
    if (!ctx->fields[f].set) return set_error(ctx, NALU_ERR_STATE, "mdot input field not set");
  cudaSetDevice(ctx->device);
  Field& m = ctx->fields[NALU_FIELD_MDOT_SCS];
  if (m.d.n != ctx->n_elems * 12) NALU_CUDA(ctx, m.d.alloc(ctx->n_elems * 12));
  m.comps = 12;
  int rc = launch_mdot(ctx, *opts);
  if (rc) return rc;
  m.set = true;
  return NALU_OK;
}

// ---- nodal geometry and gradients -------------------------------------------------
int nalu_compute_dual_volume(nalu_ctx* ctx) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx) return NALU_ERR_ARG;
  if (!ctx->fields[NALU_FIELD_COORDINATES].set) return set_error(ctx, NALU_ERR_STATE, "no mesh");
  cudaSetDevice(ctx->device);
  Field& v = ctx->fields[NALU_FIELD_DUAL_VOLUME];
  if (v.d.n != ctx->n_nodes) NALU_CUDA(ctx, v.d.alloc(ctx->n_nodes));
  v.comps = 1;
  int rc = launch_dual_volume(ctx, v.d.p, -1, nullptr);
  if (rc) return rc;
  v.set = true;
  return NALU_OK;
}

int nalu_capture_scv_volumes(nalu_ctx* ctx, int64_t elem, double* vol) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || !vol || elem < 0 || elem >= ctx->n_elems) return NALU_ERR_ARG;
  if (!ctx->fields[NALU_FIELD_COORDINATES].set) return set_error(ctx, NALU_ERR_STATE, "no mesh");
  cudaSetDevice(ctx->device);
  DBuf<double> d;
  NALU_CUDA(ctx, d.alloc(8));
  int rc = launch_dual_volume(ctx, nullptr, elem, d.p);
  if (rc) return rc;
  NALU_CUDA(ctx, cudaMemcpyAsync(vol, d.p, sizeof(double) * 8, cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

int nalu_compute_nodal_gradient(nalu_ctx* ctx, int src_field, int dst_field, int shifted, int arith) {
  if (ctx) NALU_RESOLVE_UPLOADS(ctx);
  if (!ctx || src_field < 0 || src_field >= NALU_FIELD_COUNT || dst_field < 0 || dst_field >= NALU_FIELD_COUNT ||
      src_field == NALU_FIELD_MDOT_SCS || dst_field == NALU_FIELD_MDOT_SCS || src_field == dst_field)
    return set_error(ctx, NALU_ERR_ARG, "gradient fields");
  const int sc = field_comps(src_field), dc = field_comps(dst_field);
  if (!((sc == 1 && dc == 3) || (sc == 3 && dc == 9)))
    return set_error(ctx, NALU_ERR_ARG, "gradient of a scalar needs a 3-vector field, of a vector a 9-component one");
  if (!ctx->fields[src_field].set) return set_error(ctx, NALU_ERR_STATE, "gradient source field not set");
  if (!ctx->fields[NALU_FIELD_DUAL_VOLUME].set)
    return set_error(ctx, NALU_ERR_STATE, "dual_nodal_volume not computed (nalu_compute_dual_volume)");
  cudaSetDevice(ctx->device);
  Field& g = ctx->fields[dst_field];
  if (g.d.n != ctx->n_nodes * dc) NALU_CUDA(ctx, g.d.alloc(ctx->n_nodes * dc));
  g.comps = dc;
  if (arith != NALU_ARITH_FP64 && arith != NALU_ARITH_DF64) return set_error(ctx, NALU_ERR_ARG, "arith");
  int rc = launch_nodal_grad(ctx, ctx->fields[src_field].d.p, sc, ctx->fields[NALU_FIELD_DUAL_VOLUME].d.p, g.d.p,
                             shifted != 0, arith);
  if (rc) return rc;
  g.set = true;
  return NALU_OK;
}

// ---- solve --------------------------------------------------------------------
void nalu_solver_opts_default(nalu_solver_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->method = NALU_SOLVER_CG;
  o->precond = NALU_PRECOND_JACOBI;
  o->precision = NALU_PRECISION_FP64;
  o->max_iters = 10000;
  o->restart = 50;
  o->cheb_degree = 4;
  o->check_every = 25;
  o->x0_zero = 1;
  o->tol = 1e-8;
  o->inner_tol = 1e-4;
  o->stall_window = 20;
  o->learned_probe = 1;
}

int nalu_solve(nalu_ctx* ctx, const nalu_solver_opts* opts, nalu_solve_info* info) {
  if (!ctx || !opts) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  nalu_solve_info tmp{};
  return solve(ctx, *opts, info ? info : &tmp);
}

int nalu_solution_get(nalu_ctx* ctx, double* x, int dst_is_device) {
  if (!ctx || !x) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  NALU_CUDA(ctx, cudaMemcpyAsync(x, ctx->d_x.p, sizeof(double) * ctx->n_rows,
                                 dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

int nalu_solution_set(nalu_ctx* ctx, const double* x, int src_is_device) {
  if (!ctx || !x) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  NALU_CUDA(ctx, cudaMemcpyAsync(ctx->d_x.p, x, sizeof(double) * ctx->n_rows,
                                 src_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
  NALU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return NALU_OK;
}

int nalu_spmv(nalu_ctx* ctx, const double* x, double* y, int is_device) {
  if (!ctx || !x || !y) return NALU_ERR_ARG;
  if (ctx->num_dof == 0) return set_error(ctx, NALU_ERR_STATE, "no graph");
  cudaSetDevice(ctx->device);
  const int64_t n = ctx->n_rows;
  if (is_device) return spmv_fp64(ctx, x, y);
  DBuf<double> dx, dy;
  NALU_CUDA(ctx, dx.alloc(n));
  NALU_CUDA(ctx, dy.alloc(n));
  NALU_CUDA(ctx, cudaMemcpyAsync(dx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  int rc = spmv_fp64(ctx, dx.p, dy.p);
  if (rc == NALU_OK)
    rc = cuda_check(ctx, cudaMemcpyAsync(y, dy.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream), "copy");
  cudaStreamSynchronize(ctx->stream);
  dx.free();
  dy.free();
  return rc;
}

}  // extern "C"

int nalu_multilevel_levels(const nalu_ctx* ctx, int max_levels, int64_t* rows, int64_t* nnz) {
  if (!ctx || max_levels < 0) return NALU_ERR_ARG;
  return nalu_gb300::ml_levels(ctx, max_levels, rows, nnz);
}
