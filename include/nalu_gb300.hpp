// nalu_gb300.hpp -- C++ host interface over the C ABI (nalu_gb300.h),
// mirroring the reference classes a Nalu caller uses on this path:
//
//   LinearSystem                 include/LinearSystem.h:39-167 (TpetraLinearSystem)
//   Kernel + the element kernels include/kernel/Kernel.h:95-125, src/kernel/*.C
//   AssembleElemSolverAlgorithm  include/AssembleElemSolverAlgorithm.h:38-112
//   HexSCS, HexSCV               include/master_element/Hex8CVFEM.h:67-234
//   ComputeMdotElemAlgorithm, AssembleNodalGrad{Elem,Boundary}Algorithm,
//   AssembleFaceElemSolverAlgorithm and the continuity face kernels
//
// Header only; every call forwards to the C ABI and turns a non-zero status
// into nalu_gb300::Error.  Method names and argument meaning follow the
// reference (buildElemToNodeGraph, finalizeLinearSystem, zeroSystem, sumInto,
// applyDirichletBCs, resetRows, loadComplete, solve, activeKernels_, execute).
#ifndef NALU_GB300_HPP
#define NALU_GB300_HPP

#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "nalu_gb300.h"

namespace nalu_gb300 {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

// One device + stream + mesh + linear system.
class Context {
 public:
  explicit Context(int device = 0) {
    const int rc = nalu_create(device, &ctx_);
    if (rc) throw Error(rc, std::string("nalu_create: ") + nalu_status_string(rc));
  }
  ~Context() {
    if (ctx_) nalu_destroy(ctx_);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  nalu_ctx* get() const { return ctx_; }
  void check(int rc, const char* what) const {
    if (rc) throw Error(rc, std::string(what) + ": " + nalu_status_string(rc) + ": " + nalu_last_error(ctx_));
  }
  // STK bulk data of one Hex8 block: conn [E][8] node indices, gid (nullable), coords [n][3]
  void mesh(int64_t n_nodes, int64_t n_elems, const int32_t* conn, const int64_t* gid, const double* coords) {
    check(nalu_mesh_create(ctx_, n_nodes, n_elems, conn, gid, coords), "nalu_mesh_create");
    n_nodes_ = n_nodes;
  }
  void field(nalu_field f, const double* v, int64_t count) {
    check(nalu_field_set(ctx_, f, v, count, 0), "nalu_field_set");
  }
  // a boundary part as a side set: face k is side ordinal[k] of element elem[k]
  void sideSet(int set, const std::vector<int64_t>& elem, const std::vector<int32_t>& ordinal) {
    if (elem.size() != ordinal.size()) throw Error(NALU_ERR_ARG, "sideSet: elem and ordinal differ in length");
    check(nalu_faceset_define(ctx_, set, (int64_t)elem.size(), elem.data(), ordinal.data()), "nalu_faceset_define");
  }
  // all exposed sides of the mesh as side set `set`; returns their number
  int64_t skin(int set) {
    int64_t n = 0;
    check(nalu_faceset_skin(ctx_, set, &n), "nalu_faceset_skin");
    return n;
  }
  int64_t n_nodes() const { return n_nodes_; }
  // a field back to the host (count values, in the caller's node order)
  void fieldGet(nalu_field f, double* v, int64_t count) const {
    check(nalu_field_get(ctx_, f, v, count, 0), "nalu_field_get");
  }
  // dual_nodal_volume from the coordinates (ComputeGeometryInteriorAlgorithm,
  // src/ComputeGeometryInteriorAlgorithm.C): NALU_FIELD_DUAL_VOLUME
  void computeDualNodalVolume() { check(nalu_compute_dual_volume(ctx_), "nalu_compute_dual_volume"); }

 private:
  nalu_ctx* ctx_ = nullptr;
  int64_t n_nodes_ = 0;
};

// Hex8 master elements (src/master_element/Hex8CVFEM.C), batched: the
// MasterElement calls for nelem elements at once on the device.  coords
// [nelem][8][3] in the element's node order (host arrays); outputs in the
// reference's layouts.  The grad ops return false where some element has
// det(J) <= 0 at one of its points (outputs still written), as the reference's
// legacy grad_op reports through its error argument; other failures throw.
class HexSCS {
 public:
  explicit HexSCS(Context& ctx) : ctx_(ctx) {}
  // HexSCS::determinant (:547-580): areav [nelem][12][3]
  void determinant(int64_t nelem, const double* coords, double* areav) const {
    ctx_.check(nalu_hex_scs_determinant(ctx_.get(), nelem, coords, areav, 0), "HexSCS::determinant");
  }
  // HexSCS::grad_op (:523-529): gradop, deriv [nelem][12][8][3]; deriv may be null
  bool grad_op(int64_t nelem, const double* coords, double* gradop, double* deriv = nullptr) const {
    return jac_ok(nalu_hex_scs_grad_op(ctx_.get(), nelem, coords, 0, gradop, deriv, 0), "HexSCS::grad_op");
  }
  // HexSCS::shifted_grad_op (:535-541)
  bool shifted_grad_op(int64_t nelem, const double* coords, double* gradop, double* deriv = nullptr) const {
    return jac_ok(nalu_hex_scs_grad_op(ctx_.get(), nelem, coords, 1, gradop, deriv, 0), "HexSCS::shifted_grad_op");
  }
  // HexSCS::face_grad_op / shifted_face_grad_op (:668-684) at the exposed-face
  // ips of side side[e] of each element: gradop [nelem][4][8][3]
  bool face_grad_op(int64_t nelem, const int32_t* side, const double* coords, double* gradop,
                    bool shifted = false) const {
    return jac_ok(nalu_hex_face_grad_op(ctx_.get(), nelem, side, coords, shifted ? 1 : 0, gradop, 0),
                  "HexSCS::face_grad_op");
  }
  // HexSCS::adjacentNodes (lrscv_): left/right node of each of the 12 ips
  static std::vector<int32_t> adjacentNodes() {
    std::vector<int32_t> v(24);
    nalu_hex_scs_adjacent_nodes(v.data());
    return v;
  }
  // HexSCS::shape_fcn / shifted_shape_fcn: [12][8]
  static std::vector<double> shape_fcn(bool shifted = false) {
    std::vector<double> v(96);
    nalu_hex_scs_shape_fcn(shifted ? 1 : 0, v.data());
    return v;
  }
  // HexSCS::side_node_ordinals: the 4 nodes of side `side`
  static std::vector<int32_t> sideNodeOrdinals(int side) {
    std::vector<int32_t> v(4);
    nalu_hex_side_node_ordinals(side, v.data());
    return v;
  }

 private:
  bool jac_ok(int rc, const char* what) const {
    if (rc == NALU_ERR_NEG_JACOBIAN) return false;
    ctx_.check(rc, what);
    return true;
  }
  Context& ctx_;
};

class HexSCV {
 public:
  explicit HexSCV(Context& ctx) : ctx_(ctx) {}
  // HexSCV::determinant (:149-180): vol [nelem][8]
  void determinant(int64_t nelem, const double* coords, double* vol) const {
    ctx_.check(nalu_hex_scv_determinant(ctx_.get(), nelem, coords, vol, 0), "HexSCV::determinant");
  }
  // HexSCV::grad_op / shifted_grad_op (:185-232): gradop, deriv [nelem][8][8][3]
  bool grad_op(int64_t nelem, const double* coords, double* gradop, double* deriv = nullptr,
               bool shifted = false) const {
    const int rc = nalu_hex_scv_grad_op(ctx_.get(), nelem, coords, shifted ? 1 : 0, gradop, deriv, 0);
    if (rc == NALU_ERR_NEG_JACOBIAN) return false;
    ctx_.check(rc, "HexSCV::grad_op");
    return true;
  }

 private:
  Context& ctx_;
};

// The TimeIntegrator values the kernels' setup() reads (BDF coefficients
// gamma1 phi^{n+1} + gamma2 phi^n + gamma3 phi^{n-1}; BDF1 by default).
struct TimeIntegrator {
  double dt = 1.0, gamma1 = 1.0, gamma2 = -1.0, gamma3 = 0.0;
};

// Kernel: the reference's Kernel interface, reduced to what selects a device
// kernel (its id) and its solution options; setup() takes the time integrator.
class Kernel {
 public:
  virtual ~Kernel() = default;
  virtual void setup(const TimeIntegrator& /*ti*/) {}
  virtual int numDof() const { return 1; }
  int id() const { return id_; }
  nalu_assemble_opts opts;

 protected:
  explicit Kernel(int id) : id_(id) { nalu_assemble_opts_default(&opts); }

 private:
  int id_;
};

class ScalarDiffElemKernel : public Kernel {
 public:
  explicit ScalarDiffElemKernel(bool shiftedGradOp = false) : Kernel(NALU_KERNEL_SCALAR_DIFF) {
    opts.shifted_grad_op = shiftedGradOp;
  }
};

class ContinuityAdvElemKernel : public Kernel {
 public:
  ContinuityAdvElemKernel(bool shiftMdot = false, bool shiftPoisson = false, bool reducedSens = false)
      : Kernel(NALU_KERNEL_CONTINUITY_ADV) {
    opts.shift_mdot = shiftMdot;
    opts.shift_poisson = shiftPoisson;
    opts.reduced_sens = reducedSens || shiftPoisson;  // SolutionOptions.C:719-724
  }
  void setup(const TimeIntegrator& ti) override { opts.proj_time_scale = ti.dt / ti.gamma1; }
};

// time terms (src/kernel/ContinuityMassElemKernel.C, MomentumMassElemKernel.C)
class ContinuityMassElemKernel : public Kernel {
 public:
  explicit ContinuityMassElemKernel(bool lumpedMass = false) : ContinuityMassElemKernel(lumpedMass, NALU_KERNEL_CONTINUITY_MASS) {}
  ContinuityMassElemKernel(bool lumpedMass, int id) : Kernel(id) { opts.lumped_mass = lumpedMass; }
  void setup(const TimeIntegrator& ti) override {
    opts.dt = ti.dt;
    opts.gamma1 = ti.gamma1;
    opts.gamma2 = ti.gamma2;
    opts.gamma3 = ti.gamma3;
  }
};

class MomentumMassElemKernel : public ContinuityMassElemKernel {
 public:
  explicit MomentumMassElemKernel(bool lumpedMass = false, bool balancedForce = false)
      : ContinuityMassElemKernel(lumpedMass, NALU_KERNEL_MOMENTUM_MASS) {
    opts.balanced_force = balancedForce;
  }
  int numDof() const override { return 3; }
};

class MomentumAdvDiffElemKernel : public Kernel {
 public:
  explicit MomentumAdvDiffElemKernel(double includeDivU = 0.0, bool shiftedGradOp = false, bool skewSymmetric = false)
      : Kernel(NALU_KERNEL_MOMENTUM_ADV_DIFF) {
    opts.include_divu = includeDivU;
    opts.shifted_grad_op = shiftedGradOp;
    opts.skew_symmetric = skewSymmetric;
  }
  int numDof() const override { return 3; }
};

class MomentumUpwAdvDiffElemKernel : public Kernel {
 public:
  MomentumUpwAdvDiffElemKernel(double alpha, double alphaUpw, double upwFactor, double hybridFactor,
                               bool useLimiter, double includeDivU = 0.0)
      : Kernel(NALU_KERNEL_MOMENTUM_UPW_ADV_DIFF) {
    opts.alpha = alpha;
    opts.alpha_upw = alphaUpw;
    opts.upw_factor = upwFactor;
    opts.hybrid_factor = hybridFactor;
    opts.use_limiter = useLimiter;
    opts.include_divu = includeDivU;
  }
  int numDof() const override { return 3; }
};

// TpetraLinearSystem on one GPU.
class LinearSystem {
 public:
  LinearSystem(Context& ctx, int numDof) : ctx_(ctx), numDof_(numDof) { nalu_solver_opts_default(&solverOpts); }
  void buildElemToNodeGraph() { ctx_.check(nalu_linsys_build_elem_graph(ctx_.get(), numDof_), "buildElemToNodeGraph"); }
  void finalizeLinearSystem() {}  // the CRS graph is complete after buildElemToNodeGraph
  void zeroSystem() { ctx_.check(nalu_linsys_zero(ctx_.get()), "zeroSystem"); }
  // whole element matrices of the given elements (additive)
  void sumInto(const std::vector<int64_t>& elems, const std::vector<double>& lhs, const std::vector<double>& rhs) {
    ctx_.check(nalu_linsys_sum_into(ctx_.get(), (int64_t)elems.size(), elems.data(), lhs.data(), rhs.data()),
               "sumInto");
  }
  void applyDirichletBCs(const std::vector<int32_t>& nodes, const std::vector<double>& bc,
                         const std::vector<double>& solution, unsigned beginPos, unsigned endPos) {
    ctx_.check(nalu_linsys_apply_dirichlet(ctx_.get(), (int64_t)nodes.size(), nodes.data(), (int)beginPos,
                                           (int)endPos, bc.data(), solution.data()),
               "applyDirichletBCs");
  }
  void resetRows(const std::vector<int32_t>& nodes, unsigned beginPos, unsigned endPos) {
    ctx_.check(nalu_linsys_reset_rows(ctx_.get(), (int64_t)nodes.size(), nodes.data(), (int)beginPos, (int)endPos),
               "resetRows");
  }
  void sumIntoDiagonal(int32_t node, int dof, double diag, double rhs) {
    ctx_.check(nalu_linsys_sum_into_diag(ctx_.get(), node, dof, diag, rhs), "sumInto(diag)");
  }
  void loadComplete() { ctx_.check(nalu_linsys_load_complete(ctx_.get()), "loadComplete"); }
  // returns the solver status (0 = converged), like TpetraLinearSystem::solve
  int solve() {
    nalu_solve_info info{};
    const int rc = nalu_solve(ctx_.get(), &solverOpts, &info);
    linearSolveIterations_ = info.iterations;
    linearResidual_ = info.true_rel_res;
    return rc;
  }
  std::vector<double> solution() const {
    int64_t n = 0;
    nalu_linsys_sizes(ctx_.get(), &n, nullptr, nullptr);
    std::vector<double> x((size_t)n);
    ctx_.check(nalu_solution_get(ctx_.get(), x.data(), 0), "solution");
    return x;
  }
  // the assembled values [nnz] and rhs [rows] (either may be null) and the
  // CRS graph (rowptr [rows + 1], colind [nnz]), in Tpetra row order
  void values(double* vals, double* rhs) const { ctx_.check(nalu_linsys_copy(ctx_.get(), vals, rhs, 0), "copy"); }
  void graph(int64_t* rowptr, int32_t* colind) const {
    ctx_.check(nalu_linsys_graph(ctx_.get(), rowptr, colind), "graph");
  }
  void sizes(int64_t* rows, int64_t* nnz) const { ctx_.check(nalu_linsys_sizes(ctx_.get(), rows, nnz, nullptr), "sizes"); }
  // writeToFile / writeSolutionToFile (src/TpetraLinearSystem.C:1967-2117): MatrixMarket dumps
  void writeToFile(const char* base) { ctx_.check(nalu_linsys_write_system(ctx_.get(), base), "writeToFile"); }
  void writeSolutionToFile(const char* base) {
    ctx_.check(nalu_linsys_write_solution(ctx_.get(), base), "writeSolutionToFile");
  }
  int numDof() const { return numDof_; }
  int linearSolveIterations() const { return linearSolveIterations_; }
  double linearResidual() const { return linearResidual_; }
  Context& context() { return ctx_; }
  nalu_solver_opts solverOpts;

 private:
  Context& ctx_;
  int numDof_;
  int linearSolveIterations_ = 0;
  double linearResidual_ = 0.0;
};

// Element loop driver: each active kernel runs as one fused device pass.
class AssembleElemSolverAlgorithm {
 public:
  explicit AssembleElemSolverAlgorithm(LinearSystem& ls) : linsys_(ls) {}
  void initialize_connectivity() { linsys_.buildElemToNodeGraph(); }
  void execute(const TimeIntegrator& ti = TimeIntegrator()) {
    for (Kernel* k : activeKernels_) {
      if (k->numDof() != linsys_.numDof()) throw Error(NALU_ERR_STATE, "kernel numDof != linear system numDof");
      k->setup(ti);
      linsys_.context().check(nalu_assemble(linsys_.context().get(), k->id(), &k->opts), "execute");
    }
  }
  std::vector<Kernel*> activeKernels_;

 private:
  LinearSystem& linsys_;
};

// Face (and face-element) kernels of one boundary part
// (src/kernel/ContinuityInflowElemKernel.C, ContinuityOpenElemKernel.C)
class FaceKernel {
 public:
  explicit FaceKernel(int id) : id_(id) { nalu_assemble_opts_default(&opts); }
  virtual ~FaceKernel() = default;
  virtual void setup(const TimeIntegrator& ti) { opts.proj_time_scale = ti.dt / ti.gamma1; }
  int id() const { return id_; }
  nalu_assemble_opts opts;

 private:
  int id_;
};

class ContinuityInflowElemKernel : public FaceKernel {
 public:
  explicit ContinuityInflowElemKernel(bool useShifted = false) : FaceKernel(NALU_FACE_CONTINUITY_INFLOW) {
    opts.shift_mdot = useShifted;
  }
};

class ContinuityOpenElemKernel : public FaceKernel {
 public:
  ContinuityOpenElemKernel(bool shiftMdot = false, bool shiftPoisson = false, bool reducedSens = false)
      : FaceKernel(NALU_FACE_CONTINUITY_OPEN) {
    opts.shift_mdot = shiftMdot;
    opts.shift_poisson = shiftPoisson;
    opts.reduced_sens = reducedSens || shiftPoisson;
  }
};

// AssembleFaceElemSolverAlgorithm over one side set
class AssembleFaceElemSolverAlgorithm {
 public:
  AssembleFaceElemSolverAlgorithm(LinearSystem& ls, int sideSet) : linsys_(ls), set_(sideSet) {}
  void execute(const TimeIntegrator& ti = TimeIntegrator()) {
    if (linsys_.numDof() != 1) throw Error(NALU_ERR_STATE, "face kernels need a numDof 1 system");
    for (FaceKernel* k : activeKernels_) {
      k->setup(ti);
      linsys_.context().check(nalu_assemble_faces(linsys_.context().get(), set_, k->id(), &k->opts), "execute");
    }
  }
  std::vector<FaceKernel*> activeKernels_;

 private:
  LinearSystem& linsys_;
  int set_;
};

// ComputeMdotElemAlgorithm (src/ComputeMdotElemAlgorithm.C:85-250): the SCS
// mass flow rates (NALU_FIELD_MDOT_SCS) from density, velocity_rtm, pressure
// and dpdx; tau = dt / gamma1.  arith: NALU_ARITH_FP64 or NALU_ARITH_DF64.
class ComputeMdotElemAlgorithm {
 public:
  ComputeMdotElemAlgorithm(Context& ctx, bool shiftMdot = false, bool shiftPoisson = false, int arith = NALU_ARITH_FP64)
      : ctx_(ctx) {
    nalu_assemble_opts_default(&opts);
    opts.shift_mdot = shiftMdot;
    opts.shift_poisson = shiftPoisson;
    opts.arith = arith;
  }
  void execute(const TimeIntegrator& ti = TimeIntegrator()) {
    opts.proj_time_scale = ti.dt / ti.gamma1;
    ctx_.check(nalu_compute_mdot(ctx_.get(), &opts), "ComputeMdotElemAlgorithm::execute");
  }
  nalu_assemble_opts opts;

 private:
  Context& ctx_;
};

// AssembleNodalGradElemAlgorithm / AssembleNodalGradUElemAlgorithm
// (src/AssembleNodalGradElemAlgorithm.C): the element part of the projected
// nodal gradient of src into dst (zeroed first; needs the dual nodal volume),
// then, per boundary side set, AssembleNodalGradBoundaryAlgorithm
// (src/AssembleNodalGradBoundaryAlgorithm.C:75-153) adds the face closure.
class AssembleNodalGradElemAlgorithm {
 public:
  AssembleNodalGradElemAlgorithm(Context& ctx, nalu_field src, nalu_field dst, bool shifted = false,
                                 int arith = NALU_ARITH_FP64)
      : ctx_(ctx), src_(src), dst_(dst), shifted_(shifted), arith_(arith) {}
  void execute() {
    ctx_.check(nalu_compute_nodal_gradient(ctx_.get(), src_, dst_, shifted_ ? 1 : 0, arith_),
               "AssembleNodalGradElemAlgorithm::execute");
    for (int set : boundarySets_)
      ctx_.check(nalu_nodal_gradient_boundary(ctx_.get(), set, src_, dst_, shifted_ ? 1 : 0),
                 "AssembleNodalGradBoundaryAlgorithm::execute");
  }
  std::vector<int> boundarySets_;

 private:
  Context& ctx_;
  nalu_field src_, dst_;
  bool shifted_;
  int arith_;
};

}  // namespace nalu_gb300
#endif
