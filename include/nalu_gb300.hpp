// nalu_gb300.hpp -- C++ host interface over the C ABI (nalu_gb300.h),
// mirroring the reference classes a Nalu caller uses on this path:
//
//   LinearSystem                 include/LinearSystem.h:39-167 (TpetraLinearSystem)
//   Kernel + the four kernels    include/kernel/Kernel.h:95-125, src/kernel/*.C
//   AssembleElemSolverAlgorithm  include/AssembleElemSolverAlgorithm.h:38-112
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

 private:
  nalu_ctx* ctx_ = nullptr;
  int64_t n_nodes_ = 0;
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

}  // namespace nalu_gb300
#endif
