/*
 * nalu_gb300.h -- C ABI of the GB300 (sm_103a) Hex8 CVFEM assembly and
 * continuity-solve library.
 *
 * One opaque context = one CUDA device + one CUDA stream + one Hex8 mesh +
 * its nodal/element fields + one linear system (CRS matrix, rhs, solution).
 * Every function returns an int status (NALU_OK = 0, negative on error); no
 * C++ exception crosses this boundary.  nalu_last_error() gives the message
 * of the last failure on a context.  All pointers are plain host pointers
 * unless a function says "device".  Node arrays are in the caller's node
 * order; matrix rows/columns follow the reference's Tpetra numbering (nodes
 * ordered by global id, numDof consecutive dofs per node).
 *
 * Each entry point names the reference interface it replaces
 * (file:line within NaluCFD/Nalu).
 */
#ifndef NALU_GB300_H
#define NALU_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NALU_OK 0
#define NALU_ERR_ARG (-1)          /* bad argument (null pointer, size, enum) */
#define NALU_ERR_CUDA (-2)         /* CUDA runtime failure */
#define NALU_ERR_STATE (-3)        /* call out of order (e.g. assemble before graph) */
#define NALU_ERR_NEG_JACOBIAN (-4) /* an element has det(J) <= 0 at an integration point */
#define NALU_ERR_NONFINITE (-5)    /* NaN/Inf in assembled values or solver scalars */
#define NALU_ERR_CAPACITY (-6)     /* a graph row exceeds the supported length */
#define NALU_ERR_NOT_CONVERGED (-7)/* solver hit max iterations */
#define NALU_ERR_GRAPH (-8)        /* element entry not present in the CRS graph */
#define NALU_ERR_NO_DEVICE (-9)    /* no usable CUDA device */

typedef struct nalu_ctx nalu_ctx;

/* ---- context ----------------------------------------------------------- */
int nalu_create(int device, nalu_ctx** out);
int nalu_destroy(nalu_ctx* ctx);
const char* nalu_last_error(const nalu_ctx* ctx);
const char* nalu_status_string(int status);
/* the context's CUDA stream (cudaStream_t), for callers that overlap work */
int nalu_get_stream(nalu_ctx* ctx, void** stream);
int nalu_synchronize(nalu_ctx* ctx);

/* ---- mesh (STK bulk data for one Hex8 block) ---------------------------
 * conn: [n_elems][8] 0-based node indices in the reference's Hex8 node order
 * (include/master_element/Hex8CVFEM.h); gid: node global ids (NULL => i+1),
 * which fix the row order exactly as TpetraLinearSystem::
 * beginLinearSystemConstruction does (src/TpetraLinearSystem.C:189-327);
 * coords: [n_nodes][3]. */
int nalu_mesh_create(nalu_ctx* ctx, int64_t n_nodes, int64_t n_elems, const int32_t* conn,
                     const int64_t* gid, const double* coords);

/* ---- fields (stk::mesh::field_data gathers, src/ScratchViews.C:408-483) -- */
enum nalu_field {
  NALU_FIELD_COORDINATES = 0,  /* [n][3] */
  NALU_FIELD_SCALAR_Q = 1,     /* [n]    ScalarDiffElemKernel scalarQ */
  NALU_FIELD_DIFF_COEFF = 2,   /* [n]    ScalarDiffElemKernel diffFluxCoeff */
  NALU_FIELD_VELOCITY = 3,     /* [n][3] */
  NALU_FIELD_VELOCITY_RTM = 4, /* [n][3] */
  NALU_FIELD_DENSITY = 5,      /* [n]    */
  NALU_FIELD_PRESSURE = 6,     /* [n]    */
  NALU_FIELD_DPDX = 7,         /* [n][3] Gpdx */
  NALU_FIELD_VISCOSITY = 8,    /* [n]    */
  NALU_FIELD_DUDX = 9,         /* [n][3][3] Gju */
  NALU_FIELD_MDOT_SCS = 10,    /* element field [E][12] mass_flow_rate_scs */
  NALU_FIELD_DUAL_VOLUME = 11, /* [n]    dual_nodal_volume (nalu_compute_dual_volume) */
  /* older time levels of the two-/three-state fields (stk::mesh::StateN /
   * StateNM1); DENSITY and VELOCITY above are state N+1.  The mass kernels
   * read N-1 as N when N-1 is not set (a two-state field). */
  NALU_FIELD_DENSITY_N = 12,    /* [n]    */
  NALU_FIELD_DENSITY_NM1 = 13,  /* [n]    */
  NALU_FIELD_VELOCITY_N = 14,   /* [n][3] */
  NALU_FIELD_VELOCITY_NM1 = 15, /* [n][3] */
  /* boundary-condition fields of the face kernels */
  NALU_FIELD_PRESSURE_BC = 16,  /* [n]    pressure_bc (open boundary) */
  NALU_FIELD_VELOCITY_BC = 17,  /* [n][3] cont_velocity_bc (inflow boundary) */
  NALU_FIELD_COUNT = 18
};
/* copy a field in (host or device source, caller node order) */
int nalu_field_set(nalu_ctx* ctx, int field, const double* src, int64_t count, int src_is_device);
int nalu_field_get(nalu_ctx* ctx, int field, double* dst, int64_t count, int dst_is_device);
/* The same upload without joining the compute stream: the copy (from host
 * memory, pinned with nalu_host_alloc for it to be asynchronous) runs on an
 * upload stream into a second buffer of the field, and the next call that
 * reads fields (assembly, mdot, gradients, face kernels, field_get, ...) waits
 * for it in stream order and swaps it in.  The upload of step k+1 so overlaps
 * the assembly of step k.  The host buffer must stay unchanged until then
 * (nalu_synchronize waits for every stream).  No reference counterpart (STK
 * fields live on the host). */
int nalu_field_set_async(nalu_ctx* ctx, int field, const double* src, int64_t count);

/* ---- linear system (LinearSystem, include/LinearSystem.h:39-167) -------- */
/* buildElemToNodeGraph + finalizeLinearSystem (src/TpetraLinearSystem.C:430-435,
 * 1256-1353): CRS graph with rows = numDof x nodes (Tpetra row order) */
int nalu_linsys_build_elem_graph(nalu_ctx* ctx, int num_dof);
int nalu_linsys_sizes(nalu_ctx* ctx, int64_t* n_rows, int64_t* nnz, int* num_dof);
/* copy the CRS graph out (rowptr [n_rows+1] as size_t-compatible int64, colind int32) */
int nalu_linsys_graph(nalu_ctx* ctx, int64_t* rowptr, int32_t* colind);
/* device pointers of the system arrays (valid until the next graph build) */
int nalu_linsys_device_arrays(nalu_ctx* ctx, const int64_t** rowptr, const int32_t** colind,
                              double** values, double** rhs, double** solution);
/* zeroSystem (src/TpetraLinearSystem.C:1355-1373) */
int nalu_linsys_zero(nalu_ctx* ctx);
/* sumInto of whole element matrices (src/TpetraLinearSystem.C:1458-1522):
 * additive; lhs [n][(8 numDof)^2] row-major, rhs [n][8 numDof] */
int nalu_linsys_sum_into(nalu_ctx* ctx, int64_t n, const int64_t* elem_ids, const double* lhs,
                         const double* rhs);
/* applyDirichletBCs (src/TpetraLinearSystem.C:1579-1653): for node rows
 * dofs [begin,end): row -> unit diagonal, rhs = bc - solution
 * (bc, solution: [n_nodes_bc][numDof] in the order of node_idx) */
int nalu_linsys_apply_dirichlet(nalu_ctx* ctx, int64_t n, const int32_t* node_idx, int begin_dof,
                                int end_dof, const double* bc, const double* solution);
/* resetRows (src/TpetraLinearSystem.C:1707-1755): rows and rhs -> 0 */
int nalu_linsys_reset_rows(nalu_ctx* ctx, int64_t n, const int32_t* node_idx, int begin_dof,
                           int end_dof);
/* 1x1 sumInto on a diagonal (FixPressureAtNodeAlgorithm, src/FixPressureAtNodeAlgorithm.C:53-80) */
int nalu_linsys_sum_into_diag(nalu_ctx* ctx, int32_t node_idx, int dof, double diag, double rhs);
/* loadComplete (src/TpetraLinearSystem.C:1757-1778): one rank, no export */
int nalu_linsys_load_complete(nalu_ctx* ctx);
/* copy values [nnz] and rhs [n_rows] out (either may be NULL) */
int nalu_linsys_copy(nalu_ctx* ctx, double* values, double* rhs, int dst_is_device);
/* The same download without blocking the next assembly: the current values
 * and rhs are snapshotted on the device (stream order) and sent to the host
 * on a second stream, so the transfer overlaps whatever is queued next
 * (field uploads, zeroSystem, assembly).  values / rhs are host buffers,
 * pinned (nalu_host_alloc) for the transfer to be asynchronous; they hold the
 * result after nalu_linsys_copy_wait or nalu_synchronize.  Two snapshots
 * are used in turn: a call waits on the device only for the download two
 * calls back, so consecutive downloads run back to back.  Downloads complete
 * in call order; calls that share host buffers leave the last call's result
 * there.  No reference counterpart (Tpetra's matrix lives on the host). */
int nalu_linsys_copy_async(nalu_ctx* ctx, double* values, double* rhs);
int nalu_linsys_copy_wait(nalu_ctx* ctx);

/* MatrixMarket dumps (TpetraLinearSystem::writeToFile / writeSolutionToFile,
 * src/TpetraLinearSystem.C:1967-2117): <base>-O-<count>.mm.1 (coordinate real
 * general, 1-based global ids ndof (gid - 1) + idof + 1) and .rhs.1 (array);
 * write_solution writes .sln.1 and advances count, as the reference's solve
 * does after the solver returns (:1794-1817) */
int nalu_linsys_write_system(nalu_ctx* ctx, const char* base);
int nalu_linsys_write_solution(nalu_ctx* ctx, const char* base);

/* ---- assembly (AssembleElemSolverAlgorithm::execute + Kernel::execute) --- */
enum nalu_kernel {
  NALU_KERNEL_SCALAR_DIFF = 0,        /* src/kernel/ScalarDiffElemKernel.C */
  NALU_KERNEL_CONTINUITY_ADV = 1,     /* src/kernel/ContinuityAdvElemKernel.C */
  NALU_KERNEL_MOMENTUM_ADV_DIFF = 2,  /* src/kernel/MomentumAdvDiffElemKernel.C */
  NALU_KERNEL_MOMENTUM_UPW_ADV_DIFF = 3, /* src/kernel/MomentumUpwAdvDiffElemKernel.C */
  /* time terms (gamma1 phi^{n+1} + gamma2 phi^n + gamma3 phi^{n-1}) / dt over
   * the sub-control volumes; dt and the gammas come from the opts below */
  NALU_KERNEL_CONTINUITY_MASS = 4,  /* src/kernel/ContinuityMassElemKernel.C (rhs only) */
  NALU_KERNEL_MOMENTUM_MASS = 5     /* src/kernel/MomentumMassElemKernel.C (reads DPDX as Gjp) */
};
enum nalu_scatter {
  NALU_SCATTER_AUTO = 0,    /* autotuned choice, cached per context */
  NALU_SCATTER_ATOMIC = 1,  /* FP64 atomics into the CRS values */
  NALU_SCATTER_COLOURED = 2 /* element colouring, plain read-modify-write (deterministic) */
};
/* solution options that change the kernels (src/SolutionOptions.C) and the
 * time-integrator scale (ContinuityAdvElemKernel::setup, :79-84) */
typedef struct nalu_assemble_opts {
  int shifted_grad_op;      /* get_shifted_grad_op(dof) */
  int shift_mdot;           /* cvfemShiftMdot_ */
  int shift_poisson;        /* get_shifted_grad_op("pressure") */
  int reduced_sens;         /* cvfemReducedSensPoisson_ */
  int skew_symmetric;       /* get_skew_symmetric(dof) */
  int use_limiter;          /* primitive_uses_limiter(dof) */
  double proj_time_scale;   /* dt / gamma1 */
  double include_divu;      /* includeDivU_ */
  double alpha;             /* get_alpha_factor */
  double alpha_upw;         /* get_alpha_upw_factor */
  double upw_factor;        /* get_upw_factor */
  double hybrid_factor;     /* get_hybrid_factor (classic Peclet function, A = 5) */
  int scatter;              /* enum nalu_scatter */
  int arith;                /* enum nalu_arith (scalar kernels) */
  int lumped_mass;          /* mass kernels: lumped (shifted_shape_fcn) */
  int balanced_force;       /* MomentumMass: solnOpts.balancedForce_ (Gjp scaled by rho) */
  double dt;                /* TimeIntegrator::get_time_step, > 0 for the mass kernels */
  double gamma1;            /* TimeIntegrator::get_gamma1 (default 1, BDF1) */
  double gamma2;            /* get_gamma2 (default -1) */
  double gamma3;            /* get_gamma3 (default 0) */
  int schedule;             /* enum nalu_schedule (double-float scalar kernels) */
  int reserved[3];
} nalu_assemble_opts;
/* arithmetic of the element math; inputs, outputs, the CRS scatter and the
 * residual's -lhs.q term stay FP64 in both modes */
enum nalu_arith {
  NALU_ARITH_FP64 = 0,  /* FP64 throughout */
  NALU_ARITH_DF64 = 1   /* double-float (hi+lo FP32 pair, ~48-bit) on the FP32 pipes */
};
/* how the double-float scalar kernels (ARITH_DF64, ScalarDiff / ContinuityAdv)
 * map elements to threads; AUTO times every schedule x scatter pair on the
 * first call of a context and kernel and keeps the fastest
 * (nalu_assemble_tuning reports the table) */
enum nalu_schedule {
  NALU_SCHEDULE_AUTO = 0,
  NALU_SCHEDULE_ELEMENT = 1, /* one thread per element, 64-thread blocks */
  NALU_SCHEDULE_IP8 = 2,     /* one thread per (element, SCS ip), 8 elements per block */
  NALU_SCHEDULE_IP16 = 3     /* the same, 16 elements per block, tighter register budget */
};
void nalu_assemble_opts_default(nalu_assemble_opts* opts);
/* run one element kernel over all elements and sum into the system */
int nalu_assemble(nalu_ctx* ctx, int kernel, const nalu_assemble_opts* opts);
/* mock capture (unit_tests/UnitTestLinearSystem.h:39-55): element matrix and
 * rhs of element `elem`, without touching the system */
int nalu_capture_element(nalu_ctx* ctx, int kernel, const nalu_assemble_opts* opts, int64_t elem,
                         double* lhs, double* rhs);
/* ComputeMdotElemAlgorithm (src/ComputeMdotElemAlgorithm.C:85-250):
 * fills NALU_FIELD_MDOT_SCS from density, velocity_rtm, pressure, dpdx */
int nalu_compute_mdot(nalu_ctx* ctx, const nalu_assemble_opts* opts);

/* ---- nodal geometry and gradients --------------------------------------- */
/* dual_nodal_volume: ComputeGeometryInteriorAlgorithm
 * (src/ComputeGeometryInteriorAlgorithm.C) sums the eight sub-control volumes
 * of HexSCV::determinant (src/master_element/Hex8CVFEM.C:149-180) into their
 * nodes; fills NALU_FIELD_DUAL_VOLUME from the coordinates */
int nalu_compute_dual_volume(nalu_ctx* ctx);
/* HexSCV::determinant of one element: vol[8] (host) */
int nalu_capture_scv_volumes(nalu_ctx* ctx, int64_t elem, double* vol);
/* Element part of the projected nodal gradient (AssembleNodalGradElemAlgorithm,
 * src/AssembleNodalGradElemAlgorithm.C; AssembleNodalGradUElemAlgorithm for a
 * vector field): dst = sum over SCS of q_ip A / V, zeroed first.  src is a
 * scalar field (dst 3 components, e.g. PRESSURE -> DPDX) or a 3-vector field
 * (dst 9 components, d src_i / dx_j at 3 i + j, e.g. VELOCITY -> DUDX).
 * Needs NALU_FIELD_DUAL_VOLUME.  The boundary-face closure
 * (AssembleNodalGradBoundaryAlgorithm) is not part of this call.
 * shifted: shifted_shape_fcn at the ips.  arith: NALU_ARITH_FP64, or
 * NALU_ARITH_DF64 (areas and sums as FP32 pairs, about 48 bits). */
int nalu_compute_nodal_gradient(nalu_ctx* ctx, int src_field, int dst_field, int shifted, int arith);

/* ---- Hex8 master element, batched (src/master_element/Hex8CVFEM.C) --------
 * MasterElement calls for nelem elements at once, evaluated on the device:
 * coords [nelem][8][3] in the element's node order; outputs per element in
 * the reference's layouts.  on_device: the arrays are device pointers (else
 * host arrays, copied).  The grad ops return NALU_ERR_NEG_JACOBIAN when some
 * element has det(J) <= 0 at one of its points (outputs still written). */
/* HexSCS::determinant (:547-580): areav [nelem][12][3] */
int nalu_hex_scs_determinant(nalu_ctx* ctx, int64_t nelem, const double* coords, double* areav, int on_device);
/* HexSCS::grad_op / shifted_grad_op (:523-541, generic_grad_op):
 * gradop, deriv [nelem][12][8][3] (deriv may be NULL) */
int nalu_hex_scs_grad_op(nalu_ctx* ctx, int64_t nelem, const double* coords, int shifted, double* gradop,
                         double* deriv, int on_device);
/* HexSCV::grad_op / shifted_grad_op (:185-232): [nelem][8][8][3] */
int nalu_hex_scv_grad_op(nalu_ctx* ctx, int64_t nelem, const double* coords, int shifted, double* gradop,
                         double* deriv, int on_device);
/* HexSCV::determinant (:149-180): vol [nelem][8] */
int nalu_hex_scv_determinant(nalu_ctx* ctx, int64_t nelem, const double* coords, double* vol, int on_device);
/* HexSCS::face_grad_op / shifted_face_grad_op (:668-684) at the exposed-face
 * ips of side side[e] of each element: gradop [nelem][4][8][3] */
int nalu_hex_face_grad_op(nalu_ctx* ctx, int64_t nelem, const int32_t* side, const double* coords, int shifted,
                          double* gradop, int on_device);
/* constant tables: HexSCS::adjacentNodes (lrscv_, int[24]), HexSCS::shape_fcn /
 * shifted_shape_fcn ([12][8]), HexSCS::side_node_ordinals (int[4]) */
void nalu_hex_scs_adjacent_nodes(int32_t* lrscv);
void nalu_hex_scs_shape_fcn(int shifted, double* shp);
void nalu_hex_side_node_ordinals(int side, int32_t* nodes4);

/* ---- boundary faces ------------------------------------------------------
 * A side set is a list of element sides, as the mesh's boundary parts hold
 * them: face k is side side[k] of element elem[k], with the Hex8 side
 * numbering of HexSCS::sideNodeOrdinals_ (src/master_element/Hex8CVFEM.C:
 * 415-422): 0 {0,1,5,4}, 1 {1,2,6,5}, 2 {2,3,7,6}, 3 {0,4,7,3}, 4 {0,3,2,1},
 * 5 {4,5,6,7} (outward normals).  Face ip k sits at side node k
 * (Quad3DSCS / HexSCS::ipNodeMap(side)). */
#define NALU_MAX_FACE_SETS 16
int nalu_faceset_define(nalu_ctx* ctx, int set, int64_t n, const int64_t* elem, const int32_t* side);
/* the mesh's exposed sides (sides of exactly one element) as face set `set`,
 * ordered by element then side; n_faces (may be NULL) receives the count */
int nalu_faceset_skin(nalu_ctx* ctx, int set, int64_t* n_faces);
int nalu_faceset_size(nalu_ctx* ctx, int set, int64_t* n_faces);
int nalu_faceset_get(nalu_ctx* ctx, int set, int64_t* elem, int32_t* side);
/* dynamic_pressure at the face ips, [n][4] host (ContinuityOpen's pbc offset);
 * NULL clears it to zero */
int nalu_faceset_dynamic_pressure(nalu_ctx* ctx, int set, const double* dynp);
/* exposed_area_vector (ComputeGeometryBoundaryAlgorithm, Quad3DSCS::determinant
 * = quad3d_scs_det, src/master_element/MasterElementWork.F:1467-1590) of the
 * set's faces: area [n][4][3] (host), ip k at side node k */
int nalu_faceset_exposed_area(nalu_ctx* ctx, int set, double* area);
/* boundary closure of the projected nodal gradient over one side set
 * (AssembleNodalGradBoundaryAlgorithm, src/AssembleNodalGradBoundaryAlgorithm.C:
 * 75-153): dst[nn] += q_ip A_ip / V_nn, ADDED to a gradient made by
 * nalu_compute_nodal_gradient with the same fields */
int nalu_nodal_gradient_boundary(nalu_ctx* ctx, int set, int src_field, int dst_field, int shifted);
enum nalu_face_kernel {
  /* src/kernel/ContinuityInflowElemKernel.C: rhs -= rho u_bc . A / tau at
   * the face nodes; reads DENSITY, VELOCITY_BC; shift_mdot selects the
   * shifted face shape functions; tau = opts.proj_time_scale */
  NALU_FACE_CONTINUITY_INFLOW = 0,
  /* src/kernel/ContinuityOpenElemKernel.C: face-element kernel with the
   * penalty 2 tau L^-1 (p - p_bc) |A| and the element pressure gradient at
   * the exposed-face ips (HexSCS::face_grad_op); reads PRESSURE, PRESSURE_BC,
   * DENSITY, VELOCITY, DPDX and the set's dynamic pressure; options
   * shift_poisson, reduced_sens, shift_mdot as for ContinuityAdv */
  NALU_FACE_CONTINUITY_OPEN = 1
};
/* run a face kernel over a side set and sum into the (numDof 1) system,
 * rows of the face nodes, columns of the element's nodes */
int nalu_assemble_faces(nalu_ctx* ctx, int set, int face_kernel, const nalu_assemble_opts* opts);
/* face `face` of the set in mock-capture form: lhs [8][8], rhs [8] in the
 * element's node order (rows of the side's four nodes filled) */
int nalu_capture_face(nalu_ctx* ctx, int set, int face_kernel, const nalu_assemble_opts* opts, int64_t face,
                      double* lhs, double* rhs);

/* ---- linear solve (TpetraLinearSolver::solve, src/LinearSolver.C:183-232) */
enum nalu_solver_method {
  NALU_SOLVER_CG = 0,       /* preconditioned CG */
  NALU_SOLVER_GMRES = 1     /* right-preconditioned restarted GMRES(m) */
};
enum nalu_precond {
  NALU_PRECOND_NONE = 0,
  NALU_PRECOND_JACOBI = 1,    /* Ifpack2 RELAXATION Jacobi, one sweep */
  NALU_PRECOND_CHEBYSHEV = 2, /* Chebyshev polynomial in D^-1 A */
  NALU_PRECOND_LEARNED = 3,   /* learned 27-point stencil (below) in flexible CG;
                                 scalar systems, FP64, needs weights */
  /* aggregation multigrid in flexible CG, the GPU counterpart of the MueLu
   * choice (src/LinearSolverConfig.C:92-96): pairwise aggregation on the
   * strong couplings, Galerkin coarse operators, V- or K-cycle, FP32 cycle inside
   * FP64 flexible CG; scalar systems, FP64 precision.  MULTILEVEL smooths with
   * damped Jacobi on every level; LEARNED_MULTILEVEL with the learned
   * 27-point stencil on the fine level (needs weights) */
  NALU_PRECOND_MULTILEVEL = 4,
  NALU_PRECOND_LEARNED_MULTILEVEL = 5
};
enum nalu_precision {
  NALU_PRECISION_FP64 = 0,          /* everything FP64 */
  NALU_PRECISION_FP32_INNER_IR = 1  /* FP32 inner solver, FP64 iterative refinement */
};
typedef struct nalu_solver_opts {
  int method;        /* enum nalu_solver_method */
  int precond;       /* enum nalu_precond */
  int precision;     /* enum nalu_precision */
  int max_iters;
  int restart;       /* GMRES kspace */
  int cheb_degree;
  int check_every;   /* residual checks every N iterations (host sync) */
  int x0_zero;       /* 1: start from 0 (else from the current solution) */
  double tol;        /* stop on true ||b - A x|| / ||b|| <= tol */
  double inner_tol;  /* inner tolerance for iterative refinement */
  int stall_window;  /* learned FCG stalls when the residual norm has no new
                        minimum for max(stall_window, 10 x the iterations taken
                        to reach the current minimum); Chebyshev-Jacobi PCG
                        then finishes (default 20) */
  int learned_probe; /* learned FCG: 1 (default) opens with a short run of each
                        of Jacobi-CG and the learned FCG and keeps the faster per
                        unit of device time, and bounds the learned FCG by twice
                        the iterations the probe predicts for Jacobi-CG; 0 runs
                        the learned FCG with the stall fallback only */
  int ml_kcycle_levels; /* multilevel preconditioners: coarse levels 1..k solve
                           their coarse problem by K-cycle (two flexible CG steps),
                           deeper ones by V-cycle; 0 (default): V-cycle throughout
                           (the fastest on the continuity systems measured) */
  int ml_learned_sweeps; /* NALU_PRECOND_LEARNED_MULTILEVEL: the level-0 sweeps that
                            use the learned smoother, bit 0 pre-smoothing, bit 1
                            post-smoothing (the other sweeps: damped Jacobi);
                            0 (default): both, a symmetric cycle (one sweep is
                            faster on some systems, 83.7 against 92.4 ms at
                            128^3, but the cycle is then unsymmetric and
                            converged far slower on others) */
  int reserved[2];
} nalu_solver_opts;
typedef struct nalu_solve_info {
  int iterations;        /* inner iterations in total */
  int outer_iterations;  /* refinement steps (1 for plain FP64) */
  int status;
  double true_rel_res;   /* FP64 ||b - A x|| / ||b|| */
  double seconds;        /* wall time of the whole call, set-up included */
  int fallback;          /* learned FCG: 0 it finished the solve; 1 it stalled or broke
                            down and Chebyshev-Jacobi PCG (batched: Jacobi-CG)
                            finished; 2 Jacobi-CG finished, chosen by the opening
                            probe (compared per unit of device time; batched: also
                            a problem with too few iterations left to try the
                            learned one, or whose batch's first trial lost) or
                            because the learned FCG used twice the iterations the
                            probe predicts for Jacobi-CG */
  int learned_iterations;/* iterations spent in the learned FCG (probe included);
                            iterations counts the probe runs too */
  double setup_seconds;  /* learned preconditioner set-up (MLP stencil + SELL values) */
  double probe_rate_jacobi;  /* opening probe, ln(residual reduction) per ms of */
  double probe_rate_learned; /* iterations (negative; 0 when no probe ran) */
} nalu_solve_info;
void nalu_solver_opts_default(nalu_solver_opts* opts);
/* solve A x = rhs into the context's solution vector */
int nalu_solve(nalu_ctx* ctx, const nalu_solver_opts* opts, nalu_solve_info* info);
/* copy the solution [n_rows] out */
int nalu_solution_get(nalu_ctx* ctx, double* x, int dst_is_device);
int nalu_solution_set(nalu_ctx* ctx, const double* x, int src_is_device);
/* y = A x with the context's matrix (FP64), host or device vectors */
int nalu_spmv(nalu_ctx* ctx, const double* x, double* y, int is_device);

/* ---- batches of independent meshes ------------------------------------- */
/* Declare that the context's mesh is a union of n independent problems:
 * problem k owns the nodes [node_offsets[k], node_offsets[k+1]) in Tpetra row
 * order (give the meshes ascending global ids problem by problem).  Assembly
 * stays one launch over all elements (the graph is block diagonal); the
 * batched solve below keeps separate scalars and a separate stop test per
 * problem.  No reference counterpart: Nalu solves one system per rank. */
int nalu_set_problems(nalu_ctx* ctx, int n, const int64_t* node_offsets);
/* Jacobi-preconditioned CG on every problem at once (per-problem alpha/beta
 * and convergence; CUDA-graph chunks of tile kernels over the union matrix);
 * infos[k] receives problem k's iterations and true FP64 relative residual.
 * With NALU_PRECOND_LEARNED a problem changes method in place between chunks,
 * without a restart of the others or a discarded iteration: with the probe on,
 * every problem opens with Jacobi-CG; only problems with many predicted
 * iterations left are candidates, and the learned preconditioner is set up
 * (rows of that problem only) and tried on the largest one first; the others
 * follow only if it beats its own Jacobi-CG rate per unit of device time.
 * With NALU_PRECOND_MULTILEVEL every problem runs flexible CG preconditioned by
 * one aggregation-multigrid hierarchy of the union (block diagonal: each
 * problem coarsens on its own and keeps its own dense coarsest block). */
int nalu_solve_batched(nalu_ctx* ctx, const nalu_solver_opts* opts, nalu_solve_info* infos);
/* Rows per tile of the batched solve: times tiles of 256, 512, 1024 and 2048
 * rows over `iterations` (<= 0: 100) iterations of the batched Jacobi-CG from
 * zero (device time; the context's solution is overwritten) and keeps the
 * fastest for later nalu_solve_batched calls (default before tuning: 1024).
 * tile_rows: the choice; ms_per_iteration [4]: each candidate's time (either
 * may be NULL). */
int nalu_batch_autotune(nalu_ctx* ctx, int iterations, int* tile_rows, double* ms_per_iteration);

/* ---- learned preconditioner -------------------------------------------- */
/* No reference counterpart: Nalu preconditions with Ifpack2/MueLu
 * (src/LinearSolver.C:98-106).  A per-node MLP, 108 -> 64 -> 64 -> 64 -> 1
 * with GELU (tanh form), reads 27 x 4 features of the node's 27-point
 * neighbourhood (slot s = 9(dz+1) + 3(dy+1) + (dx+1) of the element-local
 * offset): [0,27) residual / its RMS over the patch, [27,54) a_ij / a_ii,
 * [54,81) neighbour mask, [81,108) a_jj / a_ii.  The correction is
 * z_i = (r_i + rms_i * mlp_i) / a_ii.  At solve set-up the MLP is evaluated
 * on the 27 unit-impulse residuals of every node (BF16 tensor-core kernel),
 * which gives a 27-point stencil C; the preconditioner is the symmetric part
 * of D^-1 (I + C) on the sparsity of A, its off-diagonals scaled symmetrically
 * so that D^1/2 M D^1/2 is diagonally dominant (M is then positive definite).
 * Parameters (FP32, NALU_LEARNED_PARAMS): W1[64][108], b1[64], W2[64][64],
 * b2[64], W3[64][64], b3[64], w4[64], b4. */
#define NALU_LEARNED_PARAMS 15361
/* deterministic initialisation: hidden layers U(-1/sqrt(fan_in), +), output 0
 * (an untrained network is exactly Jacobi) */
int nalu_learned_init(nalu_ctx* ctx, uint64_t seed);
int nalu_learned_set_weights(nalu_ctx* ctx, const float* params, int64_t n);
int nalu_learned_get_weights(nalu_ctx* ctx, float* params, int64_t n);
/* Training pairs from plain Jacobi-PCG on the context's scalar system with
 * n_rhs seeded N(0,1) right-hand sides: the first search direction
 * p0 = D^-1 b and its image q0 = A p0 are an exact (residual, error) pair.
 * n_samples random non-identity rows, spread over the right-hand sides:
 * static_feats [n][81] (features 27..107), resid_feats [n][27] (q0 over the
 * patch / its RMS), targets [n] (p0_i a_ii / RMS), rows [n] (the row of each
 * sample; may be NULL).  *n_out <= n_samples
 * (rows whose patch residual is 0 are skipped).  Host arrays. */
int nalu_learned_harvest(nalu_ctx* ctx, int n_rhs, uint64_t seed, int64_t n_samples, float* static_feats,
                         float* resid_feats, float* targets, int64_t* rows /* [n] or NULL */, int64_t* n_out);
typedef struct nalu_train_opts {
  int epochs;          /* default 40 */
  int batch;           /* samples per Adam step, default 256, <= 1024 */
  double lr;           /* Adam step size, default 1e-3 (beta 0.9/0.999, eps 1e-8) */
  double val_fraction; /* held-out share of the samples, default 0.1 */
  uint64_t seed;       /* sample order */
  int precision;       /* enum nalu_train_precision, default NALU_TRAIN_BF16 */
  int reserved[3];
} nalu_train_opts;
enum nalu_train_precision {
  NALU_TRAIN_BF16 = 0, /* fused step on the tensor cores: BF16 weights and
                          activations, FP32 accumulation, FP32 master weights
                          and Adam; two launches per step, one graph per epoch */
  NALU_TRAIN_FP32 = 1  /* FP32 CUDA-core GEMMs (the exact path) */
};
void nalu_train_opts_default(nalu_train_opts* opts);
/* Adam on the mean squared error of the stencil form
 * pred = rf_13 + sum_s mask_s mlp(impulse_s, st) / sqrt(27) * rf_s against
 * the targets, on the GPU (opts->precision).  history [epochs][2]: train and
 * held-out MSE after each epoch (may be NULL). */
int nalu_learned_train(nalu_ctx* ctx, const float* static_feats, const float* resid_feats, const float* targets,
                       int64_t n, const nalu_train_opts* opts, float* history);
/* loss and gradient of that loss at the current weights over n <= 1024
 * samples (one batch); grad [NALU_LEARNED_PARAMS], host arrays */
int nalu_learned_gradient(nalu_ctx* ctx, const float* static_feats, const float* resid_feats, const float* targets,
                          int64_t n, float* grad, double* loss);
/* the same from the fused BF16 tensor-core training step (any n >= 1) */
int nalu_learned_gradient_bf16(nalu_ctx* ctx, const float* static_feats, const float* resid_feats,
                               const float* targets, int64_t n, float* grad, double* loss);
/* the stencil of the current scalar system: stencil [n_rows][27] (host),
 * mlp(impulse_s) / sqrt(27) per slot, 0 for missing neighbours and for
 * identity rows */
int nalu_learned_stencil(nalu_ctx* ctx, float* stencil);

/* Jacobi-preconditioned CG on a caller-owned CRS system, allocating no device
 * memory.  This entry point has no counterpart in the reference.  It is for
 * callers that cannot let a library call cudaMalloc: codes that hand their
 * whole device-memory budget to their own pool allocator, so an allocation
 * outside the pool would fail or fragment it, and time-step loops that must
 * not allocate because cudaMalloc/cudaFree can synchronise the device.
 * rowptr [n+1], colind, values, rhs and x are device pointers; x is
 * overwritten with the solution (the solve starts from zero, with rows that
 * are identity rows taking x = rhs), and the stop rule is the true FP64
 * residual ||rhs - A x|| / ||rhs|| <= tol, as nalu_solve.  The scratch
 * vectors live in one static device array sized for at most 262,144 rows
 * (about 10.8 MB, held by every GPU that loads the library until the
 * process exits); larger n returns NALU_ERR_CAPACITY.  The first call on a
 * device looks up that array's device address and must therefore come before
 * any stream capture on that device.  All calls on a device share the array:
 * calls that overlap on the GPU race on it.  stream may be NULL (the legacy
 * default stream); the call returns after the solve has finished.
 * *iterations is the number of CG steps that moved the iterate, counted on
 * the device (steps issued past convergence inside a 25-step chunk are
 * frozen and not counted). */
int nalu_pcg_jacobi_noalloc(int64_t n, const int64_t* rowptr, const int32_t* colind,
                            const double* values, const double* rhs, double* x, double tol,
                            int max_iters, int* iterations, double* true_rel_res, void* stream);

/* the autotuned choice of the double-float scalar kernel `kernel` in this
 * context: schedule, scatter and the measured device time (ms) of every
 * candidate, ms[(schedule - 1) * 2 + (scatter - 1)] (-1 where not timed);
 * NALU_ERR_STATE before the first tuned call.  No counterpart in the
 * reference (its element loop has one fixed schedule per execution space). */
int nalu_assemble_tuning(const nalu_ctx* ctx, int kernel, int* schedule, int* scatter, double* ms);

/* the level sizes of the last multilevel solve's hierarchy: returns the
 * number of levels (0 when none was built) and fills rows[l], nnz[l] for
 * l < max_levels (either may be NULL).  No counterpart in the reference. */
int nalu_multilevel_levels(const nalu_ctx* ctx, int max_levels, int64_t* rows, int64_t* nnz);

/* ---- measurement helpers ------------------------------------------------ */
/* number of this library's kernel launches since the context was created */
int64_t nalu_kernel_launch_count(const nalu_ctx* ctx);
/* device time (ms) of the last nalu_assemble's scatter+compute kernels,
 * measured with CUDA events on the context stream */
double nalu_last_assemble_ms(const nalu_ctx* ctx);
/* FP64 multiply-add throughput of this device, measured by a short kernel
 * (TFLOP/s, 2 flops per FMA) */
int nalu_probe_fp64_tflops(nalu_ctx* ctx, double* tflops);
/* CUDA events on the context stream: record into slot 0..63, and the device
 * time between two recorded slots (waits for the later one) */
int nalu_event_record(nalu_ctx* ctx, int slot);
int nalu_event_elapsed_ms(nalu_ctx* ctx, int slot_a, int slot_b, double* ms);
/* page-locked host memory for H2D/D2H staging */
int nalu_host_alloc(size_t bytes, void** ptr);
int nalu_host_free(void* ptr);
/* write `bytes` zeros through a scratch buffer larger than L2 (cache flush) */
int nalu_flush_l2(nalu_ctx* ctx, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif
