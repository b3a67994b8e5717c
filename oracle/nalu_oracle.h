/*
 * nalu_oracle.h -- CPU FP64 oracle for the Hex8 CVFEM assembly + continuity
 * solve path of NaluCFD/Nalu.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU path is
 * compared against (tests, the smoke check, and the CPU-baseline leg of the
 * benchmark).  Nothing in the product links or calls it.
 *
 * Every function restates the reference algorithm in plain C++ and keeps the
 * reference's floating-point operation order (the library is compiled with
 * -ffp-contract=off), so that on the same inputs it reproduces the reference's
 * own compiled master-element code bit for bit (pinned by the oracle tests
 * against the reference's Hex8CVFEM.C compiled in this container, and against
 * the golden vectors of the reference's unit tests).
 *
 * Layouts: coords [8][3], nodal vectors [8][3], element matrices row-major
 * [rows][cols], grad ops [ip][node][dim] -- the same as the reference's
 * SharedMemView layouts (include/ScratchViews.h).
 */
#ifndef NALU_ORACLE_H
#define NALU_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* --- master element (src/master_element/Hex8CVFEM.C) ------------------- */
void orc_hex_scs_tables(int* lrscv24, double* intg_loc36, double* intg_loc_shift36);
void orc_hex8_shape_fcn(int npts, const double* iso, double* shape /*[npts][8]*/);
void orc_hex8_derivative(int npts, const double* iso, double* deriv /*[npts][8][3]*/);
/* returns the number of integration points whose det(J) <= tiny */
int  orc_generic_grad_op(int npts, const double* deriv, const double* coords,
                         double* gradop /*[npts][8][3]*/, double* detj /*[npts] or NULL*/);
int  orc_hex_scs_grad_op(const double* coords, int shifted, double* gradop, double* deriv);
void orc_hex_scs_areav(const double* coords, double* areav /*[12][3]*/);
void orc_hex_scv_volume(const double* coords, double* volume /*[8]*/);
int  orc_hex_scv_grad_op(const double* coords, int shifted, double* gradop, double* deriv);

/* --- element kernels (src/kernel/*.C) ----------------------------------- */
void orc_scalar_diff_elem(const double* coords, const double* q, const double* diff_coeff,
                          int shifted_grad_op, double* lhs /*[8][8]*/, double* rhs /*[8]*/);
void orc_continuity_adv_elem(const double* coords, const double* velocity /*[8][3]*/,
                             const double* density, const double* pressure,
                             const double* gpdx /*[8][3]*/, double proj_time_scale,
                             int shift_mdot, int shift_poisson, int reduced_sens,
                             double* lhs, double* rhs);
void orc_momentum_adv_diff_elem(const double* coords, const double* velocity,
                                const double* viscosity, const double* mdot /*[12]*/,
                                double include_divu, int shifted_grad_op, int skew_symmetric,
                                double* lhs /*[24][24]*/, double* rhs /*[24]*/);
void orc_momentum_upw_adv_diff_elem(const double* coords, const double* velocity,
                                    const double* velocity_rtm, const double* density,
                                    const double* viscosity, const double* gju /*[8][3][3]*/,
                                    const double* mdot, double include_divu,
                                    int shifted_grad_op, int skew_symmetric,
                                    double alpha, double alpha_upw, double upw_factor,
                                    double hybrid_factor, int use_limiter,
                                    double* lhs, double* rhs);
void orc_mdot_elem(const double* coords, const double* density, const double* velocity_rtm,
                   const double* pressure, const double* gpdx, double proj_time_scale,
                   int shift_mdot, int shift_poisson, double* mdot /*[12]*/);

/* time terms (BDF: gamma1 phi^{n+1} + gamma2 phi^n + gamma3 phi^{n-1}) at the
 * eight sub-control volumes, ip i -> node i (HexSCV::ipNodeMap), shape
 * functions at the SCV centroids or, lumped, at the nodes (shifted_shape_fcn).
 * ContinuityMassElemKernel::execute (src/kernel/ContinuityMassElemKernel.C:84-120):
 * rhs only, lhs [8][8] zero. */
void orc_continuity_mass_elem(const double* coords, const double* rho_nm1, const double* rho_n,
                              const double* rho_np1, double dt, double gamma1, double gamma2, double gamma3,
                              int lumped, double* lhs /*[8][8]*/, double* rhs /*[8]*/);
/* MomentumMassElemKernel::execute (src/kernel/MomentumMassElemKernel.C:100-171);
 * gpdx [8][3] is Gjp, balanced_force selects densFac = rho^{n+1} */
void orc_momentum_mass_elem(const double* coords, const double* rho_nm1, const double* rho_n,
                            const double* rho_np1, const double* u_nm1, const double* u_n,
                            const double* u_np1, const double* gpdx, double dt, double gamma1,
                            double gamma2, double gamma3, int lumped, int balanced_force,
                            double* lhs /*[24][24]*/, double* rhs /*[24]*/);
/* serial element-order assembly of a mass kernel through the restated sumInto;
 * momentum selects MomentumMass (num_dof 3) over ContinuityMass (num_dof 1);
 * nodal fields in node-index order, u_* and gpdx [n][3] (NULL for continuity);
 * tp = {dt, gamma1, gamma2, gamma3, lumped, balanced_force} */
int orc_assemble_mass(int momentum, int64_t n_nodes, int64_t n_elems, const int32_t* conn,
                      const int32_t* node_lid, const double* coords, const double* rho_nm1,
                      const double* rho_n, const double* rho_np1, const double* u_nm1,
                      const double* u_n, const double* u_np1, const double* gpdx, const double* tp,
                      const int64_t* rowptr, const int32_t* colind, double* values, double* rhs);

/* --- linear system (src/TpetraLinearSystem.C) --------------------------- */
/* Restated buildElemToNodeGraph + finalizeLinearSystem on one rank.
 * node_gid may be NULL (gid = index+1).  Call with colind == NULL to get
 * n_rows and nnz; then call again with buffers of those sizes. */
int orc_graph_build(int64_t n_nodes, int64_t n_elems, const int32_t* conn,
                    const int64_t* node_gid, int num_dof,
                    int64_t* n_rows, int64_t* nnz, int64_t* rowptr, int32_t* colind,
                    int32_t* node_lid /*[n_nodes] out, may be NULL*/);

/* Serial element-order assembly through the restated sumInto.  kernel:
 * 0 ScalarDiff, 1 ContinuityAdv, 2 MomentumAdvDiff, 3 MomentumUpwAdvDiff.
 * fields are in node-index order; opts is a double[16] option block:
 *  [0] shifted_grad_op [1] shift_mdot [2] shift_poisson [3] reduced_sens
 *  [4] proj_time_scale [5] include_divu [6] skew_symmetric [7] alpha
 *  [8] alpha_upw [9] upw_factor [10] hybrid_factor [11] use_limiter */
int orc_assemble(int kernel, int64_t n_nodes, int64_t n_elems, const int32_t* conn,
                 const int32_t* node_lid, const double* coords,
                 const double* f_scalar /*q or pressure*/, const double* f_coeff /*k, density or viscosity*/,
                 const double* f_vec /*velocity*/, const double* f_vec2 /*Gpdx or velocity_rtm*/,
                 const double* f_rho /*density for upwind*/, const double* f_gju /*[n][9]*/,
                 const double* elem_mdot /*[E][12]*/, const double* opts,
                 int num_dof, const int64_t* rowptr, const int32_t* colind,
                 double* values, double* rhs, int n_threads);

/* one element's sumInto (TpetraLinearSystem::sumInto :1458-1522);
 * elem_nodes_lid[8] are node LIDs, lhs is (8*num_dof)^2 row-major */
void orc_sum_into(int num_dof, const int32_t* elem_nodes_lid, const double* lhs, const double* rhs,
                  const int64_t* rowptr, const int32_t* colind, double* values, double* sysrhs);
void orc_apply_dirichlet(const int64_t* rowptr, const int32_t* colind, double* values,
                         double* rhs, int64_t n_bc, const int32_t* rows,
                         const double* bc_value, const double* current);
void orc_reset_rows(const int64_t* rowptr, double* values, double* rhs,
                    int64_t n_rows_reset, const int32_t* rows);
void orc_sum_into_diag(const int64_t* rowptr, const int32_t* colind, double* values,
                       double* rhs, int32_t row, double diag, double rhs_value);

/* --- nodal geometry and gradients -------------------------------------- */
/* dual nodal volume: ComputeGeometryInteriorAlgorithm
 * (src/ComputeGeometryInteriorAlgorithm.C) sums HexSCV::determinant's eight
 * sub-control volumes into their nodes (ipNodeMap is the identity for Hex8);
 * conn holds node indices [E][8], vol [n] is overwritten */
void orc_dual_volume(int64_t n_nodes, int64_t n_elems, const int32_t* conn, const double* coords, double* vol);
/* element part of the projected nodal gradient: AssembleNodalGradElemAlgorithm
 * (src/AssembleNodalGradElemAlgorithm.C) for ncomp = 1 (dqdx [n][3]) and the
 * vector form of AssembleNodalGradUElemAlgorithm for ncomp = 3 (dudx [n][3][3],
 * du_i/dx_j at 3 i + j); q [n][ncomp]; grad is overwritten (zeroed first, as
 * the algorithm driver does); shifted selects shifted_shape_fcn */
void orc_nodal_grad_elem(int64_t n_nodes, int64_t n_elems, const int32_t* conn, const double* coords,
                         const double* q, int ncomp, const double* dual_volume, int shifted, double* grad);

/* --- boundary faces ---------------------------------------------------- */
/* Hex8 side s (0..5) -> its four element-local nodes (HexSCS::sideNodeOrdinals_,
 * src/master_element/Hex8CVFEM.C:415-422); the same table is the face ip ->
 * node map HexSCS::ipNodeMap(face) (:380-392) */
void orc_hex_side_nodes(int side, int* nodes4);
/* Quad3DSCS::determinant = quad3d_scs_det (src/master_element/MasterElementWork.F:
 * 1467-1590): the four sub-face area vectors of a quad, nodes in side order */
void orc_quad3d_scs_areav(const double* fcoords /*[4][3]*/, double* areav /*[4][3]*/);
/* HexSCS::face_grad_op / shifted_face_grad_op (Hex8CVFEM.C:668-684):
 * hex8_derivative at the exposed-face ips of side `side` (intgExpFace_,
 * :348-373; shifted: the face nodes) and generic_grad_op; returns the number of
 * ips with det(J) <= tiny */
int orc_hex_face_grad_op(int side, int shifted, const double* coords, double* gradop /*[4][8][3]*/);
/* exposed faces: flags[6 e + s] = 1 when side s of element e is a face of no
 * other element (conn holds node indices) */
void orc_skin(int64_t n_elems, const int32_t* conn, uint8_t* flags);
/* boundary closure of the projected nodal gradient
 * (AssembleNodalGradBoundaryAlgorithm::execute, src/AssembleNodalGradBoundaryAlgorithm.C:
 * 75-153): for every face ip, grad[nn] += q_ip A_ip / V_nn (nn the ip's node),
 * ADDED to grad [n][ncomp][3]; faces in list order */
void orc_nodal_grad_boundary(int64_t n_faces, const int32_t* face_elem, const int32_t* face_side,
                             const int32_t* conn, const double* coords, const double* q, int ncomp,
                             const double* dual_volume, int shifted, double* grad);
/* ContinuityInflowElemKernel::execute (src/kernel/ContinuityInflowElemKernel.C:
 * 73-108) on side `side` of one element, nodal inputs in element-node order;
 * rows of the element: rhs[8] (no lhs) */
void orc_continuity_inflow_face(int side, const double* coords, const double* rho,
                                const double* velocity_bc /*[8][3]*/, double proj_time_scale,
                                int shifted, double* rhs /*[8]*/);
/* ContinuityOpenElemKernel::execute (src/kernel/ContinuityOpenElemKernel.C:
 * 107-199), penaltyFac 2 (include/kernel/ContinuityOpenElemKernel.h:67); dynp
 * the face's dynamic_pressure [4] (may be NULL = 0); lhs [8][8], rhs [8] */
void orc_continuity_open_face(int side, const double* coords, const double* p, const double* pbc,
                              const double* rho, const double* velocity, const double* gpdx,
                              const double* dynp, double proj_time_scale, int shift_grad_op,
                              int reduced_sens, int shift_mdot, double* lhs, double* rhs);
/* face kernels over a face list, summed in list order through sumInto with
 * the element's nodes (num_dof 1); kernel 0 inflow, 1 open; opts =
 * {proj_time_scale, shift_grad_op, reduced_sens, shift_mdot}; dynp [nf][4] or NULL */
int orc_assemble_faces(int kernel, int64_t n_faces, const int32_t* face_elem, const int32_t* face_side,
                       const int32_t* conn, const int32_t* node_lid, const double* coords,
                       const double* p, const double* pbc, const double* rho, const double* velocity,
                       const double* gpdx, const double* dynp, const double* opts,
                       const int64_t* rowptr, const int32_t* colind, double* values, double* rhs);

/* --- solvers (FP64, stand-in for Belos/Ifpack2, unpinned) -------------- */
void orc_spmv(int64_t n, const int64_t* rowptr, const int32_t* colind, const double* v,
              const double* x, double* y, int n_threads);
/* Jacobi-PCG; returns iterations; res_out = true ||b-Ax||/||b|| */
int orc_pcg_jacobi(int64_t n, const int64_t* rowptr, const int32_t* colind, const double* v,
                   const double* b, double* x, double tol, int max_it, double* res_out,
                   int n_threads);
int orc_gmres_jacobi(int64_t n, const int64_t* rowptr, const int32_t* colind, const double* v,
                     const double* b, double* x, int restart, double tol, int max_it,
                     double* res_out, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
