// ref_driver.cpp -- C entry points into the reference's own HexSCS/HexSCV
// code (src/master_element/Hex8CVFEM.C compiled from the reference tree by
// Makefile.ref).  TEST INFRASTRUCTURE ONLY: used to pin the oracle's
// restatement of the master element, never by the product.
#include <master_element/Hex8CVFEM.h>
#include <NaluEnv.h>
#include <iostream>

using sierra::nalu::SharedMemView;

extern "C" {
void ref_hex_scs_areav(const double* coords, double* areav) {
  sierra::nalu::HexSCS me;
  SharedMemView<DoubleType**> c(const_cast<double*>(coords), 8, 3), a(areav, 12, 3);
  me.determinant(c, a);
}
void ref_hex_scs_grad_op(const double* coords, int shifted, double* gradop, double* deriv) {
  sierra::nalu::HexSCS me;
  SharedMemView<DoubleType**> c(const_cast<double*>(coords), 8, 3);
  SharedMemView<DoubleType***> g(gradop, 12, 8, 3), d(deriv, 12, 8, 3);
  if (shifted) me.shifted_grad_op(c, g, d); else me.grad_op(c, g, d);
}
void ref_hex_scs_shape_fcn(int shifted, double* shp) {
  sierra::nalu::HexSCS me;
  SharedMemView<DoubleType**> s(shp, 12, 8);
  if (shifted) me.shifted_shape_fcn(s); else me.shape_fcn(s);
}
void ref_hex_scv_volume(const double* coords, double* vol) {
  sierra::nalu::HexSCV me;
  SharedMemView<DoubleType**> c(const_cast<double*>(coords), 8, 3);
  SharedMemView<DoubleType*> v(vol, 8);
  me.determinant(c, v);
}
void ref_hex_scv_grad_op(const double* coords, int shifted, double* gradop, double* deriv) {
  sierra::nalu::HexSCV me;
  SharedMemView<DoubleType**> c(const_cast<double*>(coords), 8, 3);
  SharedMemView<DoubleType***> g(gradop, 8, 8, 3), d(deriv, 8, 8, 3);
  if (shifted) me.shifted_grad_op(c, g, d); else me.grad_op(c, g, d);
}
void ref_hex_face_grad_op(int side, int shifted, const double* coords, double* gradop) {
  sierra::nalu::HexSCS me;
  SharedMemView<DoubleType**> c(const_cast<double*>(coords), 8, 3);
  SharedMemView<DoubleType***> g(gradop, 4, 8, 3);
  if (shifted) me.shifted_face_grad_op(side, c, g); else me.face_grad_op(side, c, g);
}
void ref_hex_side_nodes(int side, int* nodes4) {
  sierra::nalu::HexSCS me;
  const int* o = me.side_node_ordinals(side);
  const int* m = me.ipNodeMap(side);
  for (int k = 0; k < 4; ++k) nodes4[k] = o[k], nodes4[4 + k] = m[k];
}
const int* ref_hex_scs_adjacent_nodes() {
  static sierra::nalu::HexSCS me;
  return me.adjacentNodes();
}
}

// ---- link stubs: logging and the Fortran kernels behind the legacy double*
// overloads (never called by the entry points above). ----
namespace sierra { namespace nalu {
NaluEnv::NaluEnv()
    : parallelCommunicator_(0), pSize_(1), pRank_(0), stdoutStream_(nullptr),
      naluLogStream_(&std::cout), naluParallelStream_(&std::cout), parallelLog_(false) {}
NaluEnv::~NaluEnv() {}
NaluEnv& NaluEnv::self() { static NaluEnv env; return env; }
std::ostream& NaluEnv::naluOutput() { return std::cout; }
std::ostream& NaluEnv::naluOutputP0() { return std::cout; }
} }
#include <cstdlib>
#define NALU_REF_FORTRAN_STUB(name) extern "C" void name(...) { std::abort(); }
NALU_REF_FORTRAN_STUB(edge2d_scs_det_)
NALU_REF_FORTRAN_STUB(hex_derivative_)
NALU_REF_FORTRAN_STUB(hex_gradient_operator_)
NALU_REF_FORTRAN_STUB(hex_scs_det_)
NALU_REF_FORTRAN_STUB(hex_scv_det_)
NALU_REF_FORTRAN_STUB(hex_shape_fcn_)
NALU_REF_FORTRAN_STUB(threed_gij_)
NALU_REF_FORTRAN_STUB(tri3d_scs_det_)
NALU_REF_FORTRAN_STUB(tri_scv_det_)
