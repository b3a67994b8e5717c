"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/liboracle.so`` (built by ``make -C oracle``).  Only the tests,
the smoke check and the benchmark's CPU-baseline leg import this module; the
product never does.  The optional ``_ref`` library is the reference's own
Hex8 master element compiled from its sources, used only to pin the oracle.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
_ref = None

KERNEL_SCALAR_DIFF = 0
KERNEL_CONTINUITY_ADV = 1
KERNEL_MOMENTUM_ADV_DIFF = 2
KERNEL_MOMENTUM_UPW_ADV_DIFF = 3
KERNEL_CONTINUITY_MASS = 4
KERNEL_MOMENTUM_MASS = 5


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle not built: run `make -C oracle`")
        _lib = ctypes.CDLL(path)
        L = _lib
        L.orc_graph_build.restype = ctypes.c_int
        L.orc_graph_build.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]
        L.orc_assemble.restype = ctypes.c_int
        L.orc_assemble.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64] + [ctypes.c_void_p] * 11 + \
            [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.orc_pcg_jacobi.restype = ctypes.c_int
        L.orc_pcg_jacobi.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 5 + [ctypes.c_double, ctypes.c_int,
                                                                                ctypes.c_void_p, ctypes.c_int]
        L.orc_gmres_jacobi.restype = ctypes.c_int
        L.orc_gmres_jacobi.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.c_double,
                                                                                  ctypes.c_int, ctypes.c_void_p,
                                                                                  ctypes.c_int]
        L.orc_spmv.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 5 + [ctypes.c_int]
        L.orc_dual_volume.argtypes = [ctypes.c_int64, ctypes.c_int64] + [ctypes.c_void_p] * 3
        L.orc_nodal_grad_elem.argtypes = [ctypes.c_int64, ctypes.c_int64] + [ctypes.c_void_p] * 3 + \
            [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_continuity_adv_elem.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                                      ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_momentum_adv_diff_elem.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_double, ctypes.c_int,
                                                                         ctypes.c_int, ctypes.c_void_p,
                                                                         ctypes.c_void_p]
        L.orc_momentum_upw_adv_diff_elem.argtypes = [ctypes.c_void_p] * 7 + [ctypes.c_double, ctypes.c_int,
                                                                             ctypes.c_int] + \
            [ctypes.c_double] * 4 + [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_mdot_elem.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                            ctypes.c_void_p]
        L.orc_continuity_mass_elem.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_double] * 4 + \
            [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_momentum_mass_elem.argtypes = [ctypes.c_void_p] * 8 + [ctypes.c_double] * 4 + \
            [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_assemble_mass.restype = ctypes.c_int
        L.orc_assemble_mass.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64] + [ctypes.c_void_p] * 15
        L.orc_hex_side_nodes.argtypes = [ctypes.c_int, ctypes.c_void_p]
        L.orc_quad3d_scs_areav.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_hex_face_grad_op.restype = ctypes.c_int
        L.orc_hex_face_grad_op.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_skin.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_nodal_grad_boundary.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 5 + \
            [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_continuity_inflow_face.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 3 + \
            [ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
        L.orc_continuity_open_face.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 7 + \
            [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_assemble_faces.restype = ctypes.c_int
        L.orc_assemble_faces.argtypes = [ctypes.c_int, ctypes.c_int64] + [ctypes.c_void_p] * 16
        L.orc_apply_dirichlet.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int64] + [ctypes.c_void_p] * 3
        L.orc_reset_rows.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int64, ctypes.c_void_p]
        L.orc_sum_into.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 7
        L.orc_sum_into_diag.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int32, ctypes.c_double, ctypes.c_double]
    return _lib


def ref():
    """The reference's own HexSCS/HexSCV (None where it was not built)."""
    global _ref
    if _ref is None:
        path = os.path.join(_HERE, "_ref", "libnalu_ref_me.so")
        if not os.path.exists(path):
            return None
        _ref = ctypes.CDLL(path)
    return _ref


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


# ---- master element ---------------------------------------------------------
def scs_tables():
    lr = np.zeros(24, np.int32)
    loc = np.zeros(36)
    locs = np.zeros(36)
    lib().orc_hex_scs_tables(_p(lr), _p(loc), _p(locs))
    return lr, loc, locs


def shape_fcn(iso):
    iso = _f64(iso)
    n = iso.size // 3
    out = np.zeros(n * 8)
    lib().orc_hex8_shape_fcn(n, _p(iso), _p(out))
    return out.reshape(n, 8)


def scs_areav(coords):
    c = _f64(coords)
    out = np.zeros(36)
    lib().orc_hex_scs_areav(_p(c), _p(out))
    return out.reshape(12, 3)


def scs_grad_op(coords, shifted=False):
    c = _f64(coords)
    g = np.zeros(288)
    d = np.zeros(288)
    nbad = lib().orc_hex_scs_grad_op(_p(c), int(shifted), _p(g), _p(d))
    return g.reshape(12, 8, 3), d.reshape(12, 8, 3), nbad


def scv_grad_op(coords, shifted=False):
    c = _f64(coords)
    g = np.zeros(192)
    d = np.zeros(192)
    nbad = lib().orc_hex_scv_grad_op(_p(c), int(shifted), _p(g), _p(d))
    return g.reshape(8, 8, 3), d.reshape(8, 8, 3), nbad


def scv_volume(coords):
    c = _f64(coords)
    v = np.zeros(8)
    lib().orc_hex_scv_volume(_p(c), _p(v))
    return v


# ---- element kernels --------------------------------------------------------
def scalar_diff_elem(coords, q, k, shifted=False):
    lhs, rhs = np.zeros(64), np.zeros(8)
    lib().orc_scalar_diff_elem(_p(_f64(coords)), _p(_f64(q)), _p(_f64(k)), int(shifted), _p(lhs), _p(rhs))
    return lhs.reshape(8, 8), rhs


def continuity_adv_elem(coords, vel, rho, p, gpdx, tau=1.0, shift_mdot=0, shift_poisson=0, reduced_sens=0):
    lhs, rhs = np.zeros(64), np.zeros(8)
    lib().orc_continuity_adv_elem(_p(_f64(coords)), _p(_f64(vel)), _p(_f64(rho)), _p(_f64(p)), _p(_f64(gpdx)),
                                  float(tau), int(shift_mdot), int(shift_poisson), int(reduced_sens),
                                  _p(lhs), _p(rhs))
    return lhs.reshape(8, 8), rhs


def momentum_adv_diff_elem(coords, u, mu, mdot, include_divu=0.0, shifted=False, skew=False):
    lhs, rhs = np.zeros(576), np.zeros(24)
    lib().orc_momentum_adv_diff_elem(_p(_f64(coords)), _p(_f64(u)), _p(_f64(mu)), _p(_f64(mdot)),
                                     float(include_divu), int(shifted), int(skew), _p(lhs), _p(rhs))
    return lhs.reshape(24, 24), rhs


def mdot_elem(coords, rho, vrtm, p, gpdx, tau=1.0, shift_mdot=0, shift_poisson=0):
    out = np.zeros(12)
    lib().orc_mdot_elem(_p(_f64(coords)), _p(_f64(rho)), _p(_f64(vrtm)), _p(_f64(p)), _p(_f64(gpdx)),
                        float(tau), int(shift_mdot), int(shift_poisson), _p(out))
    return out


def continuity_mass_elem(coords, rho_nm1, rho_n, rho_np1, dt, gamma1=1.0, gamma2=-1.0, gamma3=0.0, lumped=False):
    lhs, rhs = np.zeros(64), np.zeros(8)
    lib().orc_continuity_mass_elem(_p(_f64(coords)), _p(_f64(rho_nm1)), _p(_f64(rho_n)), _p(_f64(rho_np1)),
                                   float(dt), float(gamma1), float(gamma2), float(gamma3), int(bool(lumped)),
                                   _p(lhs), _p(rhs))
    return lhs.reshape(8, 8), rhs


def momentum_mass_elem(coords, rho_nm1, rho_n, rho_np1, u_nm1, u_n, u_np1, gpdx, dt, gamma1=1.0, gamma2=-1.0,
                       gamma3=0.0, lumped=False, balanced_force=False):
    lhs, rhs = np.zeros(576), np.zeros(24)
    lib().orc_momentum_mass_elem(_p(_f64(coords)), _p(_f64(rho_nm1)), _p(_f64(rho_n)), _p(_f64(rho_np1)),
                                 _p(_f64(u_nm1)), _p(_f64(u_n)), _p(_f64(u_np1)), _p(_f64(gpdx)), float(dt),
                                 float(gamma1), float(gamma2), float(gamma3), int(bool(lumped)),
                                 int(bool(balanced_force)), _p(lhs), _p(rhs))
    return lhs.reshape(24, 24), rhs


def assemble_mass(momentum, coords, conn, rowptr, colind, lid, rho_nm1, rho_n, rho_np1, u_nm1=None, u_n=None,
                  u_np1=None, gpdx=None, dt=1.0, gamma1=1.0, gamma2=-1.0, gamma3=0.0, lumped=False,
                  balanced_force=False):
    """Whole-mesh mass-term assembly (serial element order, restated sumInto)."""
    values = np.zeros(colind.shape[0])
    rhs = np.zeros(rowptr.shape[0] - 1)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    conv = lambda a: None if a is None else _f64(a)
    tp = np.array([dt, gamma1, gamma2, gamma3, float(bool(lumped)), float(bool(balanced_force))])
    rc = lib().orc_assemble_mass(int(bool(momentum)), coords.shape[0], conn.shape[0], _p(conn), _p(lid),
                                 _p(_f64(coords)), _p(_f64(rho_nm1)), _p(_f64(rho_n)), _p(_f64(rho_np1)),
                                 _p(conv(u_nm1)), _p(conv(u_n)), _p(conv(u_np1)), _p(conv(gpdx)), _p(tp),
                                 _p(rowptr), _p(colind), _p(values), _p(rhs))
    if rc:
        raise RuntimeError("orc_assemble_mass: %d" % rc)
    return values, rhs


# ---- boundary faces ---------------------------------------------------------
FACE_CONTINUITY_INFLOW = 0
FACE_CONTINUITY_OPEN = 1


def side_nodes(side):
    out = np.zeros(4, np.int32)
    lib().orc_hex_side_nodes(int(side), _p(out))
    return out


def quad_areav(fcoords):
    out = np.zeros(12)
    lib().orc_quad3d_scs_areav(_p(_f64(fcoords)), _p(out))
    return out.reshape(4, 3)


def face_grad_op(side, coords, shifted=False):
    g = np.zeros(96)
    nbad = lib().orc_hex_face_grad_op(int(side), int(bool(shifted)), _p(_f64(coords)), _p(g))
    return g.reshape(4, 8, 3), nbad


def skin(conn):
    """(elem, side) pairs of the exposed faces, sorted by element then side"""
    conn = np.ascontiguousarray(conn, np.int32)
    flags = np.zeros(conn.shape[0] * 6, np.uint8)
    lib().orc_skin(conn.shape[0], _p(conn), _p(flags))
    idx = np.nonzero(flags)[0]
    return (idx // 6).astype(np.int64), (idx % 6).astype(np.int32)


def nodal_grad_boundary(coords, conn, face_elem, face_side, q, dual_volume, grad, shifted=False):
    """adds the boundary closure into grad ([n,3] or [n,3,3]) in place"""
    q = _f64(q)
    ncomp = 1 if q.ndim == 1 else q.shape[1]
    fe = np.ascontiguousarray(face_elem, np.int32)
    fs = np.ascontiguousarray(face_side, np.int32)
    assert grad.dtype == np.float64 and grad.flags.c_contiguous
    lib().orc_nodal_grad_boundary(fe.shape[0], _p(fe), _p(fs), _p(np.ascontiguousarray(conn, np.int32)),
                                  _p(_f64(coords)), _p(q), ncomp, _p(_f64(dual_volume)), int(bool(shifted)),
                                  _p(grad))
    return grad


def continuity_inflow_face(side, coords, rho, ubc, proj_time_scale=1.0, shifted=False):
    rhs = np.zeros(8)
    lib().orc_continuity_inflow_face(int(side), _p(_f64(coords)), _p(_f64(rho)), _p(_f64(ubc)),
                                     float(proj_time_scale), int(bool(shifted)), _p(rhs))
    return np.zeros((8, 8)), rhs


def continuity_open_face(side, coords, p, pbc, rho, u, gpdx, dynp=None, proj_time_scale=1.0, shift_grad_op=0,
                         reduced_sens=0, shift_mdot=0):
    lhs, rhs = np.zeros(64), np.zeros(8)
    lib().orc_continuity_open_face(int(side), _p(_f64(coords)), _p(_f64(p)), _p(_f64(pbc)), _p(_f64(rho)),
                                   _p(_f64(u)), _p(_f64(gpdx)), _p(None if dynp is None else _f64(dynp)),
                                   float(proj_time_scale), int(shift_grad_op), int(reduced_sens), int(shift_mdot),
                                   _p(lhs), _p(rhs))
    return lhs.reshape(8, 8), rhs


def assemble_faces(kernel, coords, conn, face_elem, face_side, rowptr, colind, lid, rho, velocity, p=None,
                   pbc=None, gpdx=None, dynp=None, proj_time_scale=1.0, shift_grad_op=0, reduced_sens=0,
                   shift_mdot=0):
    values = np.zeros(colind.shape[0])
    rhs = np.zeros(rowptr.shape[0] - 1)
    fe = np.ascontiguousarray(face_elem, np.int32)
    fs = np.ascontiguousarray(face_side, np.int32)
    conv = lambda a: None if a is None else _f64(a)
    o = np.array([proj_time_scale, shift_grad_op, reduced_sens, shift_mdot], np.float64)
    rc = lib().orc_assemble_faces(int(kernel), fe.shape[0], _p(fe), _p(fs), _p(np.ascontiguousarray(conn, np.int32)),
                                  _p(lid), _p(_f64(coords)), _p(conv(p)), _p(conv(pbc)), _p(_f64(rho)),
                                  _p(_f64(velocity)), _p(conv(gpdx)), _p(conv(dynp)), _p(o), _p(rowptr), _p(colind),
                                  _p(values), _p(rhs))
    if rc:
        raise RuntimeError("orc_assemble_faces: %d" % rc)
    return values, rhs


# ---- linear system ----------------------------------------------------------
def graph(n_nodes, conn, num_dof=1, gid=None):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    gid = None if gid is None else np.ascontiguousarray(gid, dtype=np.int64)
    nr = ctypes.c_int64(0)
    nnz = ctypes.c_int64(0)
    rc = lib().orc_graph_build(n_nodes, conn.shape[0], _p(conn), _p(gid), num_dof, ctypes.byref(nr),
                               ctypes.byref(nnz), None, None, None)
    if rc:
        raise RuntimeError("orc_graph_build: %d" % rc)
    rowptr = np.zeros(nr.value + 1, np.int64)
    colind = np.zeros(nnz.value, np.int32)
    lid = np.zeros(n_nodes, np.int32)
    rc = lib().orc_graph_build(n_nodes, conn.shape[0], _p(conn), _p(gid), num_dof, ctypes.byref(nr),
                               ctypes.byref(nnz), _p(rowptr), _p(colind), _p(lid))
    if rc:
        raise RuntimeError("orc_graph_build: %d" % rc)
    return rowptr, colind[:nnz.value], lid


def opts_block(shifted_grad_op=0, shift_mdot=0, shift_poisson=0, reduced_sens=0, proj_time_scale=1.0,
               include_divu=0.0, skew_symmetric=0, alpha=0.0, alpha_upw=1.0, upw_factor=1.0,
               hybrid_factor=0.0, use_limiter=0):
    o = np.zeros(16)
    o[:12] = [shifted_grad_op, shift_mdot, shift_poisson, reduced_sens, proj_time_scale, include_divu,
              skew_symmetric, alpha, alpha_upw, upw_factor, hybrid_factor, use_limiter]
    return o


def assemble(kernel, coords, conn, rowptr, colind, lid=None, scalar=None, coeff=None, vec=None, vec2=None,
             rho=None, gju=None, mdot=None, opts=None, n_threads=1):
    num_dof = 3 if kernel >= 2 else 1
    n = coords.shape[0]
    values = np.zeros(colind.shape[0])
    rhs = np.zeros(rowptr.shape[0] - 1)
    opts = opts_block() if opts is None else opts
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    conv = lambda a: None if a is None else _f64(a)
    rc = lib().orc_assemble(kernel, n, conn.shape[0], _p(conn), _p(lid), _p(_f64(coords)), _p(conv(scalar)),
                            _p(conv(coeff)), _p(conv(vec)), _p(conv(vec2)), _p(conv(rho)), _p(conv(gju)),
                            _p(conv(mdot)), _p(_f64(opts)), num_dof, _p(rowptr), _p(colind), _p(values),
                            _p(rhs), int(n_threads))
    if rc:
        raise RuntimeError("orc_assemble: %d" % rc)
    return values, rhs


def sum_into(num_dof, elem_lids, lhs, rhs, rowptr, colind, values, sysrhs):
    lids = np.ascontiguousarray(elem_lids, np.int32)
    lib().orc_sum_into(int(num_dof), _p(lids), _p(_f64(lhs)), _p(_f64(rhs)), _p(rowptr), _p(colind),
                       _p(values), _p(sysrhs))


def apply_dirichlet(rowptr, colind, values, rhs, rows, bc, current):
    rows = np.ascontiguousarray(rows, np.int32)
    lib().orc_apply_dirichlet(_p(rowptr), _p(colind), _p(values), _p(rhs), rows.size, _p(rows),
                              _p(_f64(bc)), _p(_f64(current)))


def reset_rows(rowptr, values, rhs, rows):
    rows = np.ascontiguousarray(rows, np.int32)
    lib().orc_reset_rows(_p(rowptr), _p(values), _p(rhs), rows.size, _p(rows))


def sum_into_diag(rowptr, colind, values, rhs, row, diag, rhs_value):
    lib().orc_sum_into_diag(_p(rowptr), _p(colind), _p(values), _p(rhs), int(row), float(diag), float(rhs_value))


def spmv(rowptr, colind, values, x, n_threads=1):
    y = np.zeros(rowptr.shape[0] - 1)
    lib().orc_spmv(y.size, _p(rowptr), _p(colind), _p(values), _p(_f64(x)), _p(y), int(n_threads))
    return y


def pcg_jacobi(rowptr, colind, values, b, tol=1e-8, max_it=10000, x0=None, n_threads=1):
    n = rowptr.shape[0] - 1
    x = np.zeros(n) if x0 is None else _f64(x0).copy()
    res = ctypes.c_double(0)
    it = lib().orc_pcg_jacobi(n, _p(rowptr), _p(colind), _p(values), _p(_f64(b)), _p(x), float(tol), int(max_it),
                              ctypes.byref(res), int(n_threads))
    return x, it, res.value


def gmres_jacobi(rowptr, colind, values, b, restart=50, tol=1e-8, max_it=10000, x0=None, n_threads=1):
    n = rowptr.shape[0] - 1
    x = np.zeros(n) if x0 is None else _f64(x0).copy()
    res = ctypes.c_double(0)
    it = lib().orc_gmres_jacobi(n, _p(rowptr), _p(colind), _p(values), _p(_f64(b)), _p(x), int(restart),
                                float(tol), int(max_it), ctypes.byref(res), int(n_threads))
    return x, it, res.value


def dual_volume(coords, conn):
    """Dual nodal volume (sum of HexSCV sub-control volumes per node)."""
    coords = _f64(coords)
    conn = np.ascontiguousarray(conn, np.int32)
    vol = np.zeros(coords.shape[0])
    lib().orc_dual_volume(coords.shape[0], conn.shape[0], _p(conn), _p(coords), _p(vol))
    return vol


def nodal_grad_elem(coords, conn, q, dual_volume, shifted=False):
    """Element part of the projected nodal gradient; q [n] -> [n,3], q [n,3] -> [n,3,3]."""
    coords = _f64(coords)
    conn = np.ascontiguousarray(conn, np.int32)
    q = _f64(q)
    ncomp = 1 if q.ndim == 1 else q.shape[1]
    grad = np.zeros((coords.shape[0], ncomp, 3))
    lib().orc_nodal_grad_elem(coords.shape[0], conn.shape[0], _p(conn), _p(coords), _p(q), ncomp,
                              _p(_f64(dual_volume)), int(bool(shifted)), _p(grad))
    return grad[:, 0, :] if ncomp == 1 else grad
