"""nalu_gb300 -- GB300 (sm_103a) Hex8 CVFEM assembly and continuity solve.

Python front end of the C ABI declared in ``include/nalu_gb300.h``.  The
compute runs in ``nalu_gb300/_lib/libnalu_gb300.so`` (built in tree by
``python -m nalu_gb300.build``); there is no CPU fallback: if the library or a
CUDA device is missing, every call raises.

The classes mirror the reference's host interface for this path:

* ``Context``            -- one device/stream/mesh/linear system (C ``nalu_ctx``)
* ``LinearSystem``       -- TpetraLinearSystem's graph/zero/sumInto/BC/solve API
* ``AssembleElemSolverAlgorithm`` -- runs the registered element kernels
* ``ScalarDiffElemKernel``, ``ContinuityAdvElemKernel``,
  ``MomentumAdvDiffElemKernel``, ``MomentumUpwAdvDiffElemKernel``
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libnalu_gb300.so")
CHECK_LIB_PATH = os.path.join(_HERE, "_lib", "libnalu_elemcheck.so")

NALU_OK = 0
STATUS = {0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "call out of order",
          -4: "negative Jacobian", -5: "non-finite value", -6: "capacity exceeded",
          -7: "not converged", -8: "entry missing from graph", -9: "no CUDA device"}

FIELD = {"coordinates": 0, "scalar_q": 1, "diff_coeff": 2, "velocity": 3, "velocity_rtm": 4,
         "density": 5, "pressure": 6, "dpdx": 7, "viscosity": 8, "dudx": 9, "mass_flow_rate_scs": 10,
         "dual_nodal_volume": 11, "density_n": 12, "density_nm1": 13, "velocity_n": 14, "velocity_nm1": 15,
         "pressure_bc": 16, "cont_velocity_bc": 17}
KERNEL_SCALAR_DIFF = 0
KERNEL_CONTINUITY_ADV = 1
KERNEL_MOMENTUM_ADV_DIFF = 2
KERNEL_MOMENTUM_UPW_ADV_DIFF = 3
KERNEL_CONTINUITY_MASS = 4
KERNEL_MOMENTUM_MASS = 5
FACE_CONTINUITY_INFLOW, FACE_CONTINUITY_OPEN = 0, 1
MAX_FACE_SETS = 16
SCATTER_AUTO, SCATTER_ATOMIC, SCATTER_COLOURED = 0, 1, 2
ARITH_FP64, ARITH_DF64 = 0, 1
SCHEDULE_AUTO, SCHEDULE_ELEMENT, SCHEDULE_IP8, SCHEDULE_IP16 = 0, 1, 2, 3
SCHEDULE_NAMES = {SCHEDULE_ELEMENT: "element", SCHEDULE_IP8: "ip8", SCHEDULE_IP16: "ip16"}
SOLVER_CG, SOLVER_GMRES = 0, 1
PRECOND_NONE, PRECOND_JACOBI, PRECOND_CHEBYSHEV, PRECOND_LEARNED = 0, 1, 2, 3
PRECOND_MULTILEVEL, PRECOND_LEARNED_MULTILEVEL = 4, 5
TRAIN_BF16, TRAIN_FP32 = 0, 1
LEARNED_PARAMS = 15361
PRECISION_FP64, PRECISION_FP32_INNER_IR = 0, 1


class NaluError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "error"), status, msg))
        self.status = status


class AssembleOpts(ctypes.Structure):
    _fields_ = [("shifted_grad_op", ctypes.c_int), ("shift_mdot", ctypes.c_int), ("shift_poisson", ctypes.c_int),
                ("reduced_sens", ctypes.c_int), ("skew_symmetric", ctypes.c_int), ("use_limiter", ctypes.c_int),
                ("proj_time_scale", ctypes.c_double), ("include_divu", ctypes.c_double),
                ("alpha", ctypes.c_double), ("alpha_upw", ctypes.c_double), ("upw_factor", ctypes.c_double),
                ("hybrid_factor", ctypes.c_double), ("scatter", ctypes.c_int), ("arith", ctypes.c_int),
                ("lumped_mass", ctypes.c_int), ("balanced_force", ctypes.c_int), ("dt", ctypes.c_double),
                ("gamma1", ctypes.c_double), ("gamma2", ctypes.c_double), ("gamma3", ctypes.c_double),
                ("schedule", ctypes.c_int), ("reserved", ctypes.c_int * 3)]


class SolverOpts(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("precond", ctypes.c_int), ("precision", ctypes.c_int),
                ("max_iters", ctypes.c_int), ("restart", ctypes.c_int), ("cheb_degree", ctypes.c_int),
                ("check_every", ctypes.c_int), ("x0_zero", ctypes.c_int), ("tol", ctypes.c_double),
                ("inner_tol", ctypes.c_double), ("stall_window", ctypes.c_int), ("learned_probe", ctypes.c_int),
                ("ml_kcycle_levels", ctypes.c_int), ("ml_learned_sweeps", ctypes.c_int),
                ("reserved", ctypes.c_int * 2)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("outer_iterations", ctypes.c_int), ("status", ctypes.c_int),
                ("true_rel_res", ctypes.c_double), ("seconds", ctypes.c_double), ("fallback", ctypes.c_int),
                ("learned_iterations", ctypes.c_int), ("setup_seconds", ctypes.c_double),
                ("probe_rate_jacobi", ctypes.c_double), ("probe_rate_learned", ctypes.c_double)]


class TrainOpts(ctypes.Structure):
    _fields_ = [("epochs", ctypes.c_int), ("batch", ctypes.c_int), ("lr", ctypes.c_double),
                ("val_fraction", ctypes.c_double), ("seed", ctypes.c_uint64), ("precision", ctypes.c_int),
                ("reserved", ctypes.c_int * 3)]


_lib = None


def lib():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("nalu_gb300 CUDA library missing: %s (run python -m nalu_gb300.build)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        P, I, I64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
        sig = {
            "nalu_create": (I, [I, ctypes.POINTER(P)]),
            "nalu_destroy": (I, [P]),
            "nalu_last_error": (ctypes.c_char_p, [P]),
            "nalu_status_string": (ctypes.c_char_p, [I]),
            "nalu_get_stream": (I, [P, ctypes.POINTER(P)]),
            "nalu_synchronize": (I, [P]),
            "nalu_mesh_create": (I, [P, I64, I64, P, P, P]),
            "nalu_field_set": (I, [P, I, P, I64, I]),
            "nalu_field_get": (I, [P, I, P, I64, I]),
            "nalu_field_set_async": (I, [P, I, P, I64]),
            "nalu_linsys_build_elem_graph": (I, [P, I]),
            "nalu_linsys_sizes": (I, [P, P, P, P]),
            "nalu_linsys_graph": (I, [P, P, P]),
            "nalu_linsys_device_arrays": (I, [P, P, P, P, P, P]),
            "nalu_linsys_zero": (I, [P]),
            "nalu_linsys_sum_into": (I, [P, I64, P, P, P]),
            "nalu_linsys_apply_dirichlet": (I, [P, I64, P, I, I, P, P]),
            "nalu_linsys_reset_rows": (I, [P, I64, P, I, I]),
            "nalu_linsys_sum_into_diag": (I, [P, ctypes.c_int32, I, D, D]),
            "nalu_linsys_load_complete": (I, [P]),
            "nalu_linsys_copy": (I, [P, P, P, I]),
            "nalu_linsys_copy_async": (I, [P, P, P]),
            "nalu_linsys_copy_wait": (I, [P]),
            "nalu_assemble_opts_default": (None, [P]),
            "nalu_assemble": (I, [P, I, P]),
            "nalu_capture_element": (I, [P, I, P, I64, P, P]),
            "nalu_compute_mdot": (I, [P, P]),
            "nalu_compute_dual_volume": (I, [P]),
            "nalu_capture_scv_volumes": (I, [P, I64, P]),
            "nalu_compute_nodal_gradient": (I, [P, I, I, I, I]),
            "nalu_linsys_write_system": (I, [P, ctypes.c_char_p]),
            "nalu_linsys_write_solution": (I, [P, ctypes.c_char_p]),
            "nalu_hex_scs_determinant": (I, [P, I64, P, P, I]),
            "nalu_hex_scs_grad_op": (I, [P, I64, P, I, P, P, I]),
            "nalu_hex_scv_grad_op": (I, [P, I64, P, I, P, P, I]),
            "nalu_hex_scv_determinant": (I, [P, I64, P, P, I]),
            "nalu_hex_face_grad_op": (I, [P, I64, P, P, I, P, I]),
            "nalu_hex_scs_adjacent_nodes": (None, [P]),
            "nalu_hex_scs_shape_fcn": (None, [I, P]),
            "nalu_hex_side_node_ordinals": (None, [I, P]),
            "nalu_faceset_define": (I, [P, I, I64, P, P]),
            "nalu_faceset_skin": (I, [P, I, ctypes.POINTER(I64)]),
            "nalu_faceset_size": (I, [P, I, ctypes.POINTER(I64)]),
            "nalu_faceset_get": (I, [P, I, P, P]),
            "nalu_faceset_dynamic_pressure": (I, [P, I, P]),
            "nalu_faceset_exposed_area": (I, [P, I, P]),
            "nalu_nodal_gradient_boundary": (I, [P, I, I, I, I]),
            "nalu_assemble_faces": (I, [P, I, I, P]),
            "nalu_capture_face": (I, [P, I, I, P, I64, P, P]),
            "nalu_solver_opts_default": (None, [P]),
            "nalu_solve": (I, [P, P, P]),
            "nalu_solution_get": (I, [P, P, I]),
            "nalu_solution_set": (I, [P, P, I]),
            "nalu_spmv": (I, [P, P, P, I]),
            "nalu_set_problems": (I, [P, I, P]),
            "nalu_learned_init": (I, [P, ctypes.c_uint64]),
            "nalu_learned_set_weights": (I, [P, P, I64]),
            "nalu_learned_get_weights": (I, [P, P, I64]),
            "nalu_learned_harvest": (I, [P, I, ctypes.c_uint64, I64, P, P, P, P, ctypes.POINTER(I64)]),
            "nalu_train_opts_default": (None, [P]),
            "nalu_learned_train": (I, [P, P, P, P, I64, P, P]),
            "nalu_batch_autotune": (I, [P, I, ctypes.POINTER(I), P]),
            "nalu_learned_gradient": (I, [P, P, P, P, I64, P, ctypes.POINTER(D)]),
            "nalu_learned_gradient_bf16": (I, [P, P, P, P, I64, P, ctypes.POINTER(D)]),
            "nalu_learned_stencil": (I, [P, P]),
            "nalu_solve_batched": (I, [P, P, P]),
            "nalu_assemble_tuning": (I, [P, I, ctypes.POINTER(I), ctypes.POINTER(I), P]),
            "nalu_multilevel_levels": (I, [P, I, P, P]),
            "nalu_kernel_launch_count": (I64, [P]),
            "nalu_last_assemble_ms": (D, [P]),
            "nalu_probe_fp64_tflops": (I, [P, ctypes.POINTER(D)]),
            "nalu_event_record": (I, [P, I]),
            "nalu_event_elapsed_ms": (I, [P, I, I, ctypes.POINTER(D)]),
            "nalu_host_alloc": (I, [ctypes.c_size_t, ctypes.POINTER(P)]),
            "nalu_host_free": (I, [P]),
            "nalu_flush_l2": (I, [P, ctypes.c_size_t]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def default_assemble_opts(**kw):
    o = AssembleOpts()
    lib().nalu_assemble_opts_default(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def default_solver_opts(**kw):
    o = SolverOpts()
    lib().nalu_solver_opts_default(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Context:
    """One device, one stream, one Hex8 mesh and its linear system."""

    def __init__(self, device=0):
        self._h = ctypes.c_void_p()
        rc = lib().nalu_create(device, ctypes.byref(self._h))
        if rc:
            raise NaluError(rc, "nalu_create(device=%d)" % device)

    def _check(self, rc, what=""):
        if rc:
            msg = lib().nalu_last_error(self._h)
            raise NaluError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    def close(self):
        if self._h:
            lib().nalu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # mesh / fields
    def mesh_create(self, coords, conn, gid=None):
        coords = np.ascontiguousarray(coords, np.float64)
        conn = np.ascontiguousarray(conn, np.int32)
        gid = None if gid is None else np.ascontiguousarray(gid, np.int64)
        self.n_nodes, self.n_elems = coords.shape[0], conn.shape[0]
        self._check(lib().nalu_mesh_create(self._h, self.n_nodes, self.n_elems, _ptr(conn), _ptr(gid),
                                           _ptr(coords)), "mesh_create")

    def field_set(self, name, values):
        a = np.ascontiguousarray(values, np.float64)
        self._check(lib().nalu_field_set(self._h, FIELD[name], _ptr(a), a.size, 0), "field_set(%s)" % name)

    def field_get(self, name, shape):
        out = np.zeros(shape, np.float64)
        self._check(lib().nalu_field_get(self._h, FIELD[name], _ptr(out), out.size, 0), "field_get(%s)" % name)
        return out

    # linear system
    def build_elem_graph(self, num_dof):
        self._check(lib().nalu_linsys_build_elem_graph(self._h, num_dof), "build_elem_graph")

    def sizes(self):
        nr, nnz, nd = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        self._check(lib().nalu_linsys_sizes(self._h, ctypes.byref(nr), ctypes.byref(nnz), ctypes.byref(nd)))
        return nr.value, nnz.value, nd.value

    def graph(self):
        nr, nnz, _ = self.sizes()
        rp = np.zeros(nr + 1, np.int64)
        ci = np.zeros(nnz, np.int32)
        self._check(lib().nalu_linsys_graph(self._h, _ptr(rp), _ptr(ci)), "graph")
        return rp, ci

    def zero(self):
        self._check(lib().nalu_linsys_zero(self._h), "zero")

    def sum_into(self, elem_ids, lhs, rhs):
        e = np.ascontiguousarray(elem_ids, np.int64)
        l_ = np.ascontiguousarray(lhs, np.float64)
        r_ = np.ascontiguousarray(rhs, np.float64)
        self._check(lib().nalu_linsys_sum_into(self._h, e.size, _ptr(e), _ptr(l_), _ptr(r_)), "sum_into")

    def apply_dirichlet(self, nodes, bc, solution, begin_dof=0, end_dof=None):
        nodes = np.ascontiguousarray(nodes, np.int32)
        _, _, nd = self.sizes()
        end_dof = nd if end_dof is None else end_dof
        bc = np.ascontiguousarray(bc, np.float64)
        solution = np.ascontiguousarray(solution, np.float64)
        self._check(lib().nalu_linsys_apply_dirichlet(self._h, nodes.size, _ptr(nodes), begin_dof, end_dof,
                                                      _ptr(bc), _ptr(solution)), "apply_dirichlet")

    def reset_rows(self, nodes, begin_dof=0, end_dof=None):
        nodes = np.ascontiguousarray(nodes, np.int32)
        _, _, nd = self.sizes()
        end_dof = nd if end_dof is None else end_dof
        self._check(lib().nalu_linsys_reset_rows(self._h, nodes.size, _ptr(nodes), begin_dof, end_dof),
                    "reset_rows")

    def sum_into_diag(self, node, dof, diag, rhs):
        self._check(lib().nalu_linsys_sum_into_diag(self._h, int(node), int(dof), float(diag), float(rhs)),
                    "sum_into_diag")

    def load_complete(self):
        self._check(lib().nalu_linsys_load_complete(self._h), "load_complete")

    def system(self):
        nr, nnz, _ = self.sizes()
        v = np.zeros(nnz)
        r = np.zeros(nr)
        self._check(lib().nalu_linsys_copy(self._h, _ptr(v), _ptr(r), 0), "copy")
        return v, r

    # assembly
    def assemble(self, kernel, opts=None):
        opts = default_assemble_opts() if opts is None else opts
        self._check(lib().nalu_assemble(self._h, kernel, ctypes.byref(opts)), "assemble")

    def assemble_tuning(self, kernel):
        """the autotuned (schedule, scatter) of a double-float scalar kernel and
        the device time (ms) of every candidate {(schedule, scatter): ms}"""
        sch, sc = ctypes.c_int(), ctypes.c_int()
        ms = np.zeros(6)
        self._check(lib().nalu_assemble_tuning(self._h, kernel, ctypes.byref(sch), ctypes.byref(sc), _ptr(ms)),
                    "assemble_tuning")
        table = {(SCHEDULE_NAMES[1 + k // 2], {0: "atomic", 1: "coloured"}[k % 2]): float(ms[k])
                 for k in range(6) if ms[k] >= 0}
        return sch.value, sc.value, table

    def batch_autotune(self, iterations=100):
        """rows per tile of the batched solve, chosen by device time; returns
        (tile_rows, {rows: ms per iteration})"""
        tr = ctypes.c_int()
        ms = np.zeros(4)
        self._check(lib().nalu_batch_autotune(self._h, int(iterations), ctypes.byref(tr), _ptr(ms)), "batch_autotune")
        return tr.value, {r: float(m) for r, m in zip((256, 512, 1024, 2048), ms)}

    def multilevel_levels(self):
        """(rows, nnz) per level of the last multilevel solve's hierarchy"""
        rows, nnz = np.zeros(16, np.int64), np.zeros(16, np.int64)
        nl = lib().nalu_multilevel_levels(self._h, 16, _ptr(rows), _ptr(nnz))
        return rows[:nl].tolist(), nnz[:nl].tolist()

    def capture_element(self, kernel, elem, opts=None):
        opts = default_assemble_opts() if opts is None else opts
        ne = 24 if kernel in (KERNEL_MOMENTUM_ADV_DIFF, KERNEL_MOMENTUM_UPW_ADV_DIFF, KERNEL_MOMENTUM_MASS) else 8
        lhs = np.zeros((ne, ne))
        rhs = np.zeros(ne)
        self._check(lib().nalu_capture_element(self._h, kernel, ctypes.byref(opts), int(elem), _ptr(lhs), _ptr(rhs)),
                    "capture_element")
        return lhs, rhs

    def compute_mdot(self, opts=None):
        opts = default_assemble_opts() if opts is None else opts
        self._check(lib().nalu_compute_mdot(self._h, ctypes.byref(opts)), "compute_mdot")

    # nodal geometry and gradients
    def compute_dual_volume(self):
        self._check(lib().nalu_compute_dual_volume(self._h), "compute_dual_volume")

    def capture_scv_volumes(self, elem):
        v = np.zeros(8)
        self._check(lib().nalu_capture_scv_volumes(self._h, int(elem), _ptr(v)), "capture_scv_volumes")
        return v

    def compute_nodal_gradient(self, src, dst, shifted=False, arith=ARITH_FP64):
        self._check(lib().nalu_compute_nodal_gradient(self._h, FIELD[src], FIELD[dst], int(bool(shifted)),
                                                      int(arith)), "compute_nodal_gradient")

    # MatrixMarket dumps
    def write_system(self, base):
        self._check(lib().nalu_linsys_write_system(self._h, os.fsencode(base)), "write_system")

    def write_solution(self, base):
        self._check(lib().nalu_linsys_write_solution(self._h, os.fsencode(base)), "write_solution")

    # Hex8 master element, batched over elements (coords [nelem, 8, 3])
    def hex_scs_determinant(self, coords):
        c = np.ascontiguousarray(coords, np.float64).reshape(-1, 8, 3)
        a = np.zeros((c.shape[0], 12, 3))
        self._check(lib().nalu_hex_scs_determinant(self._h, c.shape[0], _ptr(c), _ptr(a), 0), "hex_scs_determinant")
        return a

    def hex_scs_grad_op(self, coords, shifted=False):
        c = np.ascontiguousarray(coords, np.float64).reshape(-1, 8, 3)
        g, d = np.zeros((c.shape[0], 12, 8, 3)), np.zeros((c.shape[0], 12, 8, 3))
        self._check(lib().nalu_hex_scs_grad_op(self._h, c.shape[0], _ptr(c), int(bool(shifted)), _ptr(g), _ptr(d), 0),
                    "hex_scs_grad_op")
        return g, d

    def hex_scv_grad_op(self, coords, shifted=False):
        c = np.ascontiguousarray(coords, np.float64).reshape(-1, 8, 3)
        g, d = np.zeros((c.shape[0], 8, 8, 3)), np.zeros((c.shape[0], 8, 8, 3))
        self._check(lib().nalu_hex_scv_grad_op(self._h, c.shape[0], _ptr(c), int(bool(shifted)), _ptr(g), _ptr(d), 0),
                    "hex_scv_grad_op")
        return g, d

    def hex_scv_determinant(self, coords):
        c = np.ascontiguousarray(coords, np.float64).reshape(-1, 8, 3)
        v = np.zeros((c.shape[0], 8))
        self._check(lib().nalu_hex_scv_determinant(self._h, c.shape[0], _ptr(c), _ptr(v), 0), "hex_scv_determinant")
        return v

    def hex_face_grad_op(self, coords, side, shifted=False):
        c = np.ascontiguousarray(coords, np.float64).reshape(-1, 8, 3)
        sd = np.ascontiguousarray(side, np.int32)
        g = np.zeros((c.shape[0], 4, 8, 3))
        self._check(lib().nalu_hex_face_grad_op(self._h, c.shape[0], _ptr(sd), _ptr(c), int(bool(shifted)), _ptr(g),
                                                0), "hex_face_grad_op")
        return g

    # boundary faces (side sets)
    def faceset_define(self, set_id, elem, side):
        e = np.ascontiguousarray(elem, np.int64)
        sd = np.ascontiguousarray(side, np.int32)
        if e.shape != sd.shape:
            raise ValueError("elem and side differ in length")
        self._check(lib().nalu_faceset_define(self._h, int(set_id), e.size, _ptr(e), _ptr(sd)), "faceset_define")

    def faceset_skin(self, set_id):
        n = ctypes.c_int64(0)
        self._check(lib().nalu_faceset_skin(self._h, int(set_id), ctypes.byref(n)), "faceset_skin")
        return n.value

    def faceset_get(self, set_id):
        n = ctypes.c_int64(0)
        self._check(lib().nalu_faceset_size(self._h, int(set_id), ctypes.byref(n)), "faceset_size")
        e = np.zeros(n.value, np.int64)
        sd = np.zeros(n.value, np.int32)
        self._check(lib().nalu_faceset_get(self._h, int(set_id), _ptr(e), _ptr(sd)), "faceset_get")
        return e, sd

    def faceset_dynamic_pressure(self, set_id, dynp=None):
        d = None if dynp is None else np.ascontiguousarray(dynp, np.float64)
        self._check(lib().nalu_faceset_dynamic_pressure(self._h, int(set_id), _ptr(d) if d is not None else None),
                    "faceset_dynamic_pressure")

    def faceset_exposed_area(self, set_id):
        n = ctypes.c_int64(0)
        self._check(lib().nalu_faceset_size(self._h, int(set_id), ctypes.byref(n)), "faceset_size")
        a = np.zeros((n.value, 4, 3))
        if n.value:
            self._check(lib().nalu_faceset_exposed_area(self._h, int(set_id), _ptr(a)), "faceset_exposed_area")
        return a

    def nodal_gradient_boundary(self, set_id, src, dst, shifted=False):
        self._check(lib().nalu_nodal_gradient_boundary(self._h, int(set_id), FIELD[src], FIELD[dst],
                                                       int(bool(shifted))), "nodal_gradient_boundary")

    def assemble_faces(self, set_id, kernel, opts=None):
        opts = default_assemble_opts() if opts is None else opts
        self._check(lib().nalu_assemble_faces(self._h, int(set_id), int(kernel), ctypes.byref(opts)),
                    "assemble_faces")

    def capture_face(self, set_id, kernel, face, opts=None):
        opts = default_assemble_opts() if opts is None else opts
        lhs, rhs = np.zeros((8, 8)), np.zeros(8)
        self._check(lib().nalu_capture_face(self._h, int(set_id), int(kernel), ctypes.byref(opts), int(face),
                                            _ptr(lhs), _ptr(rhs)), "capture_face")
        return lhs, rhs

    # solve
    def solve(self, opts=None, raise_on_error=True):
        opts = default_solver_opts() if opts is None else opts
        info = SolveInfo()
        rc = lib().nalu_solve(self._h, ctypes.byref(opts), ctypes.byref(info))
        if raise_on_error:
            self._check(rc, "solve")
        return info

    def set_problems(self, node_offsets):
        """Declare the mesh a union of independent problems (node offsets in row order)."""
        off = np.ascontiguousarray(node_offsets, np.int64)
        self._check(lib().nalu_set_problems(self._h, len(off) - 1, _ptr(off)), "set_problems")
        self._n_problems = len(off) - 1

    def solve_batched(self, opts=None, raise_on_error=True):
        """Jacobi-CG on every problem at once; a list of SolveInfo, one per problem."""
        opts = default_solver_opts() if opts is None else opts
        infos = (SolveInfo * self._n_problems)()
        rc = lib().nalu_solve_batched(self._h, ctypes.byref(opts), infos)
        if raise_on_error:
            self._check(rc, "solve_batched")
        return list(infos)

    # learned preconditioner
    def learned_init(self, seed=0):
        self._check(lib().nalu_learned_init(self._h, int(seed)), "learned_init")

    def learned_set_weights(self, params):
        w = np.ascontiguousarray(params, np.float32)
        self._check(lib().nalu_learned_set_weights(self._h, _ptr(w), w.size), "learned_set_weights")

    def learned_weights(self):
        w = np.zeros(LEARNED_PARAMS, np.float32)
        self._check(lib().nalu_learned_get_weights(self._h, _ptr(w), w.size), "learned_get_weights")
        return w

    def learned_harvest(self, n_samples=20000, n_rhs=4, seed=0, with_rows=False):
        """(static [n,81], residual [n,27], targets [n]) float32 training pairs (+ rows)."""
        st = np.zeros((n_samples, 81), np.float32)
        rf = np.zeros((n_samples, 27), np.float32)
        tg = np.zeros(n_samples, np.float32)
        rows = np.zeros(n_samples, np.int64)
        got = ctypes.c_int64()
        self._check(lib().nalu_learned_harvest(self._h, int(n_rhs), int(seed), int(n_samples), _ptr(st), _ptr(rf),
                                               _ptr(tg), _ptr(rows), ctypes.byref(got)), "learned_harvest")
        k = got.value
        out = (st[:k].copy(), rf[:k].copy(), tg[:k].copy())
        return out + (rows[:k].copy(),) if with_rows else out

    def learned_train(self, st, rf, tg, **kw):
        """Adam on the GPU; returns the [epochs, 2] train / held-out MSE history."""
        o = TrainOpts()
        lib().nalu_train_opts_default(ctypes.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        st, rf, tg = (np.ascontiguousarray(a, np.float32) for a in (st, rf, tg))
        hist = np.zeros((o.epochs, 2), np.float32)
        self._check(lib().nalu_learned_train(self._h, _ptr(st), _ptr(rf), _ptr(tg), tg.size, ctypes.byref(o),
                                             _ptr(hist)), "learned_train")
        return hist

    def learned_gradient(self, st, rf, tg, precision=None):
        """loss and gradient at the current weights: the FP32 path (default)
        or the fused BF16 tensor-core step (precision=TRAIN_BF16)"""
        st, rf, tg = (np.ascontiguousarray(a, np.float32) for a in (st, rf, tg))
        g = np.zeros(LEARNED_PARAMS, np.float32)
        loss = ctypes.c_double()
        fn = lib().nalu_learned_gradient_bf16 if precision == TRAIN_BF16 else lib().nalu_learned_gradient
        self._check(fn(self._h, _ptr(st), _ptr(rf), _ptr(tg), tg.size, _ptr(g), ctypes.byref(loss)),
                    "learned_gradient")
        return loss.value, g

    def learned_stencil(self):
        nr, _, _ = self.sizes()
        c = np.zeros((nr, 27), np.float32)
        self._check(lib().nalu_learned_stencil(self._h, _ptr(c)), "learned_stencil")
        return c

    def solution(self):
        nr, _, _ = self.sizes()
        x = np.zeros(nr)
        self._check(lib().nalu_solution_get(self._h, _ptr(x), 0), "solution_get")
        return x

    def spmv(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self._check(lib().nalu_spmv(self._h, _ptr(x), _ptr(y), 0), "spmv")
        return y

    def synchronize(self):
        self._check(lib().nalu_synchronize(self._h), "synchronize")

    def launches(self):
        return lib().nalu_kernel_launch_count(self._h)

    def last_assemble_ms(self):
        return lib().nalu_last_assemble_ms(self._h)

    def probe_fp64_tflops(self):
        t = ctypes.c_double()
        self._check(lib().nalu_probe_fp64_tflops(self._h, ctypes.byref(t)), "probe")
        return t.value

    def event_record(self, slot):
        self._check(lib().nalu_event_record(self._h, slot), "event_record")

    def event_elapsed_ms(self, a, b):
        t = ctypes.c_double()
        self._check(lib().nalu_event_elapsed_ms(self._h, a, b, ctypes.byref(t)), "event_elapsed")
        return t.value

    def flush_l2(self, nbytes=512 << 20):
        self._check(lib().nalu_flush_l2(self._h, nbytes), "flush_l2")

    # raw pointer variants (pinned host buffers)
    def field_set_async_ptr(self, name, ptr, count):
        """staged upload from (pinned) host memory; swapped in by the next call that reads fields"""
        self._check(lib().nalu_field_set_async(self._h, FIELD[name], ptr, count), "field_set_async(%s)" % name)

    def field_set_ptr(self, name, ptr, count):
        self._check(lib().nalu_field_set(self._h, FIELD[name], ptr, count, 0), "field_set(%s)" % name)

    def system_to_ptr(self, values_ptr, rhs_ptr):
        self._check(lib().nalu_linsys_copy(self._h, values_ptr, rhs_ptr, 0), "copy")

    def system_to_ptr_async(self, values_ptr, rhs_ptr):
        """Start the download of values/rhs into pinned host memory; returns at once."""
        self._check(lib().nalu_linsys_copy_async(self._h, values_ptr, rhs_ptr), "copy_async")

    def copy_wait(self):
        self._check(lib().nalu_linsys_copy_wait(self._h), "copy_wait")


class PinnedArray:
    """numpy view of page-locked host memory from nalu_host_alloc."""

    def __init__(self, shape, dtype=np.float64):
        dt = np.dtype(dtype)
        n = int(np.prod(shape))
        self._p = ctypes.c_void_p()
        rc = lib().nalu_host_alloc(max(n * dt.itemsize, 1), ctypes.byref(self._p))
        if rc:
            raise NaluError(rc, "nalu_host_alloc")
        buf = (ctypes.c_char * (n * dt.itemsize)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=dt, count=n).reshape(shape)

    @property
    def ptr(self):
        return self._p

    def free(self):
        if self._p:
            self.array = None
            lib().nalu_host_free(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


from .linear_system import (AssembleElemSolverAlgorithm, ContinuityAdvElemKernel, LinearSystem,  # noqa: E402
                            MomentumAdvDiffElemKernel, MomentumUpwAdvDiffElemKernel, ScalarDiffElemKernel)
