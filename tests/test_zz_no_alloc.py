"""nalu_pcg_jacobi_noalloc: the Jacobi-CG entry point that allocates no
device memory, for callers that own all device memory themselves (their own
pool allocator) or must not allocate inside a time-step loop.

It is called through the C ABI on a system assembled by the library, twice in
a row on the same buffers (its scratch array keeps the previous call's
contents), and each result is checked against nalu_solve's Jacobi-CG with the
tolerances the solver tests use: true FP64 relative residual <= 1e-8 and the
solution within 1e-4 of the largest entry.  This file sorts last so that a
stop-at-first-failure run has executed every other test before it.
"""
import ctypes

import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import block_mesh

pytestmark = pytest.mark.gpu


def _heat_system(N=40):
    c, conn, gid = block_mesh(N, jitter=0.1, seed=31)
    n = c.shape[0]
    T = np.random.default_rng(32).uniform(0, 1, n)
    ctx = ng.Context(0)
    ctx.mesh_create(c, conn, gid)
    ctx.field_set("scalar_q", T)
    ctx.field_set("diff_coeff", np.ones(n))
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_SCALAR_DIFF, ng.default_assemble_opts(scatter=ng.SCATTER_COLOURED))
    left, right = np.where(c[:, 0] == 0.0)[0], np.where(c[:, 0] == 1.0)[0]
    nodes = np.concatenate([left, right])
    ctx.apply_dirichlet(nodes, np.concatenate([np.zeros(left.size), np.ones(right.size)]), T[nodes])
    ctx.load_complete()
    return ctx


def test_noalloc_pcg_matches_nalu_solve(oracle):
    L = ng.lib()
    f = L.nalu_pcg_jacobi_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 5 + [ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                                             ctypes.c_void_p, ctypes.c_void_p]
    ctx = _heat_system()
    n, nnz, _ = ctx.sizes()
    info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=20000))
    x_ref = ctx.solution()
    assert info.true_rel_res <= 1e-8
    rp_d, ci_d, v_d, b_d, x_d = (ctypes.c_void_p() for _ in range(5))
    assert L.nalu_linsys_device_arrays(ctx.handle, ctypes.byref(rp_d), ctypes.byref(ci_d), ctypes.byref(v_d),
                                       ctypes.byref(b_d), ctypes.byref(x_d)) == 0
    stream = ctypes.c_void_p()
    assert L.nalu_get_stream(ctx.handle, ctypes.byref(stream)) == 0
    rp, ci = ctx.graph()
    vals, b = ctx.system()
    for call in range(2):
        iters, res = ctypes.c_int(), ctypes.c_double()
        rc = f(n, rp_d, ci_d, v_d, b_d, x_d, 1e-8, 20000, ctypes.byref(iters), ctypes.byref(res), stream)
        assert rc == 0, "call %d returned %d" % (call, rc)
        x = ctx.solution()
        true_res = np.linalg.norm(b - oracle.spmv(rp, ci, vals, x)) / np.linalg.norm(b)
        assert res.value <= 1e-8 and true_res <= 1.05e-8, (call, res.value, true_res)
        assert np.max(np.abs(x - x_ref)) <= 1e-4 * np.max(np.abs(x_ref)), call
        assert iters.value > 0
    ctx.close()


def test_noalloc_rejects_oversize_and_bad_args():
    L = ng.lib()
    f = L.nalu_pcg_jacobi_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 5 + [ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                                             ctypes.c_void_p, ctypes.c_void_p]
    dummy = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    assert f(262145, dummy, dummy, dummy, dummy, dummy, 1e-8, 10, None, None, None) == -6
    assert f(0, dummy, dummy, dummy, dummy, dummy, 1e-8, 10, None, None, None) == -1
    assert f(100, None, dummy, dummy, dummy, dummy, 1e-8, 10, None, None, None) == -1


# ---------------------------------------------------------------------------
# systems built on the host (scipy) and placed in device memory with torch
# (device-memory plumbing only): the 3-dof (wide-row) path, exact one-step
# convergence, the iteration cap and the largest supported size
# ---------------------------------------------------------------------------
def _noalloc_fn():
    L = ng.lib()
    f = L.nalu_pcg_jacobi_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 5 + [ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                                             ctypes.c_void_p, ctypes.c_void_p]
    return f


def _fem27(m):
    """27-point trilinear-FEM Laplacian on an m^3 grid of interior nodes (SPD)"""
    sp = pytest.importorskip("scipy.sparse")
    k1 = sp.diags([-np.ones(m - 1), 2 * np.ones(m), -np.ones(m - 1)], [-1, 0, 1])
    m1 = sp.diags([np.ones(m - 1), 4 * np.ones(m), np.ones(m - 1)], [-1, 0, 1]) / 6.0
    a = sp.kron(sp.kron(k1, m1), m1) + sp.kron(sp.kron(m1, k1), m1) + sp.kron(sp.kron(m1, m1), k1)
    return sp.csr_matrix(a)


def _solve_noalloc(a, b, tol=1e-8, max_iters=20000, calls=1):
    torch = pytest.importorskip("torch")
    a.sort_indices()
    dev = torch.device("cuda", 0)
    rp = torch.tensor(a.indptr.astype(np.int64), device=dev)
    ci = torch.tensor(a.indices.astype(np.int32), device=dev)
    v = torch.tensor(a.data.astype(np.float64), device=dev)
    bd = torch.tensor(b, dtype=torch.float64, device=dev)
    xd = torch.zeros(a.shape[0], dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    f = _noalloc_fn()
    out = []
    for _ in range(calls):
        iters, res = ctypes.c_int(), ctypes.c_double()
        rc = f(a.shape[0], rp.data_ptr(), ci.data_ptr(), v.data_ptr(), bd.data_ptr(), xd.data_ptr(), tol,
               max_iters, ctypes.byref(iters), ctypes.byref(res), None)
        out.append((rc, iters.value, res.value, xd.cpu().numpy().copy()))
    return out


def test_noalloc_three_dof_rows():
    """81 entries per row (node-column triples, the 16-threads-per-row SpMV)"""
    sp = pytest.importorskip("scipy.sparse")
    a = sp.csr_matrix(sp.kron(_fem27(16), np.array([[2.0, 0.5, 0.25], [0.5, 2.0, 0.5], [0.25, 0.5, 2.0]])))
    assert a.nnz > 40 * a.shape[0]
    b = np.random.default_rng(3).normal(size=a.shape[0])
    for rc, its, res, x in _solve_noalloc(a, b, calls=2):
        assert rc == 0 and res <= 1e-8 and its > 0
        assert np.linalg.norm(b - a @ x) <= 1.05e-8 * np.linalg.norm(b)


def test_noalloc_exact_one_step_convergence():
    """a diagonal system with power-of-two entries is solved exactly by one
    Jacobi-CG step; the chunk's remaining steps are frozen, not 0/0"""
    sp = pytest.importorskip("scipy.sparse")
    d = 2.0 ** np.random.default_rng(4).integers(-3, 4, 5000)
    a = sp.csr_matrix(sp.diags(d))
    b = np.random.default_rng(5).normal(size=d.size)
    for rc, its, res, x in _solve_noalloc(a, b, calls=2):
        assert rc == 0, rc
        assert its == 1, its
        np.testing.assert_allclose(x, b / d, rtol=1e-14, atol=0)


def test_noalloc_iteration_cap_and_largest_size():
    """n = 262,144 rows (the static array's capacity): max_iters = 5 reports
    NALU_ERR_NOT_CONVERGED with 5 iterations; a full solve then converges"""
    a = _fem27(64)
    assert a.shape[0] == 262144
    b = np.random.default_rng(6).normal(size=a.shape[0])
    (rc, its, res, _), = _solve_noalloc(a, b, max_iters=5)
    assert rc == -7 and its == 5 and res > 1e-8
    (rc, its, res, x), = _solve_noalloc(a, b)
    assert rc == 0 and res <= 1e-8
    assert np.linalg.norm(b - a @ x) <= 1.05e-8 * np.linalg.norm(b)
