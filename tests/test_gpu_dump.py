"""MatrixMarket dumps of the system and solution (TpetraLinearSystem::
writeToFile / writeSolutionToFile): file names with the write counter,
1-based global row/column ids ndof (gid - 1) + idof + 1, and values that read
back bit for bit."""
import os

import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import block_mesh

pytestmark = pytest.mark.gpu


@pytest.mark.filterwarnings("ignore::DeprecationWarning")  # scipy's mmread return-type notice
@pytest.mark.parametrize("num_dof", [1, 3])
def test_write_system_and_solution(gpu_ctx_factory, tmp_path, num_dof):
    sio = pytest.importorskip("scipy.io")
    c, conn, gid = block_mesh(4, 3, 3, jitter=0.2, seed=2)
    n = c.shape[0]
    gid = (gid[::-1] + 10).copy()          # global ids 11.., reversed against the caller order
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    rng = np.random.default_rng(4)
    ctx.field_set("density", 1.0 + 0.1 * rng.random(n))
    ctx.field_set("density_n", np.ones(n))
    ctx.build_elem_graph(num_dof)
    ctx.zero()
    if num_dof == 1:
        ctx.field_set("velocity", rng.standard_normal((n, 3)))
        ctx.field_set("pressure", rng.standard_normal(n))
        ctx.field_set("dpdx", np.zeros((n, 3)))
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
    else:
        ctx.field_set("velocity", rng.standard_normal((n, 3)))
        ctx.field_set("velocity_n", rng.standard_normal((n, 3)))
        ctx.field_set("dpdx", rng.standard_normal((n, 3)))
        ctx.assemble(ng.KERNEL_MOMENTUM_MASS, ng.default_assemble_opts(dt=0.1))
    vals, rhs = ctx.system()
    rp, ci = ctx.graph()
    base = os.path.join(str(tmp_path), "sys")
    ctx.write_system(base)
    A = sio.mmread(base + "-O-0.mm.1").tocsr()
    b = np.asarray(sio.mmread(base + "-O-0.rhs.1")).ravel()
    # LID -> global row id; nodes in LID order are sorted by global id
    gsorted = np.sort(gid)
    lid_gid = num_dof * (np.repeat(gsorted, num_dof) - 1) + np.tile(np.arange(num_dof), n) + 1
    nr = rp.shape[0] - 1
    dim = int(lid_gid.max())                # the largest global row id
    assert A.shape == (dim, dim) and A.nnz == ci.shape[0]
    rows = np.repeat(np.arange(nr), np.diff(rp))
    # entry (GID_r, GID_c), 1-based in the file
    from scipy.sparse import coo_matrix
    want = coo_matrix((vals, (lid_gid[rows] - 1, lid_gid[ci] - 1)), shape=(dim, dim)).tocsr()
    assert np.array_equal(A.indptr, want.indptr) and np.array_equal(A.indices, want.indices)
    assert np.array_equal(A.data, want.data)
    assert np.array_equal(b, rhs)
    # the solution file advances the counter
    ctx.solve(ng.default_solver_opts(method=ng.SOLVER_GMRES, tol=1e-10, max_iters=60), raise_on_error=False)
    x = ctx.solution()
    ctx.write_solution(base)
    s = np.asarray(sio.mmread(base + "-O-0.sln.1")).ravel()
    assert np.array_equal(s, x)
    ctx.write_system(base)
    assert os.path.exists(base + "-O-1.mm.1") and os.path.exists(base + "-O-1.rhs.1")
    ctx.close()
