"""GPU: the aggregation multigrid preconditioner in flexible CG
(NALU_PRECOND_MULTILEVEL with damped Jacobi smoothing, and
NALU_PRECOND_LEARNED_MULTILEVEL with the learned stencil as the fine-level
smoother).  Every solve is judged by the oracle's FP64 residual
||b - A x|| / ||b|| <= 1e-8 (1.05e-8 allowed for the summation order), and its
solution is compared with the oracle's Jacobi-PCG solution (1e-4 of the
largest entry, the bound of the other solver tests)."""
import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import block_mesh

pytestmark = pytest.mark.gpu


def _continuity_system(N, z_ratio=1.05, jitter=0.0, seed=3):
    c, conn, gid = block_mesh(N, z_ratio=z_ratio, jitter=jitter, seed=seed)
    n = c.shape[0]
    u = ng.meshgen.fourier_velocity(c, n_modes=16, seed=seed)
    ctx = ng.Context(0)
    ctx.mesh_create(c, conn, gid)
    for nm, v in (("velocity", u), ("density", np.ones(n)), ("pressure", np.zeros(n)), ("dpdx", np.zeros((n, 3)))):
        ctx.field_set(nm, v)
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
    ctx.reset_rows([0])
    ctx.sum_into_diag(0, 0, 1.0, 0.0)
    ctx.load_complete()
    return ctx


def _check_solution(ctx, oracle, info, x_ref=None):
    rp, ci = ctx.graph()
    vals, b = ctx.system()
    x = ctx.solution()
    res = np.linalg.norm(b - oracle.spmv(rp, ci, vals, x, n_threads=8)) / np.linalg.norm(b)
    assert info.status == 0 and res <= 1.05e-8, (info.status, res)
    if x_ref is not None:
        assert np.max(np.abs(x - x_ref)) <= 1e-4 * np.max(np.abs(x_ref))
    return res


@pytest.mark.parametrize("N,z_ratio,jitter", [(24, 1.05, 0.0), (32, 1.0, 0.1), (40, 1.1, 0.0)])
def test_multilevel_jacobi_solves(oracle, N, z_ratio, jitter):
    ctx = _continuity_system(N, z_ratio, jitter)
    rp, ci = ctx.graph()
    vals, b = ctx.system()
    x_ref, _, _ = oracle.pcg_jacobi(rp, ci, vals, b, tol=1e-12, max_it=50000, n_threads=8)
    plain = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=50000))
    for kl in (0, 1, 100):  # V-cycle, K-cycle on the first coarse level, on every coarse level
        info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=2000, precond=ng.PRECOND_MULTILEVEL,
                                                ml_kcycle_levels=kl))
        res = _check_solution(ctx, oracle, info, x_ref)
        rows, nnz = ctx.multilevel_levels()
        print("N=%d ratio=%g jitter=%g K-levels %d: levels %s, iterations %d (Jacobi-PCG %d), residual %.2e"
              % (N, z_ratio, jitter, kl, rows, info.iterations, plain.iterations, res))
        assert len(rows) >= 2 and rows[0] == ctx.sizes()[0]
        # three pairwise passes per level coarsen by 3 or more; the coarsest
        # level may come from fewer passes (it stops at 256 rows)
        assert all(rows[k + 1] * 3 <= rows[k] for k in range(len(rows) - 2)), rows
        assert rows[-1] < rows[-2]
        assert rows[-1] <= 1024
        assert info.iterations * 3 <= plain.iterations
    ctx.close()


def test_learned_multilevel_solves_and_gain(oracle):
    """The learned stencil (trained on this system's PCG first directions) as
    the fine-level smoother: the solve reaches 1e-8, and its iteration count
    is reported beside the Jacobi-smoothed one (what the network gains)."""
    ctx = _continuity_system(32, 1.05, 0.0)
    ctx.learned_init(7)
    st, rf, tg = ctx.learned_harvest(n_samples=4000, n_rhs=2, seed=11)
    ctx.learned_train(st, rf, tg, epochs=20)
    rp, ci = ctx.graph()
    vals, b = ctx.system()
    x_ref, _, _ = oracle.pcg_jacobi(rp, ci, vals, b, tol=1e-12, max_it=50000, n_threads=8)
    jac = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=2000, precond=ng.PRECOND_MULTILEVEL))
    _check_solution(ctx, oracle, jac, x_ref)
    for sweeps in (0, 1, 2, 3):  # default (pre-smoothing), pre, post, both
        lrn = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=2000, precond=ng.PRECOND_LEARNED_MULTILEVEL,
                                               ml_learned_sweeps=sweeps))
        _check_solution(ctx, oracle, lrn, x_ref)
        print("32^3: multilevel iterations Jacobi-smoothed %d, learned-smoothed (sweeps %d) %d"
              % (jac.iterations, sweeps, lrn.iterations))
        assert lrn.iterations <= 2 * jac.iterations
    ctx.close()


def test_multilevel_heat_dirichlet(oracle):
    """Heat conduction with Dirichlet rows (identity rows, their columns kept:
    a non-symmetric matrix), jittered mesh."""
    c, conn, gid = block_mesh(28, jitter=0.1, seed=5)
    n = c.shape[0]
    T = np.random.default_rng(6).uniform(0, 1, n)
    ctx = ng.Context(0)
    ctx.mesh_create(c, conn, gid)
    ctx.field_set("scalar_q", T)
    ctx.field_set("diff_coeff", np.ones(n))
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_SCALAR_DIFF)
    left, right = np.where(c[:, 0] == 0.0)[0], np.where(c[:, 0] == 1.0)[0]
    nodes = np.concatenate([left, right])
    ctx.apply_dirichlet(nodes, np.concatenate([np.zeros(left.size), np.ones(right.size)]), T[nodes])
    ctx.load_complete()
    info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=2000, precond=ng.PRECOND_MULTILEVEL))
    _check_solution(ctx, oracle, info)
    ctx.close()


def test_multilevel_small_system_single_level(oracle):
    """A system below the coarsest size (6^3 nodes) is one dense level: the
    preconditioner is its inverse and flexible CG converges at once."""
    ctx = _continuity_system(5, 1.05)
    info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=200, precond=ng.PRECOND_MULTILEVEL))
    _check_solution(ctx, oracle, info)
    rows, _ = ctx.multilevel_levels()
    assert rows == [216] and info.iterations <= 5
    ctx.close()


def test_multilevel_rejects_unsupported():
    ctx = _continuity_system(8)
    with pytest.raises(ng.NaluError) as ei:
        ctx.solve(ng.default_solver_opts(method=ng.SOLVER_GMRES, precond=ng.PRECOND_MULTILEVEL))
    assert ei.value.status == -1
    with pytest.raises(ng.NaluError) as ei:
        ctx.solve(ng.default_solver_opts(precision=ng.PRECISION_FP32_INNER_IR, precond=ng.PRECOND_MULTILEVEL))
    assert ei.value.status == -1
    ctx.close()
