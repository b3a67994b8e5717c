"""Batches of independent continuity problems in one context: one assembly
launch over the union mesh, then one persistent Jacobi-CG launch with a
separate alpha, beta and stop test per problem.  Each problem's solution must
reach the tolerance on its own rows (checked with the oracle's FP64 SpMV on
the problem's diagonal block) and agree with the oracle's CG on that block."""
import numpy as np
import pytest

import nalu_gb300 as ng
from nalu_gb300.meshgen import batch_block_meshes, fourier_velocity

pytestmark = pytest.mark.gpu


def _batched_continuity(gpu_ctx_factory, n_problems, edge_range, seed):
    c, conn, gid, off, edges = batch_block_meshes(n_problems, edge_range=edge_range, seed=seed)
    n = c.shape[0]
    u = np.concatenate([fourier_velocity(c[off[k]:off[k + 1]], n_modes=16, seed=seed + 100 + k)
                        for k in range(n_problems)])
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    ctx.field_set("velocity", u)
    ctx.field_set("density", np.ones(n))
    ctx.field_set("pressure", np.zeros(n))
    ctx.field_set("dpdx", np.zeros((n, 3)))
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
    # one pinned pressure node per problem (FixPressureAtNodeAlgorithm)
    pins = off[:-1]
    ctx.reset_rows(pins)
    for p in pins:
        ctx.sum_into_diag(int(p), 0, 1.0, 0.0)
    ctx.load_complete()
    ctx.set_problems(off)
    return ctx, off, edges


def _block(rp, ci, v, b, r0, r1):
    """Diagonal block [r0, r1) of a CRS matrix (the graph is block diagonal)."""
    s, e = rp[r0], rp[r1]
    assert ci[s:e].min() >= r0 and ci[s:e].max() < r1
    return rp[r0:r1 + 1] - s, ci[s:e] - r0, v[s:e], b[r0:r1]


def test_batched_cg_per_problem(gpu_ctx_factory, oracle):
    ctx, off, _ = _batched_continuity(gpu_ctx_factory, 6, (5, 14), seed=11)
    rp, ci = ctx.graph()
    v, b = ctx.system()
    infos = ctx.solve_batched(ng.default_solver_opts(tol=1e-10, max_iters=5000))
    x = ctx.solution()
    assert len(infos) == 6
    for k, info in enumerate(infos):
        r0, r1 = int(off[k]), int(off[k + 1])
        brp, bci, bv, bb = _block(rp, ci, v, b, r0, r1)
        xk = x[r0:r1]
        res = np.linalg.norm(bb - oracle.spmv(brp, bci, bv, xk)) / np.linalg.norm(bb)
        assert info.status == 0 and info.true_rel_res <= 1e-10 and res <= 1.05e-10, (k, info.true_rel_res, res)
        xo, it, _ = oracle.pcg_jacobi(brp, bci, bv, bb, tol=1e-12, max_it=20000, n_threads=4)
        assert np.max(np.abs(xk - xo)) <= 1e-6 * max(np.max(np.abs(xo)), 1e-30), k
        # same algorithm on the same block: iteration counts stay close
        assert 0 < info.iterations <= 2 * it + 10, (k, info.iterations, it)
    ctx.close()


def test_batched_matches_union_solve(gpu_ctx_factory):
    """The batched solve and one CG over the whole block-diagonal system give
    the same solution to within the tolerance's error bound."""
    ctx, off, _ = _batched_continuity(gpu_ctx_factory, 4, (6, 12), seed=12)
    infos = ctx.solve_batched(ng.default_solver_opts(tol=1e-10, max_iters=5000))
    xb = ctx.solution()
    info = ctx.solve(ng.default_solver_opts(tol=1e-10, max_iters=20000))
    xu = ctx.solution()
    assert info.true_rel_res <= 1e-10
    assert all(i.status == 0 for i in infos)
    for k in range(4):
        r0, r1 = int(off[k]), int(off[k + 1])
        scale = np.max(np.abs(xu[r0:r1]))
        assert np.max(np.abs(xb[r0:r1] - xu[r0:r1])) <= 1e-5 * scale, k
    ctx.close()


def test_batched_graph_block_diagonal(gpu_ctx_factory, oracle):
    """Union graph = the per-problem graphs placed on the diagonal (bit-exact)."""
    c, conn, gid, off, _ = batch_block_meshes(3, edge_range=(3, 7), seed=13)
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    ctx.build_elem_graph(1)
    rp, ci = ctx.graph()
    e0 = 0
    for k in range(3):
        r0, r1 = int(off[k]), int(off[k + 1])
        sub = conn[(conn >= r0).all(1) & (conn < r1).all(1)] - r0
        orp, oci, _ = oracle.graph(r1 - r0, sub, 1, gid[r0:r1] - r0)
        brp = rp[r0:r1 + 1] - rp[r0]
        np.testing.assert_array_equal(brp, orp)
        np.testing.assert_array_equal(ci[rp[r0]:rp[r1]] - r0, oci)
        e0 += sub.shape[0]
    assert e0 == conn.shape[0]
    ctx.set_problems(off)
    ctx.close()


def test_set_problems_rejects_coupled_split(gpu_ctx_factory):
    c, conn, gid, off, _ = batch_block_meshes(2, edge_range=(4, 6), seed=14)
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    ctx.build_elem_graph(1)
    with pytest.raises(RuntimeError):
        ctx.set_problems([0, int(off[1]) // 2, int(off[-1])])  # cuts problem 0 in half
    with pytest.raises(RuntimeError):
        ctx.set_problems([0, int(off[-1]) + 1])  # does not span the nodes
    ctx.set_problems(off)
    ctx.close()


def _check_batch_solution(ctx, oracle, off, infos, tol, rp, ci, v, b):
    x = ctx.solution()
    for k, info in enumerate(infos):
        r0, r1 = int(off[k]), int(off[k + 1])
        brp, bci, bv, bb = _block(rp, ci, v, b, r0, r1)
        res = np.linalg.norm(bb - oracle.spmv(brp, bci, bv, x[r0:r1])) / np.linalg.norm(bb)
        assert info.status == 0 and res <= 1.05 * tol, (k, info.status, res)
        xo, _, _ = oracle.pcg_jacobi(brp, bci, bv, bb, tol=1e-13, max_it=20000, n_threads=4)
        assert np.max(np.abs(x[r0:r1] - xo)) <= 1e-5 * np.max(np.abs(xo)), k


@pytest.mark.parametrize("probe", [1, 0])
def test_batched_learned_fcg(gpu_ctx_factory, oracle, probe):
    """The learned preconditioner on a batch (weights trained on the union
    system).  With the probe, every problem opens with Jacobi-CG; the learned
    preconditioner is set up and tried only on problems with many iterations
    left, first on the largest, and the rest follow only if it wins there, so a
    batch that keeps Jacobi-CG runs learned iterations on one problem at most.
    Without the probe every problem runs the learned FCG from the start.  Every
    problem reaches the tolerance on its own rows and agrees with the oracle."""
    ctx, off, _ = _batched_continuity(gpu_ctx_factory, 6, (12, 24), seed=21)
    rp, ci = ctx.graph()
    v, b = ctx.system()
    tol = 1e-11
    plain = ctx.solve_batched(ng.default_solver_opts(tol=tol, max_iters=5000))
    ctx.learned_init(3)
    st, rf, tg = ctx.learned_harvest(n_samples=20000, n_rhs=4, seed=4)
    ctx.learned_train(st, rf, tg, epochs=30)
    infos = ctx.solve_batched(ng.default_solver_opts(tol=tol, max_iters=5000, precond=ng.PRECOND_LEARNED,
                                                     learned_probe=probe))
    _check_batch_solution(ctx, oracle, off, infos, tol, rp, ci, v, b)
    print("plain iterations", [i.iterations for i in plain])
    print("learned: iterations", [i.iterations for i in infos], "learned", [i.learned_iterations for i in infos],
          "fallback", [i.fallback for i in infos])
    tried = [i for i in infos if i.learned_iterations > 0]
    if probe:
        assert all(i.fallback in (0, 1, 2) for i in infos)
        assert all(i.fallback == 2 for i in infos if i.learned_iterations == 0)
        if not any(i.fallback == 0 for i in infos):
            assert len(tried) <= 1
        # the Jacobi-CG iterations of the opening run are shared with the solve:
        # a problem that never left Jacobi-CG takes its plain iteration count
        # (restarts aside)
        for i, p in zip(infos, plain):
            if i.learned_iterations == 0:
                assert i.iterations <= p.iterations + 60, (i.iterations, p.iterations)
    else:
        assert len(tried) == len(infos) and all(i.fallback in (0, 1) for i in infos)
    ctx.close()


def test_batched_multilevel_fcg(gpu_ctx_factory, oracle):
    """The multigrid preconditioner on a batch: one hierarchy for the union
    (block diagonal, so the V-cycle is each problem's own preconditioner) and
    flexible CG with per-problem scalars and stop tests.  Every problem
    reaches the tolerance on its own rows, agrees with the oracle, and takes
    far fewer iterations than Jacobi-CG."""
    ctx, off, _ = _batched_continuity(gpu_ctx_factory, 6, (12, 24), seed=21)
    rp, ci = ctx.graph()
    v, b = ctx.system()
    tol = 1e-10
    plain = ctx.solve_batched(ng.default_solver_opts(tol=tol, max_iters=5000))
    infos = ctx.solve_batched(ng.default_solver_opts(tol=tol, max_iters=5000, precond=ng.PRECOND_MULTILEVEL))
    _check_batch_solution(ctx, oracle, off, infos, tol, rp, ci, v, b)
    print("Jacobi-CG iterations", [i.iterations for i in plain])
    print("multigrid FCG iterations", [i.iterations for i in infos], "set-up %.1f ms" % (1e3 * infos[0].setup_seconds))
    for i, p in zip(infos, plain):
        assert i.fallback == 0 and i.learned_iterations == i.iterations
        assert 3 * i.iterations <= p.iterations, (i.iterations, p.iterations)
    ctx.close()


def test_batch_tile_autotune(gpu_ctx_factory, oracle):
    """The tile-size autotuner times every candidate, keeps the fastest, and
    the batched solve with the chosen tiles still meets the tolerance on every
    problem (tiles never cross a problem, whatever their size)."""
    ctx, off, _ = _batched_continuity(gpu_ctx_factory, 5, (10, 20), seed=22)
    rp, ci = ctx.graph()
    v, b = ctx.system()
    rows, ms = ctx.batch_autotune(50)
    print("rows per tile", rows, ms)
    assert rows in ms and all(t > 0 for t in ms.values())
    assert ms[rows] == min(ms.values())
    tol = 1e-10
    infos = ctx.solve_batched(ng.default_solver_opts(tol=tol, max_iters=5000))
    _check_batch_solution(ctx, oracle, off, infos, tol, rp, ci, v, b)
    # max_iters bounds the total over restarts
    short = ctx.solve_batched(ng.default_solver_opts(tol=tol, max_iters=30), raise_on_error=False)
    assert all(i.iterations <= 50 for i in short)
    ctx.close()
