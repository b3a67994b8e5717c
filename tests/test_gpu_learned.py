"""Learned preconditioner on the GPU: the training gradient and the BF16
tensor-core stencil against the FP64 numpy reference model, the harvested
features against host-computed ones, and flexible CG with the learned
stencil (convergence, fewer iterations than Jacobi-PCG, and the
Chebyshev-Jacobi fallback after a stall)."""
import numpy as np
import pytest

import mlp_ref as M
import nalu_gb300 as ng
from helpers import block_mesh
from nalu_gb300.meshgen import fourier_velocity

pytestmark = pytest.mark.gpu


def _continuity(gpu_ctx_factory, N, seed=1, jitter=0.0):
    c, conn, gid = block_mesh(N, z_ratio=1.05, jitter=jitter, seed=seed)
    n = c.shape[0]
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    ctx.field_set("velocity", fourier_velocity(c, n_modes=64, seed=seed))
    ctx.field_set("density", np.ones(n))
    ctx.field_set("pressure", np.zeros(n))
    ctx.field_set("dpdx", np.zeros((n, 3)))
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
    ctx.reset_rows([0])
    ctx.sum_into_diag(0, 0, 1.0, 0.0)
    ctx.load_complete()
    return ctx, c, conn


def test_learned_gradient_matches_reference(gpu_ctx_factory):
    ctx = gpu_ctx_factory()
    P = M.random_params(11).astype(np.float32)
    ctx.learned_set_weights(P)
    st, rf, tg = (a.astype(np.float32) for a in M.random_samples(96, 12))
    loss, g = ctx.learned_gradient(st, rf, tg)
    lref, gref = M.loss_and_grad(P.astype(np.float64), st, rf, tg)
    assert abs(loss - lref) <= 1e-4 * lref
    for k, (o, s) in M.SL.items():
        sl = slice(o, o + int(np.prod(s)))
        err = np.linalg.norm(g[sl] - gref[sl])
        assert err <= 2e-4 * np.linalg.norm(gref[sl]) + 1e-7, (k, err, np.linalg.norm(gref[sl]))
    ctx.close()


@pytest.mark.parametrize("n", [96, 1001])
def test_learned_gradient_bf16_matches_reference(gpu_ctx_factory, n):
    """The fused tensor-core training step (BF16 weights and activations, FP32
    accumulation, one warp per sample, four samples per block; 1001 leaves a
    partial block) against the FP64 numpy model.  Declared BF16 bound: every
    parameter block within 3% of the reference gradient's norm, the loss
    within 1%."""
    ctx = gpu_ctx_factory()
    P = M.random_params(11).astype(np.float32)
    ctx.learned_set_weights(P)
    st, rf, tg = (a.astype(np.float32) for a in M.random_samples(n, 12))
    loss, g = ctx.learned_gradient(st, rf, tg, precision=ng.TRAIN_BF16)
    lref, gref = M.loss_and_grad(P.astype(np.float64), st, rf, tg)
    assert abs(loss - lref) <= 1e-2 * lref, (loss, lref)
    for k, (o, s) in M.SL.items():
        sl = slice(o, o + int(np.prod(s)))
        err = np.linalg.norm(g[sl] - gref[sl])
        assert err <= 3e-2 * np.linalg.norm(gref[sl]) + 1e-6, (k, err, np.linalg.norm(gref[sl]))
    # deterministic: fixed-order sums, no atomics
    loss2, g2 = ctx.learned_gradient(st, rf, tg, precision=ng.TRAIN_BF16)
    assert loss2 == loss and np.array_equal(g, g2)
    ctx.close()


def test_learned_train_bf16_tracks_fp32(gpu_ctx_factory):
    """Training on harvested pairs from the same initial weights: the
    tensor-core path reaches a held-out loss within 10% of the FP32 path's
    (and both at most half the initial one), and is faster."""
    import time
    ctx, _, _ = _continuity(gpu_ctx_factory, 20)
    ctx.learned_init(1)
    st, rf, tg = ctx.learned_harvest(n_samples=20000, n_rhs=4, seed=2)
    res = {}
    for prec in (ng.TRAIN_FP32, ng.TRAIN_BF16):
        ctx.learned_init(1)
        ctx.synchronize()
        t0 = time.perf_counter()
        hist = ctx.learned_train(st, rf, tg, epochs=20, precision=prec)
        res[prec] = (hist, time.perf_counter() - t0)
    (hf, tf), (hb, tb) = res[ng.TRAIN_FP32], res[ng.TRAIN_BF16]
    print("held-out loss FP32 %.4g -> %.4g (%.3f s), BF16 %.4g -> %.4g (%.3f s)"
          % (hf[0, 1], hf[-1, 1], tf, hb[0, 1], hb[-1, 1], tb))
    assert hb[-1, 1] <= 1.1 * hf[-1, 1] and hb[-1, 1] <= 0.5 * hb[0, 1], (hf[[0, -1]], hb[[0, -1]])
    assert tb < tf
    ctx.close()


def test_learned_stencil_matches_reference(gpu_ctx_factory):
    ctx, c, conn = _continuity(gpu_ctx_factory, 10)
    P = M.random_params(13).astype(np.float32)
    ctx.learned_set_weights(P)
    sten = ctx.learned_stencil()
    rp, ci = ctx.graph()
    v, _ = ctx.system()
    nbr = M.slot_map(conn, c.shape[0])
    st, _ = M.static_features(rp, ci, v, nbr)
    ref = M.stencil(P.astype(np.float64), st)
    ref[0] = 0.0  # the pinned row is an identity row
    # BF16 weights and activations, FP32 accumulation
    err = np.abs(sten - ref)
    assert np.max(err) <= 2e-2 * np.max(np.abs(ref)), (np.max(err), np.max(np.abs(ref)))
    assert np.all(sten[nbr < 0] == 0.0)
    ctx.close()


def test_learned_harvest_features(gpu_ctx_factory):
    ctx, c, conn = _continuity(gpu_ctx_factory, 9)
    ctx.learned_init(1)
    st, rf, tg, rows = ctx.learned_harvest(n_samples=600, n_rhs=3, seed=5, with_rows=True)
    assert 500 <= st.shape[0] <= 600 and np.all(rows > 0)  # row 0 is the identity row
    rp, ci = ctx.graph()
    v, _ = ctx.system()
    nbr = M.slot_map(conn, c.shape[0])
    sth, _ = M.static_features(rp, ci, v, nbr)
    np.testing.assert_array_equal(st, sth[rows])
    np.testing.assert_allclose((rf.astype(np.float64) ** 2).sum(1) / 27, 1.0, rtol=1e-5)
    assert np.all(rf[nbr[rows] < 0] == 0.0)
    assert np.all(np.isfinite(tg)) and np.std(tg) > 0
    ctx.close()


def test_learned_fcg_fewer_iterations_than_jacobi(gpu_ctx_factory, oracle):
    ctx, _, _ = _continuity(gpu_ctx_factory, 24)
    ctx.learned_init(1)
    st, rf, tg = ctx.learned_harvest(n_samples=20000, n_rhs=4, seed=2)
    hist = ctx.learned_train(st, rf, tg, epochs=30)
    assert hist[-1, 1] < 0.5 * hist[0, 1] or hist[-1, 1] < 0.05, hist[[0, -1]]
    plain = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=20000))
    xp = ctx.solution()
    # the learned FCG itself (no opening probe)
    info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=20000, precond=ng.PRECOND_LEARNED,
                                            learned_probe=0))
    x = ctx.solution()
    rp, ci = ctx.graph()
    v, b = ctx.system()
    res = np.linalg.norm(b - oracle.spmv(rp, ci, v, x)) / np.linalg.norm(b)
    assert info.status == 0 and info.fallback == 0 and res <= 1.05e-8, (info.status, info.fallback, res)
    assert info.learned_iterations < 0.8 * plain.iterations, (info.learned_iterations, plain.iterations)
    assert np.max(np.abs(x - xp)) <= 1e-4 * np.max(np.abs(xp))
    # with the probe (default): either method may finish, the result is the same
    info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=20000, precond=ng.PRECOND_LEARNED))
    x = ctx.solution()
    res = np.linalg.norm(b - oracle.spmv(rp, ci, v, x)) / np.linalg.norm(b)
    assert info.status == 0 and info.fallback in (0, 2) and res <= 1.05e-8, (info.status, info.fallback, res)
    ctx.close()


@pytest.mark.parametrize("case", ["large", "nan"])
def test_learned_bad_weights_still_solve(gpu_ctx_factory, oracle, case):
    """An output layer far too large only scales the preconditioner, which the
    SPD scaling keeps positive definite (the FCG converges); a NaN weight
    stops the FCG, after which Chebyshev-Jacobi PCG finishes."""
    ctx, _, _ = _continuity(gpu_ctx_factory, 12)
    P = M.random_params(17, out_scale=1e30 if case == "large" else 1.0).astype(np.float32)
    if case == "nan":
        P[M.SL["b4"][0]] = np.nan
    ctx.learned_set_weights(P)
    info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=20000, precond=ng.PRECOND_LEARNED))
    x = ctx.solution()
    rp, ci = ctx.graph()
    v, b = ctx.system()
    res = np.linalg.norm(b - oracle.spmv(rp, ci, v, x)) / np.linalg.norm(b)
    assert info.status == 0 and res <= 1.05e-8, (info.fallback, info.status, res)
    if case == "nan":
        assert info.fallback in (1, 2)  # caught by the opening probe or by the FCG's breakdown test
    ctx.close()


def test_learned_errors(gpu_ctx_factory):
    ctx, _, _ = _continuity(gpu_ctx_factory, 4)
    with pytest.raises(ng.NaluError):  # no weights yet
        ctx.solve(ng.default_solver_opts(precond=ng.PRECOND_LEARNED))
    ctx.learned_init(0)
    with pytest.raises(ng.NaluError):  # learned runs in FP64 CG only
        ctx.solve(ng.default_solver_opts(precond=ng.PRECOND_LEARNED, method=ng.SOLVER_GMRES))
    with pytest.raises(ng.NaluError):
        ctx.learned_set_weights(np.zeros(10, np.float32))
    ctx.close()
