"""GPU parity: the sm_103a path through the C ABI against the oracle and the
reference's golden vectors.  Tolerance for assembled FP64 values:
|a - b| <= 1e-12 max(|a|,|b|) + 1e-12 (row max |b|)  (helpers.REL / FLOOR)."""
import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import TrigFields, block_mesh, check_csr_values, check_dense, check_vec, continuity_fields

pytestmark = pytest.mark.gpu


def _ctx(gpu_ctx_factory, c, conn, gid=None):
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    return ctx


# ---------------------------------------------------------------------------
# golden vectors of the reference's kernel unit tests (mock-capture mode)
# ---------------------------------------------------------------------------
def test_golds_capture(gpu_ctx_factory, golds, oracle):
    c, conn, gid = block_mesh(1, 1, 1)
    ctx = _ctx(gpu_ctx_factory, c, conn)
    ctx.field_set("scalar_q", TrigFields.temperature(c))
    ctx.field_set("diff_coeff", np.ones(8))
    lhs, rhs = ctx.capture_element(ng.KERNEL_SCALAR_DIFF, 0)
    assert np.max(np.abs(lhs.ravel() - golds["scalar_diff"]["lhs"])) <= 1e-15
    assert np.max(np.abs(rhs)) <= 1e-15
    ctx.field_set("velocity", TrigFields.velocity(c))
    ctx.field_set("density", np.ones(8))
    ctx.field_set("pressure", TrigFields.pressure(c))
    ctx.field_set("dpdx", TrigFields.dpdx(c))
    for key, kw in [("continuity_default", {}), ("continuity_reduced_sens", {"reduced_sens": 1}),
                    ("continuity_reduced_shift", {"reduced_sens": 1, "shift_poisson": 1})]:
        lhs, rhs = ctx.capture_element(ng.KERNEL_CONTINUITY_ADV, 0, ng.default_assemble_opts(**kw))
        assert np.max(np.abs(lhs.ravel() - golds[key]["lhs"])) <= 1e-15, key
        assert np.max(np.abs(rhs - golds[key]["rhs"])) <= 1e-15, key
    # momentum: mdot from ComputeMdotElemAlgorithm with p = Gp = 0 (the unit-test helper)
    ctx.field_set("velocity_rtm", TrigFields.velocity(c))
    ctx.field_set("pressure", np.zeros(8))
    ctx.field_set("dpdx", np.zeros((8, 3)))
    ctx.compute_mdot()
    ctx.field_set("viscosity", 0.1 * np.ones(8))
    lhs, rhs = ctx.capture_element(ng.KERNEL_MOMENTUM_ADV_DIFF, 0)
    g = golds["momentum_adv_diff"]
    assert np.max(np.abs(lhs.ravel() - g["lhs"])) <= 1e-15
    assert np.max(np.abs(rhs - g["rhs"])) <= 1e-15
    ctx.close()


def test_tpetra_two_hex(gpu_ctx_factory, golds):
    """unit_tests/UnitTestTpetra.C on generated:1x1x2 through sumInto."""
    g = golds["tpetra_2hex"]
    c, conn, gid = block_mesh(1, 1, 2)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.build_elem_graph(1)
    rp, ci = ctx.graph()
    assert np.diff(rp).tolist() == g["row_lengths"]
    ctx.zero()
    ev = np.array(g["elem_vals"])
    ctx.sum_into([0, 1], np.stack([ev, ev]), np.zeros((2, 8)))
    ctx.load_complete()
    vals, _ = ctx.system()
    dense = np.zeros((12, 12))
    for i in range(12):
        dense[i, ci[rp[i]:rp[i + 1]]] = vals[rp[i]:rp[i + 1]]
    assert np.max(np.abs(dense.ravel() - g["lhs_vals"])) <= g["tol"]
    ctx.close()


# ---------------------------------------------------------------------------
# graph: bit-exact against the restated Tpetra graph
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("nd", [1, 3])
def test_graph_bit_exact_permuted_gids(gpu_ctx_factory, oracle, nd):
    c, conn, gid = block_mesh(5, 4, 3)
    rng = np.random.default_rng(7)
    pg = (rng.permutation(c.shape[0]) * 3 + 5).astype(np.int64)
    ctx = _ctx(gpu_ctx_factory, c, conn, pg)
    ctx.build_elem_graph(nd)
    rp, ci = ctx.graph()
    orp, oci, _ = oracle.graph(c.shape[0], conn, nd, pg)
    assert rp.dtype == orp.dtype and np.array_equal(rp, orp)
    assert np.array_equal(ci, oci)
    ctx.close()


def test_graph_bit_exact_32cube(gpu_ctx_factory, oracle):
    c, conn, gid = block_mesh(32, jitter=0.1, seed=1)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.build_elem_graph(1)
    rp, ci = ctx.graph()
    orp, oci, _ = oracle.graph(c.shape[0], conn, 1, gid)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert ci.size == 912673  # (3N+1)^3, N = 32
    ctx.close()


# ---------------------------------------------------------------------------
# full assembly parity
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("scatter", [ng.SCATTER_ATOMIC, ng.SCATTER_COLOURED])
@pytest.mark.parametrize("shifted", [0, 1])
def test_scalar_diff_32cube_jittered(gpu_ctx_factory, oracle, scatter, shifted):
    """Heat-conduction configuration: 32^3 unit cube, +-10% jitter, k = 1, T ~ U[0,1]."""
    c, conn, gid = block_mesh(32, jitter=0.1, seed=11)
    rng = np.random.default_rng(12)
    T, k = rng.uniform(0, 1, c.shape[0]), np.ones(c.shape[0])
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.field_set("scalar_q", T)
    ctx.field_set("diff_coeff", k)
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_SCALAR_DIFF, ng.default_assemble_opts(scatter=scatter, shifted_grad_op=shifted))
    ctx.load_complete()
    vals, rhs = ctx.system()
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(c.shape[0], conn, 1, gid)
    ov, orhs = oracle.assemble(oracle.KERNEL_SCALAR_DIFF, c, conn, rp, ci, lid, scalar=T, coeff=k,
                               opts=oracle.opts_block(shifted_grad_op=shifted), n_threads=8)
    check_csr_values(vals, ov, rp)
    check_vec(rhs, orhs)
    ctx.close()


@pytest.mark.parametrize("kw", [{}, {"reduced_sens": 1}, {"reduced_sens": 1, "shift_poisson": 1},
                                {"shift_mdot": 1}, {"proj_time_scale": 0.37}])
def test_continuity_stretched_jittered(gpu_ctx_factory, oracle, kw):
    c, conn, gid = block_mesh(12, 10, 9, jitter=0.1, seed=3, z_ratio=1.05)
    u, rho, p, gp = continuity_fields(c, seed=4)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    for n, v in (("velocity", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
        ctx.field_set(n, v)
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(**kw))
    vals, rhs = ctx.system()
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(c.shape[0], conn, 1, gid)
    o = oracle.opts_block(shift_mdot=kw.get("shift_mdot", 0), shift_poisson=kw.get("shift_poisson", 0),
                          reduced_sens=kw.get("reduced_sens", 0), proj_time_scale=kw.get("proj_time_scale", 1.0))
    ov, orhs = oracle.assemble(oracle.KERNEL_CONTINUITY_ADV, c, conn, rp, ci, lid, scalar=p, coeff=rho, vec=u,
                               vec2=gp, opts=o, n_threads=8)
    check_csr_values(vals, ov, rp)
    check_vec(rhs, orhs)
    ctx.close()


def test_continuity_128_properties(gpu_ctx_factory, oracle):
    """Continuity configuration at full size (128^3, z-stretch 1.05): row sums
    vanish (conservation), the Laplacian is symmetric on the unjittered mesh,
    atomic and coloured scatter agree, sampled elements match the oracle."""
    c, conn, gid = block_mesh(128, z_ratio=1.05)
    u = ng.meshgen.fourier_velocity(c, n_modes=64, seed=5)
    n = c.shape[0]
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.field_set("velocity", u)
    ctx.field_set("density", np.ones(n))
    ctx.field_set("pressure", np.zeros(n))
    ctx.field_set("dpdx", np.zeros((n, 3)))
    ctx.build_elem_graph(1)
    rp, ci = ctx.graph()
    assert ci.size == 57066625
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(scatter=ng.SCATTER_ATOMIC))
    va, ra = ctx.system()
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(scatter=ng.SCATTER_COLOURED))
    vc, rc = ctx.system()
    check_csr_values(va, vc, rp, what="atomic vs coloured")
    check_vec(ra, rc, what="rhs atomic vs coloured")
    rows = np.repeat(np.arange(n), np.diff(rp))
    rs = np.zeros(n)
    np.add.at(rs, rows, va)
    rmax = np.zeros(n)
    np.maximum.at(rmax, rows, np.abs(va))
    assert np.all(np.abs(rs) <= 1e-12 * rmax * 27)
    # symmetry: A[i,j] == A[j,i]
    order = np.lexsort((rows, ci))
    check_csr_values(va[order], va, rp, rel=1e-12, floor=1e-13, what="transpose")
    # sampled element matrices against the oracle
    rng = np.random.default_rng(0)
    for e in rng.integers(0, conn.shape[0], 64):
        lhs, rhs = ctx.capture_element(ng.KERNEL_CONTINUITY_ADV, int(e))
        nd = conn[e]
        ol, orr = oracle.continuity_adv_elem(c[nd], u[nd], np.ones(8), np.zeros(8), np.zeros((8, 3)), 1.0)
        check_dense(lhs, ol)
        check_dense(rhs[None], orr[None])
    ctx.close()


@pytest.mark.parametrize("arith", [ng.ARITH_FP64, ng.ARITH_DF64])
def test_mdot_matches_oracle(gpu_ctx_factory, oracle, arith):
    c, conn, gid = block_mesh(7, 6, 5, jitter=0.1, seed=8)
    u, rho, p, gp = continuity_fields(c, seed=9)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    for n, v in (("velocity_rtm", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
        ctx.field_set(n, v)
    for sm, sp in [(0, 0), (1, 0), (0, 1), (1, 1)]:
        ctx.compute_mdot(ng.default_assemble_opts(shift_mdot=sm, shift_poisson=sp, proj_time_scale=0.5,
                                                  arith=arith))
        m = ctx.field_get("mass_flow_rate_scs", (conn.shape[0], 12))
        om = np.stack([oracle.mdot_elem(c[e], rho[e], u[e], p[e], gp[e], 0.5, sm, sp) for e in conn])
        check_dense(m, om, what="mdot")
    ctx.close()


@pytest.mark.parametrize("upw", [False, True])
def test_momentum_matches_oracle(gpu_ctx_factory, oracle, upw):
    c, conn, gid = block_mesh(6, 5, 4, jitter=0.1, seed=13)
    n = c.shape[0]
    rng = np.random.default_rng(14)
    u = ng.meshgen.fourier_velocity(c, n_modes=8, seed=15)
    mu = rng.uniform(1e-3, 2e-3, n)
    rho = rng.uniform(0.9, 1.1, n)
    gju = rng.normal(size=(n, 9))
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    for nm, v in (("velocity", u), ("velocity_rtm", u), ("density", rho), ("viscosity", mu), ("dudx", gju),
                  ("pressure", np.zeros(n)), ("dpdx", np.zeros((n, 3)))):
        ctx.field_set(nm, v)
    ctx.compute_mdot()
    mdot = ctx.field_get("mass_flow_rate_scs", (conn.shape[0], 12))
    ctx.build_elem_graph(3)
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(n, conn, 3, gid)
    if upw:
        kw = dict(alpha=0.1, alpha_upw=0.5, upw_factor=1.0, hybrid_factor=1.0, use_limiter=1, include_divu=1.0)
        kid, okid = ng.KERNEL_MOMENTUM_UPW_ADV_DIFF, oracle.KERNEL_MOMENTUM_UPW_ADV_DIFF
    else:
        kw = dict(include_divu=1.0)
        kid, okid = ng.KERNEL_MOMENTUM_ADV_DIFF, oracle.KERNEL_MOMENTUM_ADV_DIFF
    for scatter in (ng.SCATTER_ATOMIC, ng.SCATTER_COLOURED):
        ctx.zero()
        ctx.assemble(kid, ng.default_assemble_opts(scatter=scatter, **kw))
        vals, rhs = ctx.system()
        ov, orhs = oracle.assemble(okid, c, conn, rp, ci, lid, coeff=mu, vec=u, vec2=u, rho=rho, gju=gju, mdot=mdot,
                                   opts=oracle.opts_block(**kw), n_threads=8)
        check_csr_values(vals, ov, rp, what="momentum values")
        check_vec(rhs, orhs, what="momentum rhs")
    ctx.close()


def test_bc_row_ops(gpu_ctx_factory, oracle):
    c, conn, gid = block_mesh(5, 5, 5, jitter=0.1, seed=2)
    n = c.shape[0]
    rng = np.random.default_rng(1)
    T = rng.uniform(size=n)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.field_set("scalar_q", T)
    ctx.field_set("diff_coeff", np.ones(n))
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_SCALAR_DIFF)
    rp, ci = ctx.graph()
    vals0, rhs0 = ctx.system()
    left = np.where(c[:, 0] == 0.0)[0]
    right = np.where(c[:, 0] == 1.0)[0]
    nodes = np.concatenate([left, right])
    bc = np.concatenate([np.zeros(left.size), np.ones(right.size)])
    ctx.apply_dirichlet(nodes, bc, T[nodes])
    ctx.reset_rows([7])
    ctx.sum_into_diag(7, 0, 1.0, 0.25)
    ctx.load_complete()
    vals, rhs = ctx.system()
    ov, orhs = vals0.copy(), rhs0.copy()
    oracle.apply_dirichlet(rp, ci, ov, orhs, nodes, bc, T[nodes])
    oracle.reset_rows(rp, ov, orhs, [7])
    oracle.sum_into_diag(rp, ci, ov, orhs, 7, 1.0, 0.25)
    assert np.array_equal(vals, ov) and np.array_equal(rhs, orhs)
    ctx.close()


def test_negative_jacobian_reported(gpu_ctx_factory):
    """An inverted element is reported as a status, not a fault."""
    c, conn, gid = block_mesh(2, 1, 1)
    bad = conn.copy()
    bad[0] = bad[0][[4, 5, 6, 7, 0, 1, 2, 3]]  # mirrored: det < 0
    ctx = _ctx(gpu_ctx_factory, c, bad)
    ctx.field_set("scalar_q", np.zeros(c.shape[0]))
    ctx.field_set("diff_coeff", np.ones(c.shape[0]))
    ctx.build_elem_graph(1)
    with pytest.raises(ng.NaluError) as ei:
        # the status surfaces at the first host synchronisation point
        ctx.assemble(ng.KERNEL_SCALAR_DIFF)
        ctx.load_complete()
    assert ei.value.status == -4
    # the context stays usable: explicit scatter, then the status again at loadComplete
    ctx.assemble(ng.KERNEL_SCALAR_DIFF, ng.default_assemble_opts(scatter=ng.SCATTER_ATOMIC))
    with pytest.raises(ng.NaluError) as ei:
        ctx.load_complete()
    assert ei.value.status == -4
    ctx.close()


@pytest.mark.parametrize("bad", [float("nan"), float("inf"), 1e300])
def test_df64_out_of_range_input_reported(gpu_ctx_factory, bad):
    """A nodal input the double-float pairs cannot hold (NaN, inf, |x| >=
    2^127) in the velocity of a continuity assembly or the diffusion
    coefficient of a heat assembly is reported as NALU_ERR_NONFINITE at the
    next host synchronisation point, and the context stays usable."""
    c, conn, gid = block_mesh(4, 3, 3)
    n = c.shape[0]
    u, rho, p, gp = continuity_fields(c, seed=3)
    u[7, 1] = bad
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    for nm, v in (("velocity", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
        ctx.field_set(nm, v)
    ctx.build_elem_graph(1)
    opts = ng.default_assemble_opts(scatter=ng.SCATTER_ATOMIC, arith=ng.ARITH_DF64, schedule=ng.SCHEDULE_IP16)
    with pytest.raises(ng.NaluError) as ei:
        ctx.zero()
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV, opts)
        ctx.load_complete()
    assert ei.value.status == -5
    u[7, 1] = 0.5
    ctx.field_set("velocity", u)
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, opts)
    ctx.load_complete()
    k = np.ones(n)
    k[5] = bad
    ctx.field_set("scalar_q", np.zeros(n))
    ctx.field_set("diff_coeff", k)
    with pytest.raises(ng.NaluError) as ei:
        ctx.zero()
        ctx.assemble(ng.KERNEL_SCALAR_DIFF, ng.default_assemble_opts(scatter=ng.SCATTER_ATOMIC, arith=ng.ARITH_DF64))
        ctx.load_complete()
    assert ei.value.status == -5
    ctx.close()


# ---------------------------------------------------------------------------
# double-float element math (ARITH_DF64) against the FP64 oracle
# ---------------------------------------------------------------------------
SCHEDULES = [ng.SCHEDULE_ELEMENT, ng.SCHEDULE_IP8, ng.SCHEDULE_IP16]


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("scatter", [ng.SCATTER_ATOMIC, ng.SCATTER_COLOURED])
def test_df64_scalar_diff_32cube(gpu_ctx_factory, oracle, scatter, schedule):
    c, conn, gid = block_mesh(32, jitter=0.1, seed=11)
    rng = np.random.default_rng(12)
    T, k = rng.uniform(0, 1, c.shape[0]), rng.uniform(0.5, 2.0, c.shape[0])
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.field_set("scalar_q", T)
    ctx.field_set("diff_coeff", k)
    ctx.build_elem_graph(1)
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(c.shape[0], conn, 1, gid)
    for shifted in (0, 1):
        ctx.zero()
        ctx.assemble(ng.KERNEL_SCALAR_DIFF, ng.default_assemble_opts(scatter=scatter, shifted_grad_op=shifted,
                                                                     arith=ng.ARITH_DF64, schedule=schedule))
        ctx.load_complete()
        vals, rhs = ctx.system()
        ov, orhs = oracle.assemble(oracle.KERNEL_SCALAR_DIFF, c, conn, rp, ci, lid, scalar=T, coeff=k,
                                   opts=oracle.opts_block(shifted_grad_op=shifted), n_threads=8)
        check_csr_values(vals, ov, rp, what="df64 values")
        check_vec(rhs, orhs, what="df64 rhs")
    ctx.close()


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("kw", [{}, {"reduced_sens": 1}, {"reduced_sens": 1, "shift_poisson": 1},
                                {"shift_mdot": 1}, {"proj_time_scale": 0.37},
                                {"reduced_sens": 1, "shift_mdot": 1, "proj_time_scale": 0.37}])
def test_df64_continuity(gpu_ctx_factory, oracle, kw, schedule):
    c, conn, gid = block_mesh(12, 10, 9, jitter=0.1, seed=3, z_ratio=1.05)
    u, rho, p, gp = continuity_fields(c, seed=4)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    for n, v in (("velocity", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
        ctx.field_set(n, v)
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(arith=ng.ARITH_DF64, schedule=schedule, **kw))
    ctx.load_complete()
    vals, rhs = ctx.system()
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(c.shape[0], conn, 1, gid)
    o = oracle.opts_block(shift_mdot=kw.get("shift_mdot", 0), shift_poisson=kw.get("shift_poisson", 0),
                          reduced_sens=kw.get("reduced_sens", 0), proj_time_scale=kw.get("proj_time_scale", 1.0))
    ov, orhs = oracle.assemble(oracle.KERNEL_CONTINUITY_ADV, c, conn, rp, ci, lid, scalar=p, coeff=rho, vec=u,
                               vec2=gp, opts=o, n_threads=8)
    check_csr_values(vals, ov, rp, what="df64 values")
    check_vec(rhs, orhs, what="df64 rhs")
    ctx.close()


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_df64_golds_capture(gpu_ctx_factory, golds, schedule):
    c, conn, gid = block_mesh(1, 1, 1)
    ctx = _ctx(gpu_ctx_factory, c, conn)
    ctx.field_set("scalar_q", TrigFields.temperature(c))
    ctx.field_set("diff_coeff", np.ones(8))
    lhs, rhs = ctx.capture_element(ng.KERNEL_SCALAR_DIFF, 0,
                                   ng.default_assemble_opts(arith=ng.ARITH_DF64, schedule=schedule))
    assert np.max(np.abs(lhs.ravel() - golds["scalar_diff"]["lhs"])) <= 1e-15
    ctx.field_set("velocity", TrigFields.velocity(c))
    ctx.field_set("density", np.ones(8))
    ctx.field_set("pressure", TrigFields.pressure(c))
    ctx.field_set("dpdx", TrigFields.dpdx(c))
    for key, kw in [("continuity_default", {}), ("continuity_reduced_sens", {"reduced_sens": 1}),
                    ("continuity_reduced_shift", {"reduced_sens": 1, "shift_poisson": 1})]:
        lhs, rhs = ctx.capture_element(ng.KERNEL_CONTINUITY_ADV, 0,
                                       ng.default_assemble_opts(arith=ng.ARITH_DF64, schedule=schedule, **kw))
        assert np.max(np.abs(lhs.ravel() - golds[key]["lhs"])) <= 1e-15, key
        assert np.max(np.abs(rhs - golds[key]["rhs"])) <= 1e-15, key
    ctx.close()


def test_async_download_matches_blocking_copy(gpu_ctx_factory):
    """nalu_linsys_copy_async: the pinned host copy equals the blocking copy,
    also for three downloads in a row with a different assembly in between
    (two snapshots in turn: the third reuses the first's once its transfer
    has ended)."""
    c, conn, gid = block_mesh(20, jitter=0.1, seed=31)
    n = c.shape[0]
    u, rho, p, gp = continuity_fields(c, seed=32)
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    for nm, val in (("velocity", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
        ctx.field_set(nm, val)
    ctx.build_elem_graph(1)
    nr, nnz, _ = ctx.sizes()
    outs = [(ng.PinnedArray((nnz,)), ng.PinnedArray((nr,))) for _ in range(3)]
    refs = []
    for k, (ov, orr) in enumerate(outs):
        ctx.field_set("density", rho * (1.0 + k))
        ctx.zero()
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
        refs.append(ctx.system())
        ctx.system_to_ptr_async(ov.ptr, orr.ptr)
    ctx.copy_wait()
    for (ov, orr), (rv, rr) in zip(outs, refs):
        np.testing.assert_array_equal(ov.array, rv)
        np.testing.assert_array_equal(orr.array, rr)
    assert not np.array_equal(outs[0][1].array, outs[1][1].array)
    assert not np.array_equal(outs[0][1].array, outs[2][1].array)
    for ov, orr in outs:
        ov.free()
        orr.free()
    ctx.close()


@pytest.mark.parametrize("upw", [False, True])
def test_df64_momentum_matches_oracle(gpu_ctx_factory, oracle, upw):
    """The double-float momentum kernel against the FP64 oracle at the
    assembly tolerance, both scatters, central and upwind-blended forms."""
    c, conn, gid = block_mesh(6, 5, 4, jitter=0.1, seed=13)
    n = c.shape[0]
    rng = np.random.default_rng(14)
    u = ng.meshgen.fourier_velocity(c, n_modes=8, seed=15)
    mu = rng.uniform(1e-3, 2e-3, n)
    rho = rng.uniform(0.9, 1.1, n)
    gju = rng.normal(size=(n, 9))
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    for nm, v in (("velocity", u), ("velocity_rtm", u), ("density", rho), ("viscosity", mu), ("dudx", gju),
                  ("pressure", np.zeros(n)), ("dpdx", np.zeros((n, 3)))):
        ctx.field_set(nm, v)
    ctx.compute_mdot()
    mdot = ctx.field_get("mass_flow_rate_scs", (conn.shape[0], 12))
    ctx.build_elem_graph(3)
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(n, conn, 3, gid)
    if upw:
        kw = dict(alpha=0.1, alpha_upw=0.5, upw_factor=1.0, hybrid_factor=1.0, use_limiter=1, include_divu=1.0)
        kid, okid = ng.KERNEL_MOMENTUM_UPW_ADV_DIFF, oracle.KERNEL_MOMENTUM_UPW_ADV_DIFF
    else:
        kw = dict(include_divu=1.0)
        kid, okid = ng.KERNEL_MOMENTUM_ADV_DIFF, oracle.KERNEL_MOMENTUM_ADV_DIFF
    ov, orhs = oracle.assemble(okid, c, conn, rp, ci, lid, coeff=mu, vec=u, vec2=u, rho=rho, gju=gju, mdot=mdot,
                               opts=oracle.opts_block(**kw), n_threads=8)
    for scatter in (ng.SCATTER_ATOMIC, ng.SCATTER_COLOURED):
        ctx.zero()
        ctx.assemble(kid, ng.default_assemble_opts(scatter=scatter, arith=ng.ARITH_DF64, **kw))
        vals, rhs = ctx.system()
        check_csr_values(vals, ov, rp, what="df64 momentum values")
        check_vec(rhs, orhs, what="df64 momentum rhs")
    ctx.close()


def test_df64_momentum_golds(gpu_ctx_factory, golds):
    """UnitTestMomentumAdvDiffElem's 24x24 gold through the df64 kernel
    (FP32-pair arithmetic: within 1e-14 of the gold; the FP64 kernel meets the
    reference's 1e-15, test_golds_capture)."""
    c, conn, gid = block_mesh(1, 1, 1)
    ctx = _ctx(gpu_ctx_factory, c, conn)
    ctx.field_set("velocity", TrigFields.velocity(c))
    ctx.field_set("velocity_rtm", TrigFields.velocity(c))
    ctx.field_set("density", np.ones(8))
    ctx.field_set("pressure", np.zeros(8))
    ctx.field_set("dpdx", np.zeros((8, 3)))
    ctx.compute_mdot()
    ctx.field_set("viscosity", 0.1 * np.ones(8))
    lhs, rhs = ctx.capture_element(ng.KERNEL_MOMENTUM_ADV_DIFF, 0, ng.default_assemble_opts(arith=ng.ARITH_DF64))
    g = golds["momentum_adv_diff"]
    assert np.max(np.abs(lhs.ravel() - g["lhs"])) <= 1e-14
    assert np.max(np.abs(rhs - g["rhs"])) <= 1e-14
    ctx.close()


def test_df64_autotuner_table(gpu_ctx_factory):
    """The first AUTO df64 assembly times every schedule x scatter pair and
    keeps the fastest; the table and the choice are reported, and the result
    is the same system as an explicit run of the chosen pair."""
    c, conn, gid = block_mesh(16, 14, 12, jitter=0.1, seed=9, z_ratio=1.05)
    u, rho, p, gp = continuity_fields(c, seed=10)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    for n, v in (("velocity", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
        ctx.field_set(n, v)
    ctx.build_elem_graph(1)
    with pytest.raises(ng.NaluError):
        ctx.assemble_tuning(ng.KERNEL_CONTINUITY_ADV)
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(arith=ng.ARITH_DF64))
    v_auto, r_auto = ctx.system()
    sch, sc, table = ctx.assemble_tuning(ng.KERNEL_CONTINUITY_ADV)
    assert len(table) == 6 and all(ms > 0 for ms in table.values())
    best = min(table, key=table.get)
    assert best == (ng.SCHEDULE_NAMES[sch], {1: "atomic", 2: "coloured"}[sc])
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(arith=ng.ARITH_DF64, schedule=sch, scatter=sc))
    v_exp, r_exp = ctx.system()
    rp, _ = ctx.graph()
    check_csr_values(v_auto, v_exp, rp, what="auto vs explicit")
    check_vec(r_auto, r_exp, what="auto vs explicit rhs")
    # the tuning did not leave its trial assemblies in the system
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(arith=ng.ARITH_DF64, schedule=sch, scatter=sc))
    v2, _ = ctx.system()
    check_csr_values(v2, v_exp, rp, what="repeat")
    ctx.close()
