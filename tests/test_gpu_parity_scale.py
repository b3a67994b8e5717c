"""GPU parity at the benchmark sizes: the double-float (ARITH_DF64) kernels the
benchmark selects, value by value against the oracle's full FP64 assembly of
the same seeded workload, at the tolerance of the smaller parity tests:
|a - b| <= 1e-12 max(|a|,|b|) + 1e-12 (row max |b|)  (helpers.REL / FLOOR).

- continuity (ContinuityAdvElemKernel) on the exact 128^3 benchmark input
  (z-stretch 1.05, cell aspect ratios up to about 80, Fourier-64 velocity,
  seed 2024), both scatters;
- continuity on the 192^3 mesh of the learned-solve configuration;
- momentum (MomentumAdvDiffElemKernel and the upwind-blended kernel with
  alpha_upw = 0.5) on the 96^3 mesh of the momentum configuration;
- the 64-mesh batched configuration's union mesh;
- coordinates scaled by 1e-9 and 1e+9, where unnormalised FP32-pair
  geometry leaves the FP32 exponent range (det J ~ h^3, adj(J)^T A ~ h^4).

Each test also asserts the measured worst error ratio (error / allowed) and
prints it, so a run's log states the error against the FP64 oracle per
result.
"""
import os

import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import REL, FLOOR, block_mesh, check_csr_values, check_vec, continuity_fields, csr_row_max

pytestmark = pytest.mark.gpu

THREADS = max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1))


def err_ratio_csr(actual, expected, rowptr):
    rm, rowid = csr_row_max(rowptr, expected)
    allowed = REL * np.maximum(np.abs(actual), np.abs(expected)) + FLOOR * rm[rowid]
    return float(np.max(np.abs(actual - expected) / allowed))


def err_ratio_vec(actual, expected):
    allowed = REL * np.maximum(np.abs(actual), np.abs(expected)) + FLOOR * np.max(np.abs(expected))
    return float(np.max(np.abs(actual - expected) / allowed))


def _continuity_ctx(c, conn, gid, u, rho, p, gp):
    ctx = ng.Context(0)
    ctx.mesh_create(c, conn, gid)
    for nm, v in (("velocity", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
        ctx.field_set(nm, v)
    ctx.build_elem_graph(1)
    return ctx


def _check_continuity(ctx, oracle, c, conn, gid, u, rho, p, gp, scatters, opts=None, what="",
                      schedules=(ng.SCHEDULE_AUTO,)):
    rp, ci = ctx.graph()
    orp, oci, lid = oracle.graph(c.shape[0], conn, 1, gid)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci), "graph differs from the restated Tpetra graph"
    kw = opts or {}
    o = oracle.opts_block(shift_mdot=kw.get("shift_mdot", 0), shift_poisson=kw.get("shift_poisson", 0),
                          reduced_sens=kw.get("reduced_sens", 0), proj_time_scale=kw.get("proj_time_scale", 1.0))
    ov, orhs = oracle.assemble(oracle.KERNEL_CONTINUITY_ADV, c, conn, rp, ci, lid, scalar=p, coeff=rho, vec=u,
                               vec2=gp, opts=o, n_threads=THREADS)
    ratios = {}
    for sch in schedules:
        for sc in scatters:
            ctx.zero()
            ctx.assemble(ng.KERNEL_CONTINUITY_ADV,
                         ng.default_assemble_opts(scatter=sc, arith=ng.ARITH_DF64, schedule=sch, **kw))
            ctx.load_complete()
            vals, rhs = ctx.system()
            tag = "%s df64 schedule %d scatter %d" % (what, sch, sc)
            check_csr_values(vals, ov, rp, what=tag + " values")
            check_vec(rhs, orhs, what=tag + " rhs")
            ratios[sch, sc] = (err_ratio_csr(vals, ov, rp), err_ratio_vec(rhs, orhs))
            print("%s: max err/tol values %.3g rhs %.3g" % (tag, *ratios[sch, sc]))
    return ratios


def test_df64_continuity_bench_workload(oracle):
    """The exact 128^3 benchmark input through the kernel the benchmark times."""
    import bench
    c, conn, gid, u, rho, p, gp = bench.make_inputs()
    ctx = _continuity_ctx(c, conn, gid, u, rho, p, gp)
    assert ctx.sizes()[1] == 57066625
    _check_continuity(ctx, oracle, c, conn, gid, u, rho, p, gp, (ng.SCATTER_ATOMIC, ng.SCATTER_COLOURED),
                      what="128^3 bench", schedules=(ng.SCHEDULE_ELEMENT, ng.SCHEDULE_IP8, ng.SCHEDULE_IP16))
    ctx.close()


def test_df64_continuity_128_pressure_and_options(oracle):
    """The benchmark mesh with non-zero pressure and pressure gradient (the
    -lhs.p and tau Gp terms) under the reduced-sensitivity and shifted options."""
    from nalu_gb300.meshgen import fourier_velocity
    c, conn, gid = block_mesh(128, z_ratio=1.05)
    n = c.shape[0]
    rng = np.random.default_rng(77)
    u = fourier_velocity(c, n_modes=64, seed=2024)
    rho, p, gp = rng.uniform(0.8, 1.2, n), rng.normal(size=n), rng.normal(size=(n, 3))
    ctx = _continuity_ctx(c, conn, gid, u, rho, p, gp)
    for kw in ({"proj_time_scale": 0.37}, {"reduced_sens": 1, "shift_poisson": 1, "shift_mdot": 1}):
        _check_continuity(ctx, oracle, c, conn, gid, u, rho, p, gp, (ng.SCATTER_ATOMIC,), opts=kw,
                          what="128^3 %s" % kw, schedules=(ng.SCHEDULE_ELEMENT, ng.SCHEDULE_IP8, ng.SCHEDULE_IP16))
    ctx.close()


def test_df64_continuity_192(oracle):
    """192^3 (7.1 M elements, 192 M non-zeros): the learned-solve mesh."""
    from nalu_gb300.meshgen import fourier_velocity
    c, conn, gid = block_mesh(192, z_ratio=1.05)
    n = c.shape[0]
    u = fourier_velocity(c, n_modes=64, seed=2024)
    ctx = _continuity_ctx(c, conn, gid, u, np.ones(n), np.zeros(n), np.zeros((n, 3)))
    assert ctx.sizes()[1] == 192100033
    _check_continuity(ctx, oracle, c, conn, gid, u, np.ones(n), np.zeros(n), np.zeros((n, 3)), (ng.SCATTER_ATOMIC,),
                      what="192^3")
    ctx.close()


def test_df64_momentum_96(oracle):
    """96^3 momentum (217 M non-zeros, 24x24 element matrices): central and
    upwind-blended (alpha_upw 0.5, hybrid factor 1, van Leer limiter)."""
    from nalu_gb300.meshgen import fourier_velocity
    c, conn, gid = block_mesh(96)
    n = c.shape[0]
    rng = np.random.default_rng(96)
    u = fourier_velocity(c, n_modes=64, kmin=1, kmax=16, seed=2024)
    mu = np.full(n, 1e-3)
    rho = np.ones(n)
    gju = 0.1 * rng.normal(size=(n, 9))
    ctx = ng.Context(0)
    ctx.mesh_create(c, conn, gid)
    for nm, v in (("velocity", u), ("velocity_rtm", u), ("density", rho), ("viscosity", mu), ("dudx", gju),
                  ("pressure", np.zeros(n)), ("dpdx", np.zeros((n, 3)))):
        ctx.field_set(nm, v)
    ctx.compute_mdot()
    mdot = ctx.field_get("mass_flow_rate_scs", (conn.shape[0], 12))
    ctx.build_elem_graph(3)
    rp, ci = ctx.graph()
    assert ci.size == 217238121
    _, _, lid = oracle.graph(n, conn, 3, gid)
    for kid, okid, kw in ((ng.KERNEL_MOMENTUM_ADV_DIFF, oracle.KERNEL_MOMENTUM_ADV_DIFF, dict(include_divu=1.0)),
                          (ng.KERNEL_MOMENTUM_UPW_ADV_DIFF, oracle.KERNEL_MOMENTUM_UPW_ADV_DIFF,
                           dict(alpha_upw=0.5, hybrid_factor=1.0, use_limiter=1, include_divu=1.0))):
        ov, orhs = oracle.assemble(okid, c, conn, rp, ci, lid, coeff=mu, vec=u, vec2=u, rho=rho, gju=gju, mdot=mdot,
                                   opts=oracle.opts_block(**kw), n_threads=THREADS)
        ctx.zero()
        ctx.assemble(kid, ng.default_assemble_opts(scatter=ng.SCATTER_ATOMIC, arith=ng.ARITH_DF64, **kw))
        vals, rhs = ctx.system()
        check_csr_values(vals, ov, rp, what="96^3 df64 momentum values (kernel %d)" % kid)
        check_vec(rhs, orhs, what="96^3 df64 momentum rhs (kernel %d)" % kid)
        print("96^3 momentum kernel %d: max err/tol values %.3g rhs %.3g"
              % (kid, err_ratio_csr(vals, ov, rp), err_ratio_vec(rhs, orhs)))
        del ov, orhs, vals, rhs
    ctx.close()


def test_df64_batch_union(oracle):
    """The 64 independent meshes of the batched configuration (edges
    log-U[16, 96] per axis, jitter 0.1, own Fourier velocity each) as one
    union-mesh assembly."""
    from nalu_gb300.meshgen import batch_block_meshes, fourier_velocity
    c, conn, gid, off, _ = batch_block_meshes(64, edge_range=(16, 96), jitter=0.1, seed=2025)
    n = c.shape[0]
    u = np.concatenate([fourier_velocity(c[off[k]:off[k + 1]], n_modes=64, seed=2025 + 1 + k) for k in range(64)])
    ctx = _continuity_ctx(c, conn, gid, u, np.ones(n), np.zeros(n), np.zeros((n, 3)))
    ctx.set_problems(off)
    _check_continuity(ctx, oracle, c, conn, gid, u, np.ones(n), np.zeros(n), np.zeros((n, 3)),
                      (ng.SCATTER_ATOMIC,), what="64-mesh batch")
    ctx.close()


@pytest.mark.parametrize("scale", [1e-9, 1e9])
def test_df64_scaled_coordinates(oracle, scale):
    """A jittered, z-stretched mesh in units 1e-9 and 1e+9 times the unit cube:
    continuity (all option sets, with pressure), heat conduction and ComputeMdot
    in df64 against the FP64 oracle."""
    c, conn, gid = block_mesh(24, 20, 16, jitter=0.1, seed=5, z_ratio=1.1)
    c = c * scale
    u, rho, p, gp = continuity_fields(c / scale, seed=6)
    gp = gp / scale
    ctx = _continuity_ctx(c, conn, gid, u, rho, p, gp)
    for kw in ({}, {"reduced_sens": 1}, {"reduced_sens": 1, "shift_poisson": 1}, {"shift_mdot": 1}):
        _check_continuity(ctx, oracle, c, conn, gid, u, rho, p, gp, (ng.SCATTER_ATOMIC, ng.SCATTER_COLOURED),
                          opts=kw, what="x%g %s" % (scale, kw),
                          schedules=(ng.SCHEDULE_ELEMENT, ng.SCHEDULE_IP8, ng.SCHEDULE_IP16))
    # heat conduction
    rng = np.random.default_rng(7)
    T, k = rng.uniform(0, 1, c.shape[0]), rng.uniform(0.5, 2.0, c.shape[0])
    ctx.field_set("scalar_q", T)
    ctx.field_set("diff_coeff", k)
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(c.shape[0], conn, 1, gid)
    for sh in (0, 1):
        ov, orhs = oracle.assemble(oracle.KERNEL_SCALAR_DIFF, c, conn, rp, ci, lid, scalar=T, coeff=k,
                                   opts=oracle.opts_block(shifted_grad_op=sh), n_threads=THREADS)
        for sch in (ng.SCHEDULE_ELEMENT, ng.SCHEDULE_IP8, ng.SCHEDULE_IP16):
            ctx.zero()
            ctx.assemble(ng.KERNEL_SCALAR_DIFF, ng.default_assemble_opts(shifted_grad_op=sh, arith=ng.ARITH_DF64,
                                                                         schedule=sch))
            ctx.load_complete()
            vals, rhs = ctx.system()
            check_csr_values(vals, ov, rp, what="x%g df64 heat values (schedule %d)" % (scale, sch))
            check_vec(rhs, orhs, what="x%g df64 heat rhs (schedule %d)" % (scale, sch))
    # mass flow rates
    for nm, v in (("velocity_rtm", u),):
        ctx.field_set(nm, v)
    ctx.compute_mdot(ng.default_assemble_opts(shift_mdot=1, shift_poisson=1, proj_time_scale=0.5,
                                              arith=ng.ARITH_DF64))
    m = ctx.field_get("mass_flow_rate_scs", (conn.shape[0], 12))
    om = np.stack([oracle.mdot_elem(c[e], rho[e], u[e], p[e], gp[e], 0.5, 1, 1) for e in conn])
    scale_row = np.max(np.abs(om), axis=1, keepdims=True)
    assert np.all(np.abs(m - om) <= REL * np.maximum(np.abs(m), np.abs(om)) + FLOOR * scale_row), "mdot x%g" % scale
    ctx.close()
