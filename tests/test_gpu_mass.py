"""GPU parity of the time-term kernels (ContinuityMassElemKernel,
MomentumMassElemKernel) through the C ABI: the reference's unit-test golds in
mock-capture mode (|a - b| <= 1e-15, the reference's own tolerance), and
whole-mesh assembly against the oracle's element-order sumInto on jittered
meshes with BDF2 states (helpers.REL / FLOOR)."""
import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import TrigFields, block_mesh, check_csr_values, check_vec

pytestmark = pytest.mark.gpu


def _ctx(gpu_ctx_factory, c, conn, gid=None):
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    return ctx


@pytest.mark.parametrize("key", ["continuity_mass", "continuity_mass_lumped", "momentum_mass",
                                 "momentum_mass_lumped"])
def test_golds_mass_capture(gpu_ctx_factory, golds, key):
    g = golds[key]
    c, conn, _ = block_mesh(1, 1, 1)
    ctx = _ctx(gpu_ctx_factory, c, conn)
    # the kernel-test fixtures fill state N+1 only
    ctx.field_set("density", np.ones(8))
    ctx.field_set("density_n", np.zeros(8))
    ctx.field_set("velocity", TrigFields.velocity(c))
    ctx.field_set("velocity_n", np.zeros((8, 3)))
    ctx.field_set("dpdx", TrigFields.dpdx(c))
    kernel = ng.KERNEL_CONTINUITY_MASS if key.startswith("continuity") else ng.KERNEL_MOMENTUM_MASS
    o = ng.default_assemble_opts(dt=g["dt"], gamma1=g["gamma1"], gamma2=g["gamma2"], gamma3=g["gamma3"],
                                 lumped_mass=int(g["lumped"]))
    lhs, rhs = ctx.capture_element(kernel, 0, o)
    assert np.max(np.abs(lhs.ravel() - g["lhs"])) <= g["tol"], key
    assert np.max(np.abs(rhs - g["rhs"])) <= g["tol"], key
    ctx.close()


def _states(n, seed):
    rng = np.random.default_rng(seed)
    rho = [1.0 + 0.2 * rng.random(n) for _ in range(3)]          # N-1, N, N+1
    u = [rng.standard_normal((n, 3)) for _ in range(3)]
    return rho, u, rng.standard_normal((n, 3))


@pytest.mark.parametrize("momentum", [False, True])
@pytest.mark.parametrize("lumped", [False, True])
@pytest.mark.parametrize("scatter", [ng.SCATTER_ATOMIC, ng.SCATTER_COLOURED])
def test_mass_mesh_vs_oracle(gpu_ctx_factory, oracle, momentum, lumped, scatter):
    c, conn, gid = block_mesh(11, 9, 7, jitter=0.3, seed=21, z_ratio=1.1)
    n = c.shape[0]
    rho, u, gp = _states(n, 5)
    nd = 3 if momentum else 1
    t = dict(dt=0.02, gamma1=1.5, gamma2=-2.0, gamma3=0.5)      # BDF2, constant dt
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.field_set("density_nm1", rho[0])
    ctx.field_set("density_n", rho[1])
    ctx.field_set("density", rho[2])
    if momentum:
        ctx.field_set("velocity_nm1", u[0])
        ctx.field_set("velocity_n", u[1])
        ctx.field_set("velocity", u[2])
        ctx.field_set("dpdx", gp)
    ctx.build_elem_graph(nd)
    ctx.zero()
    kernel = ng.KERNEL_MOMENTUM_MASS if momentum else ng.KERNEL_CONTINUITY_MASS
    ctx.assemble(kernel, ng.default_assemble_opts(scatter=scatter, lumped_mass=int(lumped),
                                                  balanced_force=int(momentum), **t))
    vals, rhs = ctx.system()
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(n, conn, nd, gid)
    ov, orhs = oracle.assemble_mass(momentum, c, conn, rp, ci, lid, *rho, *(u if momentum else (None,) * 3),
                                    gpdx=gp if momentum else None, lumped=lumped, balanced_force=momentum, **t)
    check_csr_values(vals, ov, rp)
    check_vec(rhs, orhs)
    if momentum and lumped:
        # lumped: one diagonal entry per row
        nnz_rows = np.add.reduceat((vals != 0.0).astype(np.int64), rp[:-1])
        assert np.all(nnz_rows == 1)
    ctx.close()


def test_mass_two_state_and_additivity(gpu_ctx_factory, oracle):
    """N-1 unset reads N (a two-state field); the time term adds onto an
    assembled advection/diffusion system."""
    c, conn, gid = block_mesh(6, 5, 4, jitter=0.2, seed=2)
    n = c.shape[0]
    rho, u, gp = _states(n, 9)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.field_set("density_n", rho[1])
    ctx.field_set("density", rho[2])
    ctx.field_set("velocity_n", u[1])
    ctx.field_set("velocity", u[2])
    ctx.field_set("velocity_rtm", u[2])
    ctx.field_set("dpdx", gp)
    ctx.field_set("pressure", np.zeros(n))
    ctx.field_set("viscosity", 0.01 * np.ones(n))
    ctx.compute_mdot()
    ctx.build_elem_graph(3)
    o = ng.default_assemble_opts(dt=0.1, gamma1=1.5, gamma2=-2.0, gamma3=0.5, scatter=ng.SCATTER_COLOURED)
    ctx.zero()
    ctx.assemble(ng.KERNEL_MOMENTUM_ADV_DIFF, o)
    v_adv, r_adv = ctx.system()
    ctx.assemble(ng.KERNEL_MOMENTUM_MASS, o)
    v_sum, r_sum = ctx.system()
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(n, conn, 3, gid)
    ov, orhs = oracle.assemble_mass(True, c, conn, rp, ci, lid, rho[1], rho[1], rho[2], u[1], u[1], u[2], gpdx=gp,
                                    dt=0.1, gamma1=1.5, gamma2=-2.0, gamma3=0.5)
    check_csr_values(v_sum - v_adv, ov, rp)
    check_vec(r_sum - r_adv, orhs)
    ctx.close()


def test_mass_errors(gpu_ctx_factory):
    c, conn, gid = block_mesh(2, 2, 2)
    n = c.shape[0]
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.field_set("density", np.ones(n))
    ctx.build_elem_graph(1)
    with pytest.raises(ng.NaluError) as e:        # dt not set
        ctx.assemble(ng.KERNEL_CONTINUITY_MASS, ng.default_assemble_opts())
    assert e.value.status == -1
    with pytest.raises(ng.NaluError) as e:        # gamma1 = 0
        ctx.assemble(ng.KERNEL_CONTINUITY_MASS, ng.default_assemble_opts(dt=0.1, gamma1=0.0))
    assert e.value.status == -1
    with pytest.raises(ng.NaluError) as e:        # density state N missing
        ctx.assemble(ng.KERNEL_CONTINUITY_MASS, ng.default_assemble_opts(dt=0.1))
    assert e.value.status == -3
    ctx.field_set("density_n", np.ones(n))
    with pytest.raises(ng.NaluError) as e:        # numDof 1 graph, momentum kernel
        ctx.assemble(ng.KERNEL_MOMENTUM_MASS, ng.default_assemble_opts(dt=0.1))
    assert e.value.status == -3
    with pytest.raises(ng.NaluError) as e:
        ctx.assemble(6, ng.default_assemble_opts(dt=0.1))
    assert e.value.status == -1
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_MASS, ng.default_assemble_opts(dt=0.1))
    _, rhs = ctx.system()
    assert np.max(np.abs(rhs)) == 0.0             # rho^{n+1} = rho^n: no time term
    ctx.close()


def test_mass_follows_moved_coordinates(gpu_ctx_factory, oracle):
    """the SCV volumes are kept per element between calls; new coordinates
    (mesh motion) must reach the next time term"""
    c, conn, gid = block_mesh(5, 4, 3, jitter=0.2, seed=3)
    n = c.shape[0]
    rho, _, _ = _states(n, 1)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    ctx.field_set("density_n", rho[1])
    ctx.field_set("density", rho[2])
    ctx.build_elem_graph(1)
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(n, conn, 1, gid)
    o = ng.default_assemble_opts(dt=0.1, scatter=ng.SCATTER_ATOMIC)
    for scale in (1.0, 1.7, 0.6):
        moved = c * np.array([scale, 1.0, 1.0 / scale ** 0.5])
        ctx.field_set("coordinates", moved)
        ctx.zero()
        ctx.assemble(ng.KERNEL_CONTINUITY_MASS, o)
        _, rhs = ctx.system()
        _, orhs = oracle.assemble_mass(False, moved, conn, rp, ci, lid, rho[1], rho[1], rho[2], dt=0.1)
        check_vec(rhs, orhs)
    ctx.compute_dual_volume()
    assert np.allclose(ctx.field_get("dual_nodal_volume", (n,)), oracle.dual_volume(moved, conn), rtol=1e-13)
    ctx.close()


def test_mirror_algorithms(gpu_ctx_factory):
    """the reference-shaped drivers: element kernels with a BDF2 TimeIntegrator
    and a face algorithm over a side set sum to the direct calls"""
    from nalu_gb300.linear_system import (AssembleElemSolverAlgorithm, AssembleFaceElemSolverAlgorithm,
                                          ContinuityAdvElemKernel, ContinuityMassElemKernel,
                                          ContinuityInflowElemKernel, LinearSystem, TimeIntegrator)
    c, conn, gid = block_mesh(5, 4, 4, jitter=0.2, seed=9)
    n = c.shape[0]
    rho, u, gp = _states(n, 4)
    ctx = _ctx(gpu_ctx_factory, c, conn, gid)
    for name, v in (("density", rho[2]), ("density_n", rho[1]), ("density_nm1", rho[0]), ("velocity", u[2]),
                    ("pressure", np.zeros(n)), ("dpdx", gp), ("cont_velocity_bc", u[1])):
        ctx.field_set(name, v)
    ctx.faceset_skin(0)
    ls = LinearSystem(ctx, 1)
    alg = AssembleElemSolverAlgorithm(ls)
    alg.activeKernels_ = [ContinuityAdvElemKernel(), ContinuityMassElemKernel()]
    alg.initialize_connectivity()
    face = AssembleFaceElemSolverAlgorithm(ls, 0)
    face.activeKernels_ = [ContinuityInflowElemKernel()]
    ti = TimeIntegrator(0.05, 1.5, -2.0, 0.5)
    ls.zeroSystem()
    alg.execute(ti)
    face.execute(ti)
    v1, r1 = ctx.system()
    ctx.zero()
    tau = 0.05 / 1.5
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(proj_time_scale=tau))
    ctx.assemble(ng.KERNEL_CONTINUITY_MASS, ng.default_assemble_opts(dt=0.05, gamma1=1.5, gamma2=-2.0, gamma3=0.5))
    ctx.assemble_faces(0, ng.FACE_CONTINUITY_INFLOW, ng.default_assemble_opts(proj_time_scale=tau))
    v2, r2 = ctx.system()
    rp, _ = ctx.graph()
    check_csr_values(v1, v2, rp)
    check_vec(r1, r2)
    ctx.close()
