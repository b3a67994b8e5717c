"""One continuity (pressure-projection) step end to end on the device, against
the oracle running the same pipeline on the CPU:

  dual_nodal_volume -> projected nodal gradient of p with its boundary closure
  (Gpdx) -> ContinuityAdv (interior) + ContinuityMass (BDF2 time term) +
  ContinuityInflow (x = 0) + ContinuityOpen (x = 1) summed into one system ->
  GMRES solve.

The assembled system is compared entry by entry (helpers.REL / FLOOR); the
device solution (true residual <= 1e-11) against the oracle's solution of the
oracle's system (<= 1e-13), within 1e-6 of the largest entry, the error that
cond(A) times those residuals allows."""
import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import block_mesh, check_csr_values, check_vec

pytestmark = pytest.mark.gpu


def test_continuity_step(gpu_ctx_factory, oracle):
    c, conn, gid = block_mesh(10, 8, 6, jitter=0.2, seed=17, z_ratio=1.05)
    n = c.shape[0]
    rng = np.random.default_rng(23)
    x, y, z = c[:, 0], c[:, 1], c[:, 2]
    u = np.stack([1.0 + 0.2 * np.sin(2 * y) * np.cos(z), 0.1 * np.sin(3 * x), 0.05 * np.cos(2 * x + y)], 1)
    rho_np1 = 1.0 + 0.05 * np.sin(x + 2 * z)
    rho_n = rho_np1 - 0.01 * np.cos(y)
    rho_nm1 = rho_n - 0.01 * np.cos(y)
    p = 0.3 * x * x - 0.1 * y * z + 0.01 * rng.standard_normal(n)
    pbc = np.zeros(n)
    dt, g1, g2, g3 = 0.02, 1.5, -2.0, 0.5
    tau = dt / g1

    fe_all, fs_all = oracle.skin(conn)

    def plane(axis, value):
        keep = [k for k in range(fe_all.shape[0])
                if np.allclose(c[conn[fe_all[k]][oracle.side_nodes(fs_all[k])], axis], value)]
        return fe_all[keep], fs_all[keep]
    fe_in, fs_in = plane(0, 0.0)
    fe_out, fs_out = plane(0, 1.0)

    # ---- device ----
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    for name, v in (("velocity", u), ("cont_velocity_bc", u), ("density", rho_np1), ("density_n", rho_n),
                    ("density_nm1", rho_nm1), ("pressure", p), ("pressure_bc", pbc)):
        ctx.field_set(name, v)
    ctx.compute_dual_volume()
    ctx.faceset_skin(0)
    ctx.faceset_define(1, fe_in, fs_in)
    ctx.faceset_define(2, fe_out, fs_out)
    ctx.compute_nodal_gradient("pressure", "dpdx")
    ctx.nodal_gradient_boundary(0, "pressure", "dpdx")
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(proj_time_scale=tau))
    ctx.assemble(ng.KERNEL_CONTINUITY_MASS, ng.default_assemble_opts(dt=dt, gamma1=g1, gamma2=g2, gamma3=g3))
    ctx.assemble_faces(1, ng.FACE_CONTINUITY_INFLOW, ng.default_assemble_opts(proj_time_scale=tau))
    ctx.assemble_faces(2, ng.FACE_CONTINUITY_OPEN, ng.default_assemble_opts(proj_time_scale=tau))
    ctx.load_complete()
    vals, rhs = ctx.system()
    rp, ci = ctx.graph()
    info = ctx.solve(ng.default_solver_opts(method=ng.SOLVER_GMRES, restart=60, tol=1e-11, max_iters=6000))
    assert info.status == 0 and info.true_rel_res <= 1e-11
    x_dev = ctx.solution()
    gp_dev = ctx.field_get("dpdx", (n, 3))

    # ---- oracle ----
    _, _, lid = oracle.graph(n, conn, 1, gid)
    vol = oracle.dual_volume(c, conn)
    gp = oracle.nodal_grad_elem(c, conn, p, vol)
    oracle.nodal_grad_boundary(c, conn, fe_all, fs_all, p, vol, gp)
    assert np.max(np.abs(gp_dev - gp)) <= 1e-13 * np.max(np.abs(gp))
    ov, orhs = oracle.assemble(oracle.KERNEL_CONTINUITY_ADV, c, conn, rp, ci, lid, scalar=p, coeff=rho_np1, vec=u,
                               vec2=gp, opts=oracle.opts_block(proj_time_scale=tau))
    mv, mr = oracle.assemble_mass(False, c, conn, rp, ci, lid, rho_nm1, rho_n, rho_np1, dt=dt, gamma1=g1, gamma2=g2,
                                  gamma3=g3)
    iv, ir = oracle.assemble_faces(oracle.FACE_CONTINUITY_INFLOW, c, conn, fe_in, fs_in, rp, ci, lid, rho_np1, u,
                                   proj_time_scale=tau)
    pv, pr = oracle.assemble_faces(oracle.FACE_CONTINUITY_OPEN, c, conn, fe_out, fs_out, rp, ci, lid, rho_np1, u,
                                   p=p, pbc=pbc, gpdx=gp, proj_time_scale=tau)
    sv, sr = ov + mv + iv + pv, orhs + mr + ir + pr
    check_csr_values(vals, sv, rp)
    check_vec(rhs, sr)
    x_orc, _, res = oracle.gmres_jacobi(rp, ci, sv, sr, restart=60, tol=1e-13, max_it=40000)
    assert res <= 1e-12
    assert np.max(np.abs(x_dev - x_orc)) <= 1e-6 * np.max(np.abs(x_orc))
    ctx.close()
