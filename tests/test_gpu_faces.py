"""GPU parity of the boundary-face path through the C ABI against the oracle:
the exposed-face skin (exact), exposed area vectors, the boundary closure of
the projected nodal gradient, and the ContinuityInflow / ContinuityOpen face
kernels summed into the CRS system (helpers.REL / FLOOR for assembled values;
1e-13 max-relative for gradients, whose atomics add in varying order)."""
import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import block_mesh, check_csr_values, check_dense, check_vec

pytestmark = pytest.mark.gpu


def _mesh(gpu_ctx_factory, c, conn, gid=None):
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    return ctx


def _plane_faces(oracle, c, conn, fe, fs, axis, value):
    keep = [k for k in range(fe.shape[0])
            if np.allclose(c[conn[fe[k]][oracle.side_nodes(fs[k])], axis], value)]
    return fe[keep], fs[keep]


@pytest.mark.parametrize("permuted", [False, True])
def test_skin_and_areas(gpu_ctx_factory, oracle, permuted):
    c, conn, gid = block_mesh(7, 5, 4, jitter=0.3, seed=12)
    if permuted:   # node global ids in reverse: LIDs differ from caller indices
        gid = gid[::-1].copy()
    ctx = _mesh(gpu_ctx_factory, c, conn, gid)
    n = ctx.faceset_skin(3)
    fe, fs = oracle.skin(conn)
    assert n == fe.shape[0] == 2 * (7 * 5 + 5 * 4 + 4 * 7)
    e, s = ctx.faceset_get(3)
    assert np.array_equal(e, fe) and np.array_equal(s, fs)
    a = ctx.faceset_exposed_area(3)
    ref = np.stack([oracle.quad_areav(c[conn[fe[k]][oracle.side_nodes(fs[k])]]) for k in range(n)])
    assert np.max(np.abs(a - ref)) <= 1e-15 * max(1.0, np.max(np.abs(ref)))
    # the skin of a box closes: total exposed area vector 0
    assert np.max(np.abs(a.sum((0, 1)))) <= 1e-13
    ctx.close()


@pytest.mark.parametrize("shifted", [False, True])
def test_nodal_gradient_with_boundary(gpu_ctx_factory, oracle, shifted):
    c, conn, gid = block_mesh(9, 8, 6, jitter=0.3, seed=4)
    n = c.shape[0]
    rng = np.random.default_rng(3)
    p = np.sin(3.0 * c[:, 0]) + c[:, 1] * c[:, 2] + 0.1 * rng.standard_normal(n)
    u = np.stack([c[:, 1] ** 2, np.cos(c[:, 0]), c[:, 2]], 1) + 0.05 * rng.standard_normal((n, 3))
    ctx = _mesh(gpu_ctx_factory, c, conn, gid)
    ctx.compute_dual_volume()
    nf = ctx.faceset_skin(0)
    fe, fs = oracle.skin(conn)
    assert nf == fe.shape[0]
    vol = oracle.dual_volume(c, conn)
    for name, dst, q, shape in (("pressure", "dpdx", p, (n, 3)), ("velocity", "dudx", u, (n, 9))):
        ctx.field_set(name, q)
        ctx.compute_nodal_gradient(name, dst, shifted)
        ctx.nodal_gradient_boundary(0, name, dst, shifted)
        got = ctx.field_get(dst, shape)
        ref = oracle.nodal_grad_elem(c, conn, q, vol, shifted)
        oracle.nodal_grad_boundary(c, conn, fe, fs, q, vol, ref, shifted)
        ref = ref.reshape(shape)
        assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref)), name
    ctx.close()


def test_nodal_gradient_linear_exact_on_device(gpu_ctx_factory):
    """element part + closure: exact gradient of a linear field at every node of
    an affine mesh"""
    c, conn, _ = block_mesh(5, 4, 6)
    m = np.array([[1.0, 0.3, 0.0], [-0.2, 0.9, 0.1], [0.4, 0.0, 1.3]])
    c = c @ m.T
    g = np.array([0.7, -1.3, 2.1])
    ctx = _mesh(gpu_ctx_factory, c, conn)
    ctx.compute_dual_volume()
    ctx.faceset_skin(5)
    ctx.field_set("pressure", 0.4 + c @ g)
    ctx.compute_nodal_gradient("pressure", "dpdx")
    ctx.nodal_gradient_boundary(5, "pressure", "dpdx")
    assert np.max(np.abs(ctx.field_get("dpdx", (c.shape[0], 3)) - g)) <= 1e-12
    ctx.close()


def _bc_fields(c, seed):
    rng = np.random.default_rng(seed)
    n = c.shape[0]
    return dict(rho=1.0 + 0.2 * rng.random(n), u=rng.standard_normal((n, 3)), p=rng.standard_normal(n),
                pbc=0.3 * rng.standard_normal(n), gp=rng.standard_normal((n, 3)))


def test_continuity_inflow(gpu_ctx_factory, oracle):
    c, conn, gid = block_mesh(8, 6, 5, jitter=0.25, seed=8, z_ratio=1.1)
    f = _bc_fields(c, 2)
    fe, fs = _plane_faces(oracle, c, conn, *oracle.skin(conn), axis=0, value=0.0)
    assert fe.shape[0] == 6 * 5
    ctx = _mesh(gpu_ctx_factory, c, conn, gid)
    ctx.faceset_define(1, fe, fs)
    ctx.field_set("density", f["rho"])
    ctx.field_set("cont_velocity_bc", f["u"])
    ctx.build_elem_graph(1)
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(c.shape[0], conn, 1, gid)
    for smdot in (0, 1):
        o = ng.default_assemble_opts(proj_time_scale=0.4, shift_mdot=smdot)
        ctx.zero()
        ctx.assemble_faces(1, ng.FACE_CONTINUITY_INFLOW, o)
        vals, rhs = ctx.system()
        ov, orhs = oracle.assemble_faces(oracle.FACE_CONTINUITY_INFLOW, c, conn, fe, fs, rp, ci, lid, f["rho"], f["u"],
                                         proj_time_scale=0.4, shift_mdot=smdot)
        assert np.all(vals == 0.0)
        check_vec(rhs, orhs)
        lhs, r8 = ctx.capture_face(1, ng.FACE_CONTINUITY_INFLOW, 3, o)
        e = conn[fe[3]]
        _, oref = oracle.continuity_inflow_face(fs[3], c[e], f["rho"][e], f["u"][e], 0.4, smdot)
        check_vec(r8, oref)
        assert np.all(lhs == 0.0)
    ctx.close()


@pytest.mark.parametrize("kw", [{}, {"shift_poisson": 1}, {"reduced_sens": 1}, {"shift_mdot": 1},
                                {"reduced_sens": 1, "shift_poisson": 1, "shift_mdot": 1}])
def test_continuity_open(gpu_ctx_factory, oracle, kw):
    c, conn, gid = block_mesh(7, 6, 5, jitter=0.25, seed=5, z_ratio=1.1)
    f = _bc_fields(c, 6)
    fe, fs = _plane_faces(oracle, c, conn, *oracle.skin(conn), axis=0, value=1.0)
    nf = fe.shape[0]
    dynp = 0.05 * np.random.default_rng(1).standard_normal((nf, 4))
    ctx = _mesh(gpu_ctx_factory, c, conn, gid)
    ctx.faceset_define(2, fe, fs)
    ctx.faceset_dynamic_pressure(2, dynp)
    for name, key in (("density", "rho"), ("velocity", "u"), ("pressure", "p"), ("pressure_bc", "pbc"),
                      ("dpdx", "gp")):
        ctx.field_set(name, f[key])
    ctx.build_elem_graph(1)
    rp, ci = ctx.graph()
    _, _, lid = oracle.graph(c.shape[0], conn, 1, gid)
    o = ng.default_assemble_opts(proj_time_scale=0.3, **kw)
    ctx.zero()
    ctx.assemble_faces(2, ng.FACE_CONTINUITY_OPEN, o)
    vals, rhs = ctx.system()
    ov, orhs = oracle.assemble_faces(oracle.FACE_CONTINUITY_OPEN, c, conn, fe, fs, rp, ci, lid, f["rho"], f["u"],
                                     p=f["p"], pbc=f["pbc"], gpdx=f["gp"], dynp=dynp, proj_time_scale=0.3,
                                     shift_grad_op=kw.get("shift_poisson", 0), reduced_sens=kw.get("reduced_sens", 0),
                                     shift_mdot=kw.get("shift_mdot", 0))
    check_csr_values(vals, ov, rp)
    check_vec(rhs, orhs)
    for k in (0, nf // 2, nf - 1):
        lhs, r8 = ctx.capture_face(2, ng.FACE_CONTINUITY_OPEN, k, o)
        e = conn[fe[k]]
        ol, orr = oracle.continuity_open_face(fs[k], c[e], f["p"][e], f["pbc"][e], f["rho"][e], f["u"][e], f["gp"][e],
                                              dynp[k], 0.3, kw.get("shift_poisson", 0), kw.get("reduced_sens", 0),
                                              kw.get("shift_mdot", 0))
        check_dense(lhs, ol)
        check_vec(r8, orr)
    ctx.close()


def test_face_errors(gpu_ctx_factory):
    c, conn, gid = block_mesh(2, 2, 2)
    n = c.shape[0]
    ctx = _mesh(gpu_ctx_factory, c, conn, gid)
    with pytest.raises(ng.NaluError) as e:
        ctx.faceset_get(4)
    assert e.value.status == -3
    with pytest.raises(ng.NaluError) as e:
        ctx.faceset_define(0, [0, 1], [0, 6])
    assert e.value.status == -1
    with pytest.raises(ng.NaluError) as e:
        ctx.faceset_define(0, [0, 8], [0, 1])
    assert e.value.status == -1
    with pytest.raises(ng.NaluError) as e:
        ctx.faceset_define(16, [0], [0])
    assert e.value.status == -1
    ctx.faceset_define(0, [0, 1], [3, 1])
    ctx.field_set("density", np.ones(n))
    with pytest.raises(ng.NaluError) as e:     # cont_velocity_bc missing
        ctx.assemble_faces(0, ng.FACE_CONTINUITY_INFLOW)
    assert e.value.status == -3
    ctx.field_set("cont_velocity_bc", np.ones((n, 3)))
    ctx.build_elem_graph(3)
    with pytest.raises(ng.NaluError) as e:     # numDof 3 graph
        ctx.assemble_faces(0, ng.FACE_CONTINUITY_INFLOW)
    assert e.value.status == -3
    with pytest.raises(ng.NaluError) as e:     # gradient closure before the element part
        ctx.compute_dual_volume()
        ctx.field_set("pressure", np.zeros(n))
        ctx.nodal_gradient_boundary(0, "pressure", "dpdx")
    assert e.value.status == -3
    ctx.close()


def test_face_set_edge_cases(gpu_ctx_factory, oracle):
    c, conn, gid = block_mesh(1, 1, 1)
    n = c.shape[0]
    ctx = _mesh(gpu_ctx_factory, c, conn, gid)
    # one element: all six sides exposed, in side order
    assert ctx.faceset_skin(0) == 6
    e, s = ctx.faceset_get(0)
    assert np.array_equal(e, np.zeros(6)) and np.array_equal(s, np.arange(6))
    a = ctx.faceset_exposed_area(0)
    assert np.max(np.abs(a.sum(axis=(0, 1)))) <= 1e-16 and np.allclose(np.abs(a).sum(axis=(1, 2)), 1.0)
    # an empty set is valid and does nothing
    ctx.faceset_define(1, [], [])
    assert ctx.faceset_get(1)[0].size == 0 and ctx.faceset_exposed_area(1).shape == (0, 4, 3)
    ctx.field_set("density", np.ones(n))
    ctx.field_set("cont_velocity_bc", np.ones((n, 3)))
    ctx.build_elem_graph(1)
    ctx.zero()
    ctx.assemble_faces(1, ng.FACE_CONTINUITY_INFLOW)
    vals, rhs = ctx.system()
    assert not vals.any() and not rhs.any()
    # redefining replaces; a new mesh clears every set
    ctx.faceset_define(1, [0], [5])
    assert ctx.faceset_get(1)[1].tolist() == [5]
    ctx.mesh_create(c, conn, gid)
    with pytest.raises(ng.NaluError) as err:
        ctx.faceset_get(1)
    assert err.value.status == -3
    ctx.close()
