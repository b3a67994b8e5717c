"""GPU parity of the nodal geometry and gradient calls against the oracle:
dual_nodal_volume (HexSCV::determinant scattered to the nodes) and the element
part of the projected nodal gradient (AssembleNodalGradElemAlgorithm and its
velocity form).  The device sums element contributions with atomics, so the
order of the (at most 8 per node) additions varies: tolerance
|a - b| <= 1e-13 max|b| for the gradient (FP64 and df64 arithmetic).  Volumes: 1e-13 relative.  The
device evaluates Grandy's volume in its face form about the element centroid;
the reference's corner-coordinate form (which the oracle reproduces bit for
bit) carries up to ~1e-14 relative rounding of its own on small elements away
from the origin, the face form ~5e-16 (checked against exact rational
arithmetic)."""
import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import block_mesh

pytestmark = pytest.mark.gpu


def _mesh(gpu_ctx_factory, c, conn):
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn)
    return ctx


@pytest.mark.parametrize("case", ["unit", "jitter", "stretched"])
def test_dual_volume(gpu_ctx_factory, oracle, case):
    if case == "unit":
        c, conn, _ = block_mesh(1, 1, 1)
    elif case == "jitter":
        c, conn, _ = block_mesh(17, 13, 11, jitter=0.35, seed=4)
    else:
        c, conn, _ = block_mesh(12, 12, 24, z_ratio=1.15, lengths=(2.0, 1.0, 0.5))
    ctx = _mesh(gpu_ctx_factory, c, conn)
    ctx.compute_dual_volume()
    got = ctx.field_get("dual_nodal_volume", (c.shape[0],))
    ref = oracle.dual_volume(c, conn)
    assert np.all(np.abs(got - ref) <= 1e-13 * np.abs(ref))
    for e in sorted({0, conn.shape[0] // 2, conn.shape[0] - 1}):
        v = ctx.capture_scv_volumes(e)
        assert np.max(np.abs(v - oracle.scv_volume(c[conn[e]]))) <= 1e-15 * max(1.0, np.max(np.abs(v)))
    if case == "unit":
        assert np.max(np.abs(got - 0.125)) <= 1e-15
    ctx.close()


@pytest.mark.parametrize("arith", [ng.ARITH_FP64, ng.ARITH_DF64])
@pytest.mark.parametrize("shifted", [False, True])
def test_nodal_gradient(gpu_ctx_factory, oracle, shifted, arith):
    c, conn, _ = block_mesh(19, 14, 9, jitter=0.3, seed=8)
    n = c.shape[0]
    rng = np.random.default_rng(11)
    p = np.sin(2.0 * c[:, 0]) * np.cos(c[:, 1]) + 0.1 * rng.standard_normal(n)
    u = np.stack([np.cos(c[:, 2]), c[:, 0] * c[:, 1], np.exp(-c[:, 0])], 1) + 0.05 * rng.standard_normal((n, 3))
    ctx = _mesh(gpu_ctx_factory, c, conn)
    ctx.compute_dual_volume()
    vol = oracle.dual_volume(c, conn)
    ctx.field_set("pressure", p)
    ctx.compute_nodal_gradient("pressure", "dpdx", shifted, arith)
    got = ctx.field_get("dpdx", (n, 3))
    ref = oracle.nodal_grad_elem(c, conn, p, vol, shifted)
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    ctx.field_set("velocity", u)
    ctx.compute_nodal_gradient("velocity", "dudx", shifted, arith)
    got = ctx.field_get("dudx", (n, 9)).reshape(n, 3, 3)
    ref = oracle.nodal_grad_elem(c, conn, u, vol, shifted)
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    # a second call overwrites (zeroes first) rather than accumulates
    ctx.compute_nodal_gradient("velocity", "dudx", shifted, arith)
    again = ctx.field_get("dudx", (n, 9)).reshape(n, 3, 3)
    assert np.max(np.abs(again - ref)) <= 1e-13 * np.max(np.abs(ref))
    ctx.close()


def test_nodal_gradient_feeds_continuity(gpu_ctx_factory, oracle):
    """dpdx computed on the device is the Gpdx the continuity kernel reads:
    the assembled rhs equals the one assembled from the oracle's gradient."""
    c, conn, gid = block_mesh(8, 7, 6, jitter=0.25, seed=3)
    n = c.shape[0]
    rng = np.random.default_rng(5)
    ctx = _mesh(gpu_ctx_factory, c, conn)
    ctx.build_elem_graph(1)
    ctx.field_set("velocity", rng.standard_normal((n, 3)))
    ctx.field_set("density", 1.0 + 0.1 * rng.random(n))
    p = rng.standard_normal(n)
    ctx.field_set("pressure", p)
    ctx.compute_dual_volume()
    ctx.compute_nodal_gradient("pressure", "dpdx")
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
    _, rhs_dev = ctx.system()
    ctx.field_set("dpdx", oracle.nodal_grad_elem(c, conn, p, oracle.dual_volume(c, conn)))
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
    _, rhs_orc = ctx.system()
    assert np.max(np.abs(rhs_dev - rhs_orc)) <= 1e-12 * np.max(np.abs(rhs_orc))
    ctx.close()


def test_geometry_errors(gpu_ctx_factory):
    c, conn, _ = block_mesh(2, 2, 2)
    ctx = _mesh(gpu_ctx_factory, c, conn)
    ctx.field_set("pressure", np.zeros(c.shape[0]))
    with pytest.raises(ng.NaluError) as e:
        ctx.compute_nodal_gradient("pressure", "dpdx")
    assert e.value.status == -3
    ctx.compute_dual_volume()
    for src, dst in [("pressure", "dudx"), ("velocity", "dpdx"), ("pressure", "pressure"),
                     ("pressure", "mass_flow_rate_scs")]:
        with pytest.raises(ng.NaluError) as e:
            ctx.compute_nodal_gradient(src, dst)
        assert e.value.status == -1, (src, dst)
    with pytest.raises(ng.NaluError):
        ctx.capture_scv_volumes(conn.shape[0])
    ctx.close()
