"""Staged field uploads (nalu_field_set_async): pipelined steps of
upload -> assemble -> download give the same systems as blocking uploads
(coloured scatter: deterministic, compared exactly), in caller node order
with and without permuted global ids; a later blocking upload wins over an
earlier staged one."""
import numpy as np
import pytest

import nalu_gb300 as ng
from helpers import block_mesh, continuity_fields

pytestmark = pytest.mark.gpu

NAMES = ("velocity", "density", "pressure", "dpdx")


def _inputs(c, k):
    u, rho, p, gp = continuity_fields(c, seed=40 + k)
    return dict(velocity=u, density=rho, pressure=p, dpdx=gp)


@pytest.mark.parametrize("permuted", [False, True])
def test_pipelined_uploads_match_blocking(gpu_ctx_factory, permuted):
    c, conn, gid = block_mesh(9, 7, 6, jitter=0.2, seed=3)
    if permuted:
        gid = gid[::-1].copy()
    o = ng.default_assemble_opts(scatter=ng.SCATTER_COLOURED)
    steps = [_inputs(c, k) for k in range(4)]
    # reference: blocking uploads, one step at a time
    ref = ng.Context(0)
    ref.mesh_create(c, conn, gid)
    ref.build_elem_graph(1)
    want = []
    for f in steps:
        for nm in NAMES:
            ref.field_set(nm, f[nm])
        ref.zero()
        ref.assemble(ng.KERNEL_CONTINUITY_ADV, o)
        want.append(ref.system())
    ref.close()
    # pipelined: staged uploads from pinned memory, downloads overlapping
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    ctx.build_elem_graph(1)
    nr, nnz, _ = ctx.sizes()
    pins = [{nm: ng.PinnedArray(f[nm].shape) for nm in NAMES} for f in steps]
    outs = [(ng.PinnedArray((nnz,)), ng.PinnedArray((nr,))) for _ in steps]
    for pin, f in zip(pins, steps):
        for nm in NAMES:
            pin[nm].array[...] = f[nm]
    for k in range(len(steps)):
        for nm in NAMES:
            ctx.field_set_async_ptr(nm, pins[k][nm].ptr, pins[k][nm].array.size)
        ctx.zero()
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV, o)
        ctx.system_to_ptr_async(outs[k][0].ptr, outs[k][1].ptr)
        ctx.copy_wait() if k == len(steps) - 1 else None
    ctx.synchronize()
    for k, (v, r) in enumerate(want):
        assert np.array_equal(outs[k][0].array, v), k
        assert np.array_equal(outs[k][1].array, r), k
    # the staged upload is what field_get sees; a later blocking upload wins
    extra = _inputs(c, 9)
    pin = ng.PinnedArray(extra["pressure"].shape)
    pin.array[...] = extra["pressure"]
    ctx.field_set_async_ptr("pressure", pin.ptr, pin.array.size)
    assert np.array_equal(ctx.field_get("pressure", extra["pressure"].shape), extra["pressure"])
    ctx.field_set_async_ptr("pressure", pin.ptr, pin.array.size)
    ctx.field_set("pressure", steps[0]["pressure"])
    ctx.synchronize()
    assert np.array_equal(ctx.field_get("pressure", extra["pressure"].shape), steps[0]["pressure"])
    for a in [pin] + [x for d in pins for x in d.values()] + [x for pair in outs for x in pair]:
        a.free()
    ctx.close()


def test_staged_coordinates_refresh_volumes(gpu_ctx_factory, oracle):
    """coordinates uploaded through the staged path reach the cached SCV
    volumes (the time term) and the dual volume"""
    c, conn, gid = block_mesh(4, 4, 3, jitter=0.2, seed=8)
    n = c.shape[0]
    ctx = gpu_ctx_factory()
    ctx.mesh_create(c, conn, gid)
    ctx.compute_dual_volume()
    moved = c * 1.3
    pin = ng.PinnedArray(moved.shape)
    pin.array[...] = moved
    ctx.field_set_async_ptr("coordinates", pin.ptr, pin.array.size)
    ctx.compute_dual_volume()
    assert np.allclose(ctx.field_get("dual_nodal_volume", (n,)), oracle.dual_volume(moved, conn), rtol=1e-13)
    ctx.synchronize()
    pin.free()
    ctx.close()
