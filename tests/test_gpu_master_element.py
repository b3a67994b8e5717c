"""The batched Hex8 master element on the device against the oracle (which
reproduces the compiled reference bit for bit): SCS areas, SCS/SCV grad ops
(standard and shifted), SCV volumes and face grad ops on random distorted
elements.  Derivatives are exact; the rest within 1e-13 of each element's
largest entry (FMA contraction and the cofactor form of the areas)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BASE = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)


def _elements(n, seed):
    rng = np.random.default_rng(seed)
    c = (BASE[None] + 0.2 * rng.uniform(-1, 1, (n, 8, 3))) * rng.uniform(0.01, 3, (n, 1, 1))
    return c + rng.uniform(-2, 2, (n, 1, 3))


def _close(a, b, rel=1e-13):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.abs(b).reshape(b.shape[0], -1).max(axis=1)
    err = np.abs(a - b).reshape(b.shape[0], -1).max(axis=1)
    return bool(np.all(err <= rel * scale))


def test_master_element_batched(gpu_ctx_factory, oracle):
    ctx = gpu_ctx_factory()
    c = _elements(300, 4)
    a = ctx.hex_scs_determinant(c)
    assert _close(a, np.stack([oracle.scs_areav(x) for x in c]))
    for sh in (False, True):
        g, d = ctx.hex_scs_grad_op(c, sh)
        og = [oracle.scs_grad_op(x, sh) for x in c]
        assert np.array_equal(d, np.stack([o[1] for o in og]))
        assert _close(g, np.stack([o[0] for o in og]))
        g, d = ctx.hex_scv_grad_op(c, sh)
        og = [oracle.scv_grad_op(x, sh) for x in c]
        assert np.array_equal(d, np.stack([o[1] for o in og]))
        assert _close(g, np.stack([o[0] for o in og]))
        sides = np.arange(300) % 6
        g = ctx.hex_face_grad_op(c, sides, sh)
        assert _close(g, np.stack([oracle.face_grad_op(s, x, sh)[0] for s, x in zip(sides, c)]))
    v = ctx.hex_scv_determinant(c)
    assert _close(v, np.stack([oracle.scv_volume(x) for x in c]))
    ctx.close()


def test_master_element_golds_and_errors(gpu_ctx_factory, golds):
    import nalu_gb300 as ng
    ctx = gpu_ctx_factory()
    g = golds["hex8_scv_grad_op"]
    c = np.array(g["coords"]).reshape(1, 8, 3)
    gop, _ = ctx.hex_scv_grad_op(c)
    assert np.max(np.abs(gop.ravel() - g["gradop"])) <= g["tol"]
    gop, _ = ctx.hex_scv_grad_op(c, True)
    assert np.max(np.abs(gop.ravel() - g["shifted_gradop"])) <= g["tol"]
    assert np.max(np.abs(ctx.hex_scv_determinant(BASE[None]) - 0.125)) <= 1e-16
    inverted = BASE[None][:, [4, 5, 6, 7, 0, 1, 2, 3]]        # mirrored element: det(J) < 0
    with pytest.raises(ng.NaluError) as e:
        ctx.hex_scs_grad_op(inverted)
    assert e.value.status == -4
    with pytest.raises(ng.NaluError) as e:
        ctx.hex_face_grad_op(BASE[None], [6])
    assert e.value.status == -1
    ctx.close()


def test_master_element_properties(gpu_ctx_factory):
    """the reference's master-element property tests
    (unit_tests/UnitTestMasterElements.C:104-159, 185-228): the grad ops of
    every point set reproduce the gradient of a random linear field exactly on
    distorted elements; SCV volumes scale with det(QR) under a linear map"""
    ctx = gpu_ctx_factory()
    rng = np.random.default_rng(0)
    c = _elements(200, 7)
    a, b = rng.standard_normal(3), rng.standard_normal()
    f = c @ a + b                                           # [200, 8]
    for sh in (False, True):
        for g in (ctx.hex_scs_grad_op(c, sh)[0], ctx.hex_scv_grad_op(c, sh)[0],
                  ctx.hex_face_grad_op(c, np.arange(200) % 6, sh)):
            grad = np.einsum("eknd,en->ekd", g, f)
            assert np.max(np.abs(grad - a)) <= 1e-10 * np.max(np.abs(a))
    q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    m = q @ np.diag(rng.uniform(0.5, 1.5, 3))
    if np.linalg.det(m) < 0:
        m[:, 0] *= -1.0
    v0 = ctx.hex_scv_determinant(c)
    v1 = ctx.hex_scv_determinant(c @ m.T)
    assert np.max(np.abs(v1 - np.linalg.det(m) * v0) / np.abs(v1)) <= 1e-12
    ctx.close()
