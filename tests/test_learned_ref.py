"""CPU checks of the FP64 reference model of the learned preconditioner."""
import numpy as np

import mlp_ref as M


def test_reference_gradient_finite_differences():
    P = M.random_params(3)
    st, rf, tg = M.random_samples(6, 4)
    loss, g = M.loss_and_grad(P, st, rf, tg)
    rng = np.random.default_rng(5)
    idx = np.concatenate([rng.choice(np.arange(off, off + int(np.prod(s))), 6, replace=int(np.prod(s)) < 6)
                          for off, s in M.SL.values()])
    h = 1e-6
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (M.loss_and_grad(Pp, st, rf, tg)[0] - M.loss_and_grad(Pm, st, rf, tg)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_untrained_output_layer_gives_jacobi():
    """w4 = b4 = 0: the stencil is zero, so the preconditioner is D^-1."""
    P = M.random_params(7)
    o, _ = M.SL["w4"]
    P[o:o + 65] = 0.0
    st, _, _ = M.random_samples(5, 8)
    assert np.all(M.stencil(P, st) == 0.0)


def test_slot_map_structured():
    from nalu_gb300.meshgen import block_mesh
    c, conn, _ = block_mesh(3)
    nbr = M.slot_map(conn, c.shape[0])
    # interior node (1,1,1) of a 4x4x4 node grid has all 27 neighbours at the lexicographic offsets
    i = 1 + 4 * (1 + 4 * 1)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                s = 9 * (dz + 1) + 3 * (dy + 1) + dx + 1
                assert nbr[i, s] == i + dx + 4 * (dy + 4 * dz)
    # corner node 0 has 8
    assert (nbr[0] >= 0).sum() == 8
