"""The restructured element math of the GPU kernels (nalu_gb300/csrc/hex8_elem.h),
compiled for the host, against the oracle and the reference's golds (CPU)."""
import ctypes

import numpy as np
import pytest

from helpers import TrigFields, block_mesh, check_dense

P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
BASE = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)


def _hc_scalar(L, c, q, k, sh):
    lhs, rhs = np.zeros(64), np.zeros(8)
    L.hc_scalar_diff(P(np.ascontiguousarray(c)), P(q), P(k), int(sh), P(lhs), P(rhs))
    return lhs.reshape(8, 8), rhs


def _hc_cont(L, c, u, rho, p, gp, tau, sm, sp, rd):
    lhs, rhs = np.zeros(64), np.zeros(8)
    L.hc_continuity(P(np.ascontiguousarray(c)), P(np.ascontiguousarray(u)), P(rho), P(p), P(np.ascontiguousarray(gp)),
                    float(tau), sm, sp, rd, P(lhs), P(rhs))
    return lhs.reshape(8, 8), rhs


def test_golds_through_device_math(elemcheck, golds):
    c, conn, gid = block_mesh(1, 1, 1)
    e = conn[0]
    lhs, rhs = _hc_scalar(elemcheck, c[e], TrigFields.temperature(c)[e], np.ones(8), 0)
    assert np.max(np.abs(lhs.ravel() - golds["scalar_diff"]["lhs"])) <= 1e-15
    assert np.max(np.abs(rhs)) <= 1e-15
    for key, opts in [("continuity_default", (0, 0, 0)), ("continuity_reduced_sens", (0, 0, 1)),
                      ("continuity_reduced_shift", (0, 1, 1))]:
        lhs, rhs = _hc_cont(elemcheck, c[e], TrigFields.velocity(c)[e], np.ones(8), TrigFields.pressure(c)[e],
                            TrigFields.dpdx(c)[e], 1.0, *opts)
        assert np.max(np.abs(lhs.ravel() - golds[key]["lhs"])) <= 1e-15, key
        assert np.max(np.abs(rhs - golds[key]["rhs"])) <= 1e-15, key


@pytest.mark.parametrize("shift", [0, 1])
def test_scalar_diff_random_elements(elemcheck, oracle, shift):
    rng = np.random.default_rng(10 + shift)
    for t in range(400):
        h = rng.uniform(1 / 256, 1 / 8)
        c = (BASE + 0.2 * rng.uniform(-1, 1, (8, 3))) * h + rng.uniform(0, 1, 3)
        q, k = rng.uniform(0, 1, 8), rng.uniform(0.5, 2, 8)
        l1, r1 = oracle.scalar_diff_elem(c, q, k, shift)
        l2, r2 = _hc_scalar(elemcheck, c, q, k, shift)
        check_dense(l2, l1, what="lhs")
        check_dense(r2[None], r1[None], what="rhs")


@pytest.mark.parametrize("opts", [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 0, 0), (1, 1, 1)])
def test_continuity_random_elements(elemcheck, oracle, opts):
    rng = np.random.default_rng(20)
    for t in range(300):
        h = rng.uniform(1 / 256, 1 / 8)
        c = (BASE + 0.2 * rng.uniform(-1, 1, (8, 3))) * h + rng.uniform(0, 1, 3)
        u, gp = rng.normal(size=(8, 3)), rng.normal(size=(8, 3))
        rho, p, tau = rng.uniform(0.5, 2, 8), rng.normal(size=8), rng.uniform(0.1, 2)
        l1, r1 = oracle.continuity_adv_elem(c, u, rho, p, gp, tau, *opts)
        l2, r2 = _hc_cont(elemcheck, c, u, rho, p, gp, tau, *opts)
        check_dense(l2, l1, what="lhs")
        check_dense(r2[None], r1[None], what="rhs")


@pytest.mark.parametrize("sm,sp", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_mdot_random_elements(elemcheck, oracle, sm, sp):
    rng = np.random.default_rng(30)
    for t in range(200):
        h = rng.uniform(1 / 128, 1 / 8)
        c = np.ascontiguousarray((BASE + 0.2 * rng.uniform(-1, 1, (8, 3))) * h + rng.uniform(0, 1, 3))
        u, gp = np.ascontiguousarray(rng.normal(size=(8, 3))), np.ascontiguousarray(rng.normal(size=(8, 3)))
        rho, p, tau = rng.uniform(0.5, 2, 8), rng.normal(size=8), rng.uniform(0.1, 2)
        m1 = oracle.mdot_elem(c, rho, u, p, gp, tau, sm, sp)
        m2 = np.zeros(12)
        elemcheck.hc_mdot(P(c), P(rho), P(u), P(p), P(gp), float(tau), sm, sp, P(m2))
        check_dense(m2[None], m1[None], what="mdot")


@pytest.mark.parametrize("sm,sp", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_mdot_df_random_elements(elemcheck, oracle, sm, sp):
    """df64 mdot (the ARITH_DF64 ComputeMdot kernel's element math) against the
    FP64 oracle: |a - b| <= 1e-12 (max |b|) + ..., helpers.check_dense"""
    rng = np.random.default_rng(31)
    for t in range(200):
        h = rng.uniform(1 / 128, 1 / 8)
        c = np.ascontiguousarray((BASE + 0.2 * rng.uniform(-1, 1, (8, 3))) * h + rng.uniform(0, 1, 3))
        u, gp = np.ascontiguousarray(rng.normal(size=(8, 3))), np.ascontiguousarray(rng.normal(size=(8, 3)))
        rho, p, tau = rng.uniform(0.5, 2, 8), rng.normal(size=8), rng.uniform(0.1, 2)
        m1 = oracle.mdot_elem(c, rho, u, p, gp, tau, sm, sp)
        m2 = np.zeros(12)
        elemcheck.hc_mdot_df(P(c), P(rho), P(u), P(p), P(gp), float(tau), sm, sp, P(m2))
        check_dense(m2[None], m1[None], what="mdot df64")


# ---- double-float (df64) element math of the ARITH_DF64 kernels -------------
def _hc_scalar_df(L, c, q, k, sh):
    lhs, rhs = np.zeros(64), np.zeros(8)
    L.hc_scalar_diff_df(P(np.ascontiguousarray(c)), P(q), P(k), int(sh), P(lhs), P(rhs))
    return lhs.reshape(8, 8), rhs


def _hc_cont_df(L, c, u, rho, p, gp, tau, sm, sp, rd):
    lhs, rhs = np.zeros(64), np.zeros(8)
    L.hc_continuity_df(P(np.ascontiguousarray(c)), P(np.ascontiguousarray(u)), P(rho), P(p),
                       P(np.ascontiguousarray(gp)), float(tau), sm, sp, rd, P(lhs), P(rhs))
    return lhs.reshape(8, 8), rhs


def test_golds_through_df64_math(elemcheck, golds):
    c, conn, gid = block_mesh(1, 1, 1)
    e = conn[0]
    lhs, rhs = _hc_scalar_df(elemcheck, c[e], TrigFields.temperature(c)[e], np.ones(8), 0)
    assert np.max(np.abs(lhs.ravel() - golds["scalar_diff"]["lhs"])) <= 1e-15
    for key, opts in [("continuity_default", (0, 0, 0)), ("continuity_reduced_sens", (0, 0, 1)),
                      ("continuity_reduced_shift", (0, 1, 1))]:
        lhs, rhs = _hc_cont_df(elemcheck, c[e], TrigFields.velocity(c)[e], np.ones(8), TrigFields.pressure(c)[e],
                               TrigFields.dpdx(c)[e], 1.0, *opts)
        assert np.max(np.abs(lhs.ravel() - golds[key]["lhs"])) <= 1e-15, key
        assert np.max(np.abs(rhs - golds[key]["rhs"])) <= 1e-15, key


@pytest.mark.parametrize("translate", [0.0, 1.0, 5.0])
def test_df64_random_elements(elemcheck, oracle, translate):
    """Elements of size 1/256..1/16 placed up to `translate` from the origin
    (coordinates much larger than the element: the hardest case for the
    hi+lo split, handled by FP64 differences to node 0)."""
    rng = np.random.default_rng(40 + int(translate))
    for t in range(200):
        h = rng.uniform(1 / 256, 1 / 16)
        c = (BASE + 0.2 * rng.uniform(-1, 1, (8, 3))) * h + rng.uniform(0, translate, 3)
        q, k = rng.uniform(0, 1, 8), rng.uniform(0.5, 2, 8)
        for sh in (0, 1):
            l1, r1 = oracle.scalar_diff_elem(c, q, k, sh)
            l2, r2 = _hc_scalar_df(elemcheck, c, q, k, sh)
            check_dense(l2, l1, what="df64 lhs")
            check_dense(r2[None], r1[None], what="df64 rhs")
        u, gp = rng.normal(size=(8, 3)), rng.normal(size=(8, 3))
        rho, p, tau = rng.uniform(0.5, 2, 8), rng.normal(size=8), rng.uniform(0.1, 2)
        for opts in [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 0, 0)]:
            l1, r1 = oracle.continuity_adv_elem(c, u, rho, p, gp, tau, *opts)
            l2, r2 = _hc_cont_df(elemcheck, c, u, rho, p, gp, tau, *opts)
            check_dense(l2, l1, what="df64 continuity lhs %s" % (opts,))
            check_dense(r2[None], r1[None], what="df64 continuity rhs %s" % (opts,))


@pytest.mark.parametrize("scale", [1e-9, 1e-15, 1e9, 1e15])
def test_df64_scale_invariance(elemcheck, oracle, scale):
    """Coordinates in units from 1e-15 to 1e15 (element sizes 1e-18 .. 1e14):
    the df64 math normalises every element by a power of two, so products of
    three or four lengths (det J, adj(J)^T A) never leave the FP32 exponent
    range.  Same 1e-12 rule as at unit scale, aspect ratios up to 80."""
    rng = np.random.default_rng(50)
    for t in range(120):
        h = rng.uniform(1 / 256, 1 / 16)
        c = (BASE + 0.2 * rng.uniform(-1, 1, (8, 3))) * h
        c[:, 2] *= rng.choice([1.0, 1 / 80.0])  # thin cells of the stretched meshes
        c = (c + h * rng.uniform(0, 2, 3)) * scale  # near the origin: FP64 coordinates resolve thin cells
        q, k = rng.uniform(0, 1, 8), rng.uniform(0.5, 2, 8)
        for sh in (0, 1):
            l1, r1 = oracle.scalar_diff_elem(c, q, k, sh)
            l2, r2 = _hc_scalar_df(elemcheck, c, q, k, sh)
            check_dense(l2, l1, what="df64 lhs x%g" % scale)
            check_dense(r2[None], r1[None], what="df64 rhs x%g" % scale)
        u, gp = rng.normal(size=(8, 3)), rng.normal(size=(8, 3)) / scale
        rho, p, tau = rng.uniform(0.5, 2, 8), rng.normal(size=8), rng.uniform(0.1, 2)
        for opts in [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 0, 0)]:
            l1, r1 = oracle.continuity_adv_elem(c, u, rho, p, gp, tau, *opts)
            l2, r2 = _hc_cont_df(elemcheck, c, u, rho, p, gp, tau, *opts)
            check_dense(l2, l1, what="df64 continuity lhs x%g %s" % (scale, opts))
            check_dense(r2[None], r1[None], what="df64 continuity rhs x%g %s" % (scale, opts))
        cc = np.ascontiguousarray(c)
        for sm, sp in [(0, 0), (1, 1)]:
            m1 = oracle.mdot_elem(cc, rho, u, p, gp, tau, sm, sp)
            m2 = np.zeros(12)
            elemcheck.hc_mdot_df(P(cc), P(rho), P(np.ascontiguousarray(u)), P(p), P(np.ascontiguousarray(gp)),
                                 float(tau), sm, sp, P(m2))
            check_dense(m2[None], m1[None], what="mdot df64 x%g" % scale)


def test_df64_nodal_input_combination(elemcheck):
    """The per-node pass of the df64 continuity kernels: rho u + tau gp formed
    from exact-to-2^-48 FP32-pair splits of the inputs by double-float
    products and a sum, against FP64 on 200 K random values of magnitude
    1e-20..1e20: |hi + lo - w| <= 2^-45 (|rho u| + |tau gp|).  Inputs the pairs
    cannot hold (NaN, inf, |x| >= 2^127) are reported (the device pass raises
    NALU_ERR_NONFINITE for them) and come out non-finite or clamped."""
    rng = np.random.default_rng(12)
    n = 200000
    sc = 10.0 ** rng.uniform(-20, 20, n)
    rho = rng.uniform(0.5, 2.0, n)
    u, gp = rng.normal(size=n) * sc, rng.normal(size=n) * sc
    tau = 0.37
    hi, lo = np.zeros(n, np.float32), np.zeros(n, np.float32)
    assert elemcheck.hc_nodal_w(n, P(rho), P(u), tau, P(gp), P(hi), P(lo)) == 1
    w = hi.astype(np.float64) + lo.astype(np.float64)
    err = np.abs(w - (rho * u + tau * gp)) / (np.abs(rho * u) + np.abs(tau * gp))
    assert err.max() <= 2.0 ** -45, err.max()
    for bad in (float("nan"), float("inf"), 1e300, 2.0 ** 127):
        u2 = u.copy()
        u2[5] = bad
        assert elemcheck.hc_nodal_w(n, P(rho), P(u2), tau, P(gp), P(hi), P(lo)) == 0
    assert elemcheck.hc_nodal_w(1, P(rho), P(np.array([2.0 ** 126])), tau, P(gp), P(hi), P(lo)) == 1
