"""The oracle pinned: against the reference's own compiled master element
(where built here), the reference's unit-test golden vectors, and the Tpetra
2-element graph/matrix test."""
import numpy as np
import pytest

from helpers import TrigFields, block_mesh, check_dense

BASE = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)


def _unit_cube_element():
    c, conn, gid = block_mesh(1, 1, 1)
    return c, conn


def test_oracle_bitwise_equals_reference_master_element(oracle):
    """Restated HexSCS/HexSCV == the reference's Hex8CVFEM.C compiled from its
    sources (oracle/_ref); only where that build exists."""
    import ctypes
    ref = oracle.ref()
    if ref is None:
        pytest.skip("reference master element not built here (oracle/_ref)")
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rng = np.random.default_rng(42)
    for t in range(300):
        c = np.ascontiguousarray((BASE + 0.2 * rng.uniform(-1, 1, (8, 3))) * rng.uniform(0.01, 3) + rng.uniform(-2, 2, 3))
        a1 = oracle.scs_areav(c)
        a2 = np.zeros(36)
        ref.ref_hex_scs_areav(P(c), P(a2))
        assert np.array_equal(a1.ravel(), a2)
        for sh in (0, 1):
            g1, d1, _ = oracle.scs_grad_op(c, sh)
            g2, d2 = np.zeros(288), np.zeros(288)
            ref.ref_hex_scs_grad_op(P(c), sh, P(g2), P(d2))
            assert np.array_equal(g1.ravel(), g2) and np.array_equal(d1.ravel(), d2)
            g1, d1, _ = oracle.scv_grad_op(c, sh)
            g2, d2 = np.zeros(192), np.zeros(192)
            ref.ref_hex_scv_grad_op(P(c), sh, P(g2), P(d2))
            assert np.array_equal(g1.ravel(), g2)
        v2 = np.zeros(8)
        ref.ref_hex_scv_volume(P(c), P(v2))
        assert np.array_equal(oracle.scv_volume(c), v2)
    lr, loc, locs = oracle.scs_tables()
    for sh in (0, 1):
        s2 = np.zeros(96)
        ref.ref_hex_scs_shape_fcn(sh, P(s2))
        assert np.array_equal(oracle.shape_fcn(locs if sh else loc).ravel(), s2)


def test_golds_scalar_diff(oracle, golds):
    c, conn = _unit_cube_element()
    g = golds["scalar_diff"]
    lhs, rhs = oracle.scalar_diff_elem(c[conn[0]], TrigFields.temperature(c)[conn[0]], np.ones(8))
    assert np.max(np.abs(lhs.ravel() - g["lhs"])) <= g["tol"]
    assert np.max(np.abs(rhs - np.array(g["rhs"]))) <= g["tol"]


@pytest.mark.parametrize("key,opts", [("continuity_default", (0, 0, 0)), ("continuity_reduced_sens", (0, 0, 1)),
                                      ("continuity_reduced_shift", (0, 1, 1))])
def test_golds_continuity(oracle, golds, key, opts):
    c, conn = _unit_cube_element()
    e = conn[0]
    g = golds[key]
    lhs, rhs = oracle.continuity_adv_elem(c[e], TrigFields.velocity(c)[e], np.ones(8), TrigFields.pressure(c)[e],
                                          TrigFields.dpdx(c)[e], 1.0, *opts)
    assert np.max(np.abs(lhs.ravel() - g["lhs"])) <= g["tol"]
    assert np.max(np.abs(rhs - g["rhs"])) <= g["tol"]


def test_golds_momentum(oracle, golds):
    c, conn = _unit_cube_element()
    e = conn[0]
    g = golds["momentum_adv_diff"]
    u = TrigFields.velocity(c)[e]
    mdot = oracle.mdot_elem(c[e], np.ones(8), u, np.zeros(8), np.zeros(24))
    lhs, rhs = oracle.momentum_adv_diff_elem(c[e], u, 0.1 * np.ones(8), mdot, 0.0)
    assert np.max(np.abs(lhs.ravel() - g["lhs"])) <= g["tol"]
    assert np.max(np.abs(rhs - g["rhs"])) <= g["tol"]


def test_golds_scv(oracle, golds):
    g = golds["hex8_scv_grad_op"]
    c = np.array(g["coords"]).reshape(8, 3)
    assert np.max(np.abs(oracle.scv_grad_op(c)[0].ravel() - g["gradop"])) <= g["tol"]
    assert np.max(np.abs(oracle.scv_grad_op(c, True)[0].ravel() - g["shifted_gradop"])) <= g["tol"]
    cu, conn = _unit_cube_element()
    assert np.max(np.abs(oracle.scv_volume(cu[conn[0]]) - 0.125)) <= golds["hex8_scv_volume_unit_cube"]["tol"]


def test_tpetra_two_hex_graph_and_matrix(oracle, golds):
    """unit_tests/UnitTestTpetra.C: generated:1x1x2, constant element matrix."""
    g = golds["tpetra_2hex"]
    c, conn, gid = block_mesh(1, 1, 2)
    rp, ci, lid = oracle.graph(c.shape[0], conn, 1, gid)
    assert np.diff(rp).tolist() == g["row_lengths"]
    vals = np.zeros(ci.size)
    rhs = np.zeros(rp.size - 1)
    ev = np.array(g["elem_vals"])
    for e in range(conn.shape[0]):
        oracle.sum_into(1, lid[conn[e]], ev, np.zeros(8), rp, ci, vals, rhs)
    dense = np.zeros((12, 12))
    for i in range(12):
        for k in range(rp[i], rp[i + 1]):
            dense[i, ci[k]] = vals[k]
    assert np.max(np.abs(dense.ravel() - g["lhs_vals"])) <= g["tol"]


def test_graph_dof3_layout(oracle):
    c, conn, gid = block_mesh(2, 1, 1)
    rp1, ci1, _ = oracle.graph(c.shape[0], conn, 1)
    rp3, ci3, _ = oracle.graph(c.shape[0], conn, 3)
    assert rp3.size - 1 == 3 * (rp1.size - 1)
    for a in range(rp1.size - 1):
        nb = ci1[rp1[a]:rp1[a + 1]]
        want = (3 * nb[:, None] + np.arange(3)[None, :]).ravel()
        for d in range(3):
            r = 3 * a + d
            assert np.array_equal(ci3[rp3[r]:rp3[r + 1]], want)


def test_graph_respects_global_ids(oracle):
    """Rows follow ascending global id (beginLinearSystemConstruction)."""
    c, conn, gid = block_mesh(3, 2, 2)
    rng = np.random.default_rng(3)
    perm_gid = rng.permutation(c.shape[0]).astype(np.int64) * 7 + 11
    rp, ci, lid = oracle.graph(c.shape[0], conn, 1, perm_gid)
    order = np.argsort(perm_gid, kind="stable")
    assert np.array_equal(lid[order], np.arange(c.shape[0]))
    for a in range(rp.size - 1):
        row = ci[rp[a]:rp[a + 1]]
        assert np.all(np.diff(row) > 0)


def test_oracle_threaded_matches_serial(oracle):
    c, conn, gid = block_mesh(6, 5, 4, jitter=0.1, seed=5)
    rp, ci, lid = oracle.graph(c.shape[0], conn, 1)
    rng = np.random.default_rng(0)
    q, k = rng.uniform(size=c.shape[0]), rng.uniform(0.5, 2, c.shape[0])
    v1, r1 = oracle.assemble(oracle.KERNEL_SCALAR_DIFF, c, conn, rp, ci, lid, scalar=q, coeff=k)
    v2, r2 = oracle.assemble(oracle.KERNEL_SCALAR_DIFF, c, conn, rp, ci, lid, scalar=q, coeff=k, n_threads=4)
    assert np.allclose(v1, v2, rtol=1e-13, atol=1e-15) and np.allclose(r1, r2, rtol=1e-13, atol=1e-15)


def test_oracle_solvers(oracle):
    c, conn, gid = block_mesh(6, 6, 6, jitter=0.1, seed=2)
    rp, ci, lid = oracle.graph(c.shape[0], conn, 1)
    v, r = oracle.assemble(oracle.KERNEL_SCALAR_DIFF, c, conn, rp, ci, lid, scalar=np.zeros(c.shape[0]),
                           coeff=np.ones(c.shape[0]))
    # Dirichlet on x = 0 and x = 1
    nodes = np.where((c[:, 0] == 0.0) | (c[:, 0] == 1.0))[0]
    b = np.random.default_rng(1).normal(size=rp.size - 1)
    oracle.apply_dirichlet(rp, ci, v, b, nodes, c[nodes, 0], np.zeros(nodes.size))
    x, it, res = oracle.pcg_jacobi(rp, ci, v, b, tol=1e-10)
    assert res <= 1e-10
    x2, it2, res2 = oracle.gmres_jacobi(rp, ci, v, b, restart=30, tol=1e-10)
    assert res2 <= 1e-10 and np.allclose(x, x2, atol=1e-8)


# ---------------------------------------------------------------------------
# dual nodal volume and the element part of the projected nodal gradient
# ---------------------------------------------------------------------------
def _affine_block(n, seed=3):
    """Block mesh under a random linear map of positive determinant (the
    mapping of unit_tests/UnitTestMasterElements.C:185-228)."""
    c, conn, gid = block_mesh(n, n, n)
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    m = q @ np.diag(rng.uniform(0.5, 1.5, 3))
    if np.linalg.det(m) < 0:
        m[:, 0] *= -1.0
    return c @ m.T, conn, np.linalg.det(m)


def _interior(n):
    k, j, i = np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij")
    return ((i > 0) & (i < n) & (j > 0) & (j < n) & (k > 0) & (k < n)).ravel()


def test_dual_volume(oracle):
    n = 4
    c0, conn, _ = block_mesh(n, n, n, jitter=0.3, seed=5)
    v0 = oracle.dual_volume(c0, conn)
    # scatter of HexSCV::determinant per element
    ref = np.zeros(c0.shape[0])
    for e in range(conn.shape[0]):
        np.add.at(ref, conn[e], oracle.scv_volume(c0[conn[e]]))
    assert np.max(np.abs(v0 - ref)) <= 1e-15
    assert abs(v0.sum() - 1.0) <= 1e-13
    # linear map: every volume scales by det(QR)
    ca, conna, det = _affine_block(n)
    cb, _, _ = block_mesh(n, n, n)
    assert np.max(np.abs(oracle.dual_volume(ca, conna) - det * oracle.dual_volume(cb, conna))) <= 1e-15


def _grad_restated(oracle, c, conn, q, vol, shifted):
    """sum over the 12 SCS of q_ip A into the left (+) and right (-) node of each
    face, divided by the dual volume (AssembleNodalGradElemAlgorithm.C:104-137;
    shifted_shape_fcn at :197-201)."""
    lr, loc, locs = oracle.scs_tables()
    lr = lr.reshape(12, 2)
    shp = oracle.shape_fcn((locs if shifted else loc).reshape(12, 3))
    q2 = q.reshape(q.shape[0], -1)
    g = np.zeros((c.shape[0], q2.shape[1], 3))
    for e in range(conn.shape[0]):
        a = oracle.scs_areav(c[conn[e]])
        qip = shp @ q2[conn[e]]
        for ip in range(12):
            f = qip[ip][:, None] * a[ip][None, :]
            g[conn[e][lr[ip, 0]]] += f
            g[conn[e][lr[ip, 1]]] -= f
    g /= vol[:, None, None]
    return g[:, 0, :] if q.ndim == 1 else g


@pytest.mark.parametrize("shifted", [False, True])
def test_nodal_grad_elem_restated(oracle, shifted):
    c, conn, _ = block_mesh(3, 3, 3, jitter=0.3, seed=2)
    rng = np.random.default_rng(1)
    vol = oracle.dual_volume(c, conn)
    for q in (rng.standard_normal(c.shape[0]), rng.standard_normal((c.shape[0], 3))):
        got = oracle.nodal_grad_elem(c, conn, q, vol, shifted)
        ref = _grad_restated(oracle, c, conn, q, vol, shifted)
        assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))


def test_nodal_grad_elem_exact_for_linear_fields(oracle):
    """Green-Gauss over a closed dual volume is exact for a linear field on an
    affine mesh at interior nodes (boundary nodes lack the face closure)."""
    n = 4
    c, conn, _ = _affine_block(n)
    vol = oracle.dual_volume(c, conn)
    inner = _interior(n)
    g = np.array([0.7, -1.3, 2.1])
    got = oracle.nodal_grad_elem(c, conn, 0.4 + c @ g, vol)
    assert np.max(np.abs(got[inner] - g)) <= 1e-12
    m = np.array([[1.0, 2.0, -0.5], [0.3, -1.1, 0.8], [2.2, 0.1, -0.7]])
    got = oracle.nodal_grad_elem(c, conn, c @ m.T, vol)
    assert np.max(np.abs(got[inner] - m[None])) <= 1e-12


# ---------------------------------------------------------------------------
# time terms (ContinuityMassElemKernel, MomentumMassElemKernel)
# ---------------------------------------------------------------------------
def mass_gold_inputs(c, conn):
    """the kernel-test fixtures: state N+1 filled, states N and N-1 zero"""
    e = conn[0]
    z, one, z3 = np.zeros(8), np.ones(8), np.zeros((8, 3))
    return dict(coords=c[e], rho=(z, z, one), u=(z3, z3, TrigFields.velocity(c)[e]), gpdx=TrigFields.dpdx(c)[e])


@pytest.mark.parametrize("key", ["continuity_mass", "continuity_mass_lumped", "momentum_mass",
                                 "momentum_mass_lumped"])
def test_golds_mass(oracle, golds, key):
    g = golds[key]
    c, conn = _unit_cube_element()
    f = mass_gold_inputs(c, conn)
    t = (g["dt"], g["gamma1"], g["gamma2"], g["gamma3"])
    if key.startswith("continuity"):
        lhs, rhs = oracle.continuity_mass_elem(f["coords"], *f["rho"], *t, lumped=g["lumped"])
    else:
        lhs, rhs = oracle.momentum_mass_elem(f["coords"], *f["rho"], *f["u"], f["gpdx"], *t, lumped=g["lumped"])
    assert np.max(np.abs(rhs - g["rhs"])) <= g["tol"], key
    assert np.max(np.abs(lhs.ravel() - g["lhs"])) <= g["tol"], key


def test_mass_assembly_matches_element_sum(oracle):
    """orc_assemble_mass = per-element kernel + restated sumInto, BDF2 states"""
    c, conn, gid = block_mesh(3, 2, 2, jitter=0.2, seed=6)
    n = c.shape[0]
    rng = np.random.default_rng(2)
    rho = [1.0 + 0.1 * rng.random(n) for _ in range(3)]
    u = [rng.standard_normal((n, 3)) for _ in range(3)]
    gp = rng.standard_normal((n, 3))
    t = dict(dt=0.05, gamma1=1.5, gamma2=-2.0, gamma3=0.5)
    for mom, nd in ((False, 1), (True, 3)):
        rp, ci, lid = oracle.graph(n, conn, nd, gid)
        for lumped in (False, True):
            v, r = oracle.assemble_mass(mom, c, conn, rp, ci, lid, *rho, *(u if mom else (None,) * 3),
                                        gpdx=gp if mom else None, lumped=lumped, balanced_force=mom, **t)
            v2, r2 = np.zeros_like(v), np.zeros_like(r)
            for e in range(conn.shape[0]):
                en = conn[e]
                if mom:
                    lhs, rhs = oracle.momentum_mass_elem(c[en], *[x[en] for x in rho], *[x[en] for x in u], gp[en],
                                                         t["dt"], t["gamma1"], t["gamma2"], t["gamma3"], lumped, True)
                else:
                    lhs, rhs = oracle.continuity_mass_elem(c[en], *[x[en] for x in rho], t["dt"], t["gamma1"],
                                                           t["gamma2"], t["gamma3"], lumped)
                oracle.sum_into(nd, lid[en], lhs, rhs, rp, ci, v2, r2)
            assert np.array_equal(v, v2) and np.array_equal(r, r2)


# ---------------------------------------------------------------------------
# boundary faces
# ---------------------------------------------------------------------------
def test_face_tables_and_grad_op_equal_reference(oracle):
    """side node ordinals, the face ip -> node map, and face_grad_op
    (standard and shifted) bit for bit against the compiled reference"""
    import ctypes
    ref = oracle.ref()
    if ref is None:
        pytest.skip("reference master element not built here (oracle/_ref)")
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    for s in range(6):
        t = np.zeros(8, np.int32)
        ref.ref_hex_side_nodes(s, P(t))
        assert np.array_equal(t[:4], oracle.side_nodes(s)) and np.array_equal(t[4:], oracle.side_nodes(s))
    rng = np.random.default_rng(7)
    for _ in range(100):
        c = np.ascontiguousarray((BASE + 0.2 * rng.uniform(-1, 1, (8, 3))) * rng.uniform(0.01, 3) + rng.uniform(-2, 2, 3))
        for s in range(6):
            for sh in (0, 1):
                g2 = np.zeros(96)
                ref.ref_hex_face_grad_op(s, sh, P(c), P(g2))
                assert np.array_equal(oracle.face_grad_op(s, c, sh)[0].ravel(), g2)


def test_quad_areas(oracle):
    rng = np.random.default_rng(3)
    c, conn = _unit_cube_element()
    e = conn[0]
    outward = {0: [0, -1, 0], 1: [1, 0, 0], 2: [0, 1, 0], 3: [-1, 0, 0], 4: [0, 0, -1], 5: [0, 0, 1]}
    for s in range(6):
        a = oracle.quad_areav(c[e][oracle.side_nodes(s)])
        assert np.allclose(a, 0.25 * np.array(outward[s])[None, :], atol=1e-16)
    for _ in range(50):
        p = rng.standard_normal((4, 3))
        a = oracle.quad_areav(p)
        # the four sub-faces tile the bilinear surface: sum = (p2 - p0) x (p3 - p1) / 2
        assert np.allclose(a.sum(0), 0.5 * np.cross(p[2] - p[0], p[3] - p[1]), atol=1e-14)
    # an element's six exposed faces close: their areas sum to zero
    cj, connj, _ = block_mesh(1, 1, 1, jitter=0.0)
    x = cj[connj[0]] + 0.15 * rng.uniform(-1, 1, (8, 3))
    tot = sum(oracle.quad_areav(x[oracle.side_nodes(s)]).sum(0) for s in range(6))
    assert np.max(np.abs(tot)) <= 1e-15


def test_skin(oracle):
    nx, ny, nz = 4, 3, 2
    c, conn, _ = block_mesh(nx, ny, nz, jitter=0.2, seed=1)
    fe, fs = oracle.skin(conn)
    assert fe.shape[0] == 2 * (nx * ny + ny * nz + nz * nx)
    lo, hi = c.min(0), c.max(0)
    for e, s in zip(fe, fs):
        x = c[conn[e][oracle.side_nodes(s)]]
        assert np.any(np.all(np.isclose(x, lo[None, :]), axis=0) | np.all(np.isclose(x, hi[None, :]), axis=0))


def test_nodal_gradient_with_closure_exact_everywhere(oracle):
    """element part + boundary closure: Green-Gauss over every closed dual
    volume, exact for a linear field on an affine mesh at all nodes"""
    n = 3
    c, conn, det = _affine_block(n)
    vol = oracle.dual_volume(c, conn)
    fe, fs = oracle.skin(conn)
    g = np.array([0.7, -1.3, 2.1])
    grad = oracle.nodal_grad_elem(c, conn, 0.4 + c @ g, vol)
    oracle.nodal_grad_boundary(c, conn, fe, fs, 0.4 + c @ g, vol, grad)
    assert np.max(np.abs(grad - g)) <= 1e-12
    m = np.array([[1.0, 2.0, -0.5], [0.3, -1.1, 0.8], [2.2, 0.1, -0.7]])
    grad = oracle.nodal_grad_elem(c, conn, c @ m.T, vol)
    oracle.nodal_grad_boundary(c, conn, fe, fs, c @ m.T, vol, grad)
    assert np.max(np.abs(grad - m[None])) <= 1e-12


def test_continuity_face_kernels(oracle):
    """inflow: sum of rhs = -rho U . (total face area) / tau; open with p = pbc
    and the exact gradient on an affine mesh: mdot = rho u . A exactly, so the
    open rhs equals the inflow rhs of the same velocity"""
    n = 3
    c, conn, _ = _affine_block(n, seed=9)
    fe, fs = oracle.skin(conn)
    U = np.array([0.3, -0.2, 0.5])
    rho = np.full(c.shape[0], 1.2)
    u = np.tile(U, (c.shape[0], 1))
    gvec = np.array([0.4, 0.1, -0.3])
    p = 1.0 + c @ gvec
    gp = np.tile(gvec, (c.shape[0], 1))
    tau = 0.25
    for e, s in zip(fe[:12], fs[:12]):
        x = c[conn[e]]
        _, r_in = oracle.continuity_inflow_face(s, x, rho[conn[e]], u[conn[e]], tau)
        a = oracle.quad_areav(x[oracle.side_nodes(s)])
        assert abs(r_in.sum() + 1.2 * U @ a.sum(0) / tau) <= 1e-14
        lhs, r_op = oracle.continuity_open_face(s, x, p[conn[e]], p[conn[e]], rho[conn[e]], u[conn[e]], gp[conn[e]],
                                                proj_time_scale=tau)
        assert np.max(np.abs(r_op - r_in)) <= 1e-13
        # rows off the face stay empty; each face row: penalty part sums to 2 invL |A|, gradient part to 0
        off = [k for k in range(8) if k not in oracle.side_nodes(s)]
        assert np.all(lhs[off] == 0.0) and np.all(r_op[off] == 0.0)


def test_oracle_gmres_restart_cycles(oracle):
    """The oracle's Jacobi-GMRES(10) on the 16^3 heat system (jitter 0.1, Dirichlet
    T = 0 / 1 on x = 0 / 1) converges over many restart cycles in 61 iterations,
    and its solution agrees with a direct solve. The GPU GMRES test compares its
    iteration count with this figure."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    c, conn, gid = block_mesh(16, jitter=0.1, seed=21)
    n = c.shape[0]
    T = np.random.default_rng(22).uniform(0, 1, n)
    rp, ci, lid = oracle.graph(n, conn, 1, gid)
    v, b = oracle.assemble(oracle.KERNEL_SCALAR_DIFF, c, conn, rp, ci, lid, scalar=T, coeff=np.ones(n))
    left, right = np.where(c[:, 0] == 0.0)[0], np.where(c[:, 0] == 1.0)[0]
    nodes = np.concatenate([left, right])
    bc = np.concatenate([np.zeros(left.size), np.ones(right.size)])
    rows = np.asarray(lid[nodes] if lid is not None else nodes, np.int64)
    oracle.apply_dirichlet(rp, ci, v, b, rows, bc, T[nodes])
    x, it, res = oracle.gmres_jacobi(rp, ci, v, b, restart=10, tol=1e-8, max_it=5000)
    assert res <= 1e-8 and it == 61, (it, res)
    xd = sla.spsolve(sp.csr_matrix((v, ci, rp), shape=(n, n)).tocsc(), b)
    assert np.max(np.abs(x - xd)) <= 1e-5 * np.max(np.abs(xd))
