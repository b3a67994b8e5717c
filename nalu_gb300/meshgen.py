"""Synthetic Hex8 block meshes and nodal fields.

The numbering follows STK's ``generated:NXxNYxNZ`` meshes, which the
reference's tests document as "elem 1 nodes: 1 2 4 3 5 6 8 7"
(unit_tests/UnitTestTpetra.C:101-102):

* node (i, j, k) has index ``i + (nx+1)*(j + (ny+1)*k)`` and global id index+1;
* element (i, j, k) has index ``i + nx*(j + ny*k)`` and nodes
  (i,j,k), (i+1,j,k), (i+1,j+1,k), (i,j+1,k), then the same four at k+1.

Random numbers come from numpy's PCG64 (``numpy.random.default_rng(seed)``),
which gives the same stream on every platform.
"""
import numpy as np


def block_mesh(nx, ny=None, nz=None, lengths=(1.0, 1.0, 1.0), jitter=0.0, seed=0,
               z_ratio=None):
    """Hex8 block mesh on [0,Lx]x[0,Ly]x[0,Lz].

    jitter  -- interior nodes move by U(-jitter, +jitter) * local spacing per axis
    z_ratio -- geometric spacing ratio in z (wall-normal stretching), normalised
               so that the z extent stays Lz
    Returns (coords float64 [n,3], conn int32 [E,8], gid int64 [n]).
    """
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    lx, ly, lz = lengths
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    if z_ratio is None or z_ratio == 1.0:
        zs = np.linspace(0.0, lz, nz + 1)
    else:
        dz = z_ratio ** np.arange(nz, dtype=np.float64)
        zs = np.concatenate([[0.0], np.cumsum(dz)])
        zs = zs / zs[-1] * lz
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
        interior = ((i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)).ravel()
        hx = np.full(coords.shape[0], lx / nx)
        hy = np.full(coords.shape[0], ly / ny)
        dzs = np.diff(zs)
        kk = k.ravel()
        hz = np.minimum(dzs[np.clip(kk - 1, 0, nz - 1)], dzs[np.clip(kk, 0, nz - 1)])
        h = np.stack([hx, hy, hz], axis=1)
        d = rng.uniform(-jitter, jitter, size=coords.shape) * h
        coords[interior] += d[interior]
    ek, ej, ei = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ei, ej, ek = ei.ravel(), ej.ravel(), ek.ravel()

    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    conn = np.stack([nid(ei, ej, ek), nid(ei + 1, ej, ek), nid(ei + 1, ej + 1, ek), nid(ei, ej + 1, ek),
                     nid(ei, ej, ek + 1), nid(ei + 1, ej, ek + 1), nid(ei + 1, ej + 1, ek + 1),
                     nid(ei, ej + 1, ek + 1)], axis=1).astype(np.int32)
    gid = np.arange(1, coords.shape[0] + 1, dtype=np.int64)
    return np.ascontiguousarray(coords), np.ascontiguousarray(conn), gid


def fourier_velocity(coords, n_modes=64, kmin=1, kmax=16, seed=0, amp=1.0):
    """Divergence-free sum of random Fourier modes.

    u(x) = sum_m a_m s_m sin(2 pi k_m . x + phi_m), integer wave vectors with
    |k_m| in [kmin, kmax], s_m a unit vector normal to k_m, |a_m| ~ |k_m|^(-5/3).
    """
    rng = np.random.default_rng(seed)
    ks, ss, amps, phis = [], [], [], []
    while len(ks) < n_modes:
        k = rng.integers(-kmax, kmax + 1, size=3)
        kn = np.linalg.norm(k)
        if kn < kmin or kn > kmax:
            continue
        r = rng.normal(size=3)
        s = np.cross(k, r)
        s /= np.linalg.norm(s)
        ks.append(k.astype(np.float64))
        ss.append(s)
        amps.append(amp * kn ** (-5.0 / 3.0))
        phis.append(rng.uniform(0, 2 * np.pi))
    u = np.zeros_like(coords)
    two_pi = 2.0 * np.pi
    for k, s, a, ph in zip(ks, ss, amps, phis):
        arg = two_pi * (coords @ k) + ph
        u += np.outer(a * np.sin(arg), s)
    return np.ascontiguousarray(u)


class TrigFields:
    """Trigonometric test fields of the reference's kernel unit tests
    (TrigFieldFunction, unit_tests/kernels/UnitTestKernelUtils.C:23-275:
    unot = vnot = pnot = 1, a = 0.3, k = 1, aT = 1)."""

    a = 0.3
    aT = 1.0
    k = 1.0

    @staticmethod
    def velocity(c):
        a, pi = TrigFields.a, np.pi
        x, y = c[:, 0], c[:, 1]
        u = np.zeros_like(c)
        u[:, 0] = -1.0 * np.cos(a * pi * x) * np.sin(a * pi * y)
        u[:, 1] = +1.0 * np.sin(a * pi * x) * np.cos(a * pi * y)
        return u

    @staticmethod
    def pressure(c):
        a, pi = TrigFields.a, np.pi
        x, y = c[:, 0], c[:, 1]
        return -1.0 / 4.0 * (np.cos(2.0 * a * pi * x) + np.cos(2.0 * a * pi * y))

    @staticmethod
    def dpdx(c):
        a, pi = TrigFields.a, np.pi
        x, y = c[:, 0], c[:, 1]
        g = np.zeros_like(c)
        g[:, 0] = 0.5 * a * pi * np.sin(2.0 * a * pi * x)
        g[:, 1] = 0.5 * a * pi * np.sin(2.0 * a * pi * y)
        return g

    @staticmethod
    def temperature(c):
        aT, k, pi = TrigFields.aT, TrigFields.k, np.pi
        x, y, z = c[:, 0], c[:, 1], c[:, 2]
        return (k / 4.0) * (np.cos(2.0 * aT * pi * x) + np.cos(2.0 * aT * pi * y) + np.cos(2.0 * aT * pi * z))


def batch_block_meshes(n_problems, edge_range=(16, 96), jitter=0.1, seed=0):
    """Union of independent Hex8 block meshes on the unit cube.

    Each problem draws its three edge counts log-uniformly from edge_range
    (rounded to integers) and its own interior jitter.  Problem k's nodes
    follow problem k-1's, with global ids continuing across problems, so
    every problem owns one contiguous range of rows.
    Returns (coords, conn, gid, node_offsets int64 [P+1], edges int [P,3]).
    """
    rng = np.random.default_rng(seed)
    lo, hi = np.log(edge_range[0]), np.log(edge_range[1])
    edges = np.rint(np.exp(rng.uniform(lo, hi, size=(n_problems, 3)))).astype(np.int64)
    coords, conns, offs = [], [], [0]
    for k in range(n_problems):
        nx, ny, nz = (int(e) for e in edges[k])
        c, conn, _ = block_mesh(nx, ny, nz, jitter=jitter, seed=seed * 7919 + 1 + k)
        coords.append(c)
        conns.append(conn + offs[-1])
        offs.append(offs[-1] + c.shape[0])
    coords = np.ascontiguousarray(np.concatenate(coords))
    conn = np.ascontiguousarray(np.concatenate(conns).astype(np.int32))
    gid = np.arange(1, coords.shape[0] + 1, dtype=np.int64)
    return coords, conn, gid, np.asarray(offs, dtype=np.int64), edges
