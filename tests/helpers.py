"""Test helpers: tolerance checks, meshes and fields for the parity tests."""
import numpy as np

from nalu_gb300.meshgen import TrigFields, block_mesh, fourier_velocity

REL = 1e-12     # relative tolerance for FP64 assembled values
FLOOR = 1e-12   # absolute floor, in units of the row's largest |entry|


def csr_row_max(rowptr, values):
    n = rowptr.size - 1
    lens = np.diff(rowptr)
    rowid = np.repeat(np.arange(n), lens)
    rm = np.zeros(n)
    np.maximum.at(rm, rowid, np.abs(values))
    return rm, rowid


def check_csr_values(actual, expected, rowptr, rel=REL, floor=FLOOR, what="values"):
    rm, rowid = csr_row_max(rowptr, expected)
    allowed = rel * np.maximum(np.abs(actual), np.abs(expected)) + floor * rm[rowid]
    bad = np.abs(actual - expected) > allowed
    if bad.any():
        i = int(np.argmax(np.abs(actual - expected) - allowed))
        raise AssertionError("%s: %d/%d entries outside tol; worst idx %d row %d: %.17g vs %.17g (rowmax %.3g)" % (
            what, int(bad.sum()), bad.size, i, rowid[i], actual[i], expected[i], rm[rowid[i]]))


def check_vec(actual, expected, scale=None, rel=REL, floor=FLOOR, what="rhs"):
    scale = np.max(np.abs(expected)) if scale is None else scale
    allowed = rel * np.maximum(np.abs(actual), np.abs(expected)) + floor * scale
    bad = np.abs(actual - expected) > allowed
    if bad.any():
        i = int(np.argmax(np.abs(actual - expected) - allowed))
        raise AssertionError("%s: %d/%d outside tol; worst %d: %.17g vs %.17g" % (
            what, int(bad.sum()), bad.size, i, actual[i], expected[i]))


def check_dense(actual, expected, rel=REL, floor=FLOOR, what="lhs"):
    a = np.asarray(actual)
    b = np.asarray(expected)
    rm = np.max(np.abs(b), axis=-1, keepdims=True)
    allowed = rel * np.maximum(np.abs(a), np.abs(b)) + floor * rm
    bad = np.abs(a - b) > allowed
    if bad.any():
        idx = np.unravel_index(int(np.argmax(np.abs(a - b) - allowed)), a.shape)
        raise AssertionError("%s: %d entries outside tol; worst %s: %.17g vs %.17g" % (
            what, int(bad.sum()), idx, a[idx], b[idx]))


def continuity_fields(coords, seed=0, with_pressure=True):
    u = fourier_velocity(coords, n_modes=16, seed=seed)
    rng = np.random.default_rng(seed + 1)
    rho = rng.uniform(0.8, 1.2, coords.shape[0])
    p = rng.normal(size=coords.shape[0]) if with_pressure else np.zeros(coords.shape[0])
    gp = rng.normal(size=coords.shape) if with_pressure else np.zeros_like(coords)
    return u, rho, p, gp


__all__ = ["REL", "FLOOR", "check_csr_values", "check_vec", "check_dense", "continuity_fields", "block_mesh",
           "fourier_velocity", "TrigFields"]
