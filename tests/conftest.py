"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on
CPU.  The oracle and the host build of the element math are built on demand
(g++ only); the CUDA library is built by __graft_entry__.build()."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def oracle():
    so = os.path.join(ROOT, "oracle", "liboracle.so")
    src = os.path.join(ROOT, "oracle", "nalu_oracle.cpp")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True,
                       capture_output=True)
    from oracle import oracle as O
    return O


@pytest.fixture(scope="session")
def golds():
    with open(os.path.join(ROOT, "tests", "golden", "nalu_unit_golds.json")) as f:
        return json.load(f)["golds"]


@pytest.fixture(scope="session")
def elemcheck():
    """Host build of nalu_gb300/csrc/hex8_elem.h (the device element math)."""
    import ctypes
    out = os.path.join(ROOT, "nalu_gb300", "_lib", "libnalu_elemcheck.so")
    src = os.path.join(ROOT, "nalu_gb300", "csrc", "elem_hostcheck.cpp")
    hdrs = [os.path.join(ROOT, "nalu_gb300", "csrc", h) for h in ("hex8_elem.h", "hex8_elem_df.h", "df64.h")]
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(f) for f in [src] + hdrs):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-shared", "-o", out, src],
                       check=True)
    L = ctypes.CDLL(out)
    P = ctypes.c_void_p
    L.hc_scalar_diff.argtypes = [P, P, P, ctypes.c_int, P, P]
    L.hc_continuity.argtypes = [P] * 5 + [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
    L.hc_scalar_diff_df.argtypes = [P, P, P, ctypes.c_int, P, P]
    L.hc_continuity_df.argtypes = [P] * 5 + [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
    L.hc_mdot.argtypes = [P] * 5 + [ctypes.c_double, ctypes.c_int, ctypes.c_int, P]
    L.hc_mdot_df.argtypes = [P] * 5 + [ctypes.c_double, ctypes.c_int, ctypes.c_int, P]
    L.hc_nodal_w.argtypes = [ctypes.c_int64, P, P, ctypes.c_double, P, P, P]
    L.hc_nodal_w.restype = ctypes.c_int
    return L


@pytest.fixture(scope="session")
def gpu_ctx_factory():
    import nalu_gb300 as ng
    ng.lib()  # raises if the CUDA library is missing

    def make():
        return ng.Context(0)
    return make


def assert_close_tol(actual, expected, rel=1e-12, floor=1e-12, row_axis=-1, what=""):
    """|a-b| <= rel*max(|a|,|b|) + floor*(row max |b|): the parity tolerance
    for FP64 values summed in a different order than the reference."""
    import numpy as np
    a = np.asarray(actual, dtype=np.float64)
    b = np.asarray(expected, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    rowmax = np.max(np.abs(b), axis=row_axis, keepdims=True) if b.ndim > 1 else np.max(np.abs(b))
    allowed = rel * np.maximum(np.abs(a), np.abs(b)) + floor * rowmax
    bad = np.abs(a - b) > allowed
    if bad.any():
        idx = np.argwhere(bad)[:5]
        raise AssertionError("%s: %d entries outside tolerance, e.g. %s: %s vs %s" % (
            what, int(bad.sum()), idx.tolist(), a[tuple(idx[0])], b[tuple(idx[0])]))
