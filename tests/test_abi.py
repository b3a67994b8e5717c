"""The C-ABI library loads and exports every entry point the header declares
(CPU only: no kernel is launched)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "nalu_gb300", "_lib", "libnalu_gb300.so")


def _declared():
    txt = open(os.path.join(ROOT, "include", "nalu_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(nalu_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def cudalib():
    if not os.path.exists(LIB):
        import __graft_entry__
        __graft_entry__.build()
    return ctypes.CDLL(LIB)


def test_every_declared_symbol_is_exported(cudalib):
    names = _declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(cudalib, n)]
    assert not missing, missing


def test_status_strings_and_defaults(cudalib):
    cudalib.nalu_status_string.restype = ctypes.c_char_p
    assert cudalib.nalu_status_string(0) == b"ok"
    assert cudalib.nalu_status_string(-4).startswith(b"negative")
    import nalu_gb300 as ng
    o = ng.default_assemble_opts()
    assert o.alpha_upw == 1.0 and o.upw_factor == 1.0 and o.proj_time_scale == 1.0
    s = ng.default_solver_opts()
    assert s.tol == 1e-8 and s.method == ng.SOLVER_CG


def test_null_arguments_are_rejected(cudalib):
    import nalu_gb300 as ng
    L = ng.lib()
    assert L.nalu_create(0, None) == -1
    assert L.nalu_destroy(None) == -1
    assert L.nalu_mesh_create(None, 8, 1, None, None, None) == -1
