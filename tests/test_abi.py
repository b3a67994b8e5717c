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


def test_master_element_tables(cudalib, oracle):
    """HexSCS::adjacentNodes, shape_fcn / shifted_shape_fcn and the side node
    ordinals from the library's host tables equal the oracle's (pinned to the
    compiled reference)"""
    import ctypes
    import numpy as np
    P = lambda a: ctypes.c_void_p(a.ctypes.data)
    lr = np.zeros(24, np.int32)
    cudalib.nalu_hex_scs_adjacent_nodes(P(lr))
    olr, loc, locs = oracle.scs_tables()
    assert np.array_equal(lr, olr)
    for sh, iso in ((0, loc), (1, locs)):
        shp = np.zeros(96)
        cudalib.nalu_hex_scs_shape_fcn(sh, P(shp))
        assert np.array_equal(shp.reshape(12, 8), oracle.shape_fcn(iso.reshape(12, 3)))
    for s in range(6):
        nd = np.zeros(4, np.int32)
        cudalib.nalu_hex_side_node_ordinals(s, P(nd))
        assert np.array_equal(nd, oracle.side_nodes(s))
    # interpolation at the ips reproduces a linear field on a distorted element
    # (unit_tests/UnitTestMasterElements.C:64-102)
    rng = np.random.default_rng(0)
    x = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    x = x + 0.2 * rng.uniform(-1, 1, (8, 3))
    a, b = rng.standard_normal(3), rng.standard_normal()
    for sh in (0, 1):
        shp = np.zeros(96)
        cudalib.nalu_hex_scs_shape_fcn(sh, P(shp))
        shp = shp.reshape(12, 8)
        assert np.allclose(shp @ (x @ a + b), (shp @ x) @ a + b, atol=1e-14)
        assert np.allclose(shp.sum(axis=1), 1.0, atol=1e-15)


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of the option and info structs have the size and
    field offsets that a C compiler gives the header's structs."""
    import shutil
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    import nalu_gb300 as ng
    structs = {"nalu_assemble_opts": ng.AssembleOpts, "nalu_solver_opts": ng.SolverOpts,
               "nalu_solve_info": ng.SolveInfo, "nalu_train_opts": ng.TrainOpts}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "nalu_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for field in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, field[0], cname, field[0]))
    lines += ["return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for field in py._fields_:
            assert int(got["%s.%s" % (cname, field[0])]) == getattr(py, field[0]).offset, (cname, field[0])


@pytest.mark.parametrize("example", ["heat_conduction", "continuity_step"])
def test_cpp_host_interface_compiles(example):
    """The C++ mirror (include/nalu_gb300.hpp) and the C++ callers that drive
    it compile cleanly against the header alone (no CUDA needed)."""
    import shutil
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = os.path.join(ROOT, "nalu_gb300", "examples", example + ".cpp")
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", src], check=True)
