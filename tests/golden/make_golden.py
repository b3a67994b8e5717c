"""Extract the reference's unit-test golden vectors into JSON fixtures.

Run once where the NaluCFD/Nalu source tree is available:

    python tests/golden/make_golden.py <reference checkout>

It reads the test sources as text (no reference code is executed) and writes
``tests/golden/nalu_unit_golds.json``.  The fixture records, per gold, the
reference file and line the numbers come from, the tolerance the reference
test uses, and the inputs needed to recompute it (mesh, fields, options).
"""
import json
import os
import re
import sys


def _strip_comments(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def _find_array(src, name, start=0):
    """Return (values, line) of the first `name[...] = { ... };` after start."""
    m = re.compile(r"\b" + re.escape(name) + r"\s*(\[[^\]]*\])+\s*=\s*\{").search(src, start)
    if not m:
        raise KeyError(name)
    depth, i = 0, m.end() - 1
    while True:
        c = src[i]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                break
        i += 1
    body = _strip_comments(src[m.end() - 1:i + 1])
    # expressions like 2.0*2 in the Tpetra table
    exprs = re.findall(r"[-+]?[\d.]+(?:\s*\*\s*[\d.]+)?", body)
    vals = [eval(e.replace(" ", "")) for e in exprs]
    line = src.count("\n", 0, m.start()) + 1
    return vals, line


def _namespace_start(src, ns):
    m = re.search(r"namespace\s+" + re.escape(ns) + r"\s*\{", src)
    if not m:
        raise KeyError(ns)
    return m.end()


def main(ref):
    ut = os.path.join(ref, "unit_tests")
    out = {"source": "NaluCFD/Nalu unit tests (text extraction)", "golds": {}}

    def grab(relpath, name, ns=None):
        src = open(os.path.join(ut, relpath)).read()
        start = _namespace_start(src, ns) if ns else 0
        vals, line = _find_array(src, name, start)
        return vals, "unit_tests/%s:%d" % (relpath, line)

    g = out["golds"]
    lhs, at = grab("kernels/UnitTestScalarDiffElem.C", "lhs", "cvfem_diff")
    g["scalar_diff"] = {"lhs": lhs, "rhs": [0.0] * 8, "at": at, "tol": 1.0e-15,
                        "mesh": "unit_cube", "fields": "temperature=trig(aT=1,k=1), k=1"}
    rhs, at_r = grab("kernels/UnitTestContinuityAdvElem.C", "rhs", "advection_default")
    lhs, at_l = grab("kernels/UnitTestContinuityAdvElem.C", "lhs", "advection_default")
    g["continuity_default"] = {"lhs": lhs, "rhs": rhs, "at": [at_r, at_l], "tol": 1.0e-15,
                               "opts": {"shift_mdot": 0, "shift_poisson": 0, "reduced_sens": 0,
                                        "proj_time_scale": 1.0}}
    rhs, at_r = grab("kernels/UnitTestContinuityAdvElem.C", "rhs", "advection_reduced_sensitivities")
    lhs, at_l = grab("kernels/UnitTestContinuityAdvElem.C", "lhs", "advection_reduced_sensitivities")
    g["continuity_reduced_sens"] = {"lhs": lhs, "rhs": rhs, "at": [at_r, at_l], "tol": 1.0e-15,
                                    "opts": {"shift_mdot": 0, "shift_poisson": 0, "reduced_sens": 1,
                                             "proj_time_scale": 1.0}}
    g["continuity_reduced_shift"] = dict(g["continuity_reduced_sens"])
    g["continuity_reduced_shift"]["opts"] = {"shift_mdot": 0, "shift_poisson": 1, "reduced_sens": 1,
                                             "proj_time_scale": 1.0}
    rhs, at_r = grab("kernels/UnitTestMomentumAdvDiffElem.C", "rhs", "advection_diffusion")
    lhs, at_l = grab("kernels/UnitTestMomentumAdvDiffElem.C", "lhs", "advection_diffusion")
    assert len(rhs) == 24 and len(lhs) == 576, (len(rhs), len(lhs))
    g["momentum_adv_diff"] = {"lhs": lhs, "rhs": rhs, "at": [at_r, at_l], "tol": 1.0e-15,
                              "opts": {"include_divu": 0.0, "viscosity": 0.1}}
    ev, at_e = grab("UnitTestTpetra.C", "elemVals")
    lv, at_l = grab("UnitTestTpetra.C", "lhsVals")
    src = open(os.path.join(ut, "UnitTestTpetra.C")).read()
    m = re.search(r"goldRowLengths\s*=\s*\{([^}]*)\}", src)
    rl = [int(x) for x in m.group(1).split(",")]
    g["tpetra_2hex"] = {"elem_vals": ev, "lhs_vals": lv, "row_lengths": rl, "tol": 1.0e-9,
                        "at": [at_e, at_l, "unit_tests/UnitTestTpetra.C:%d" % (src.count("\n", 0, m.start()) + 1)],
                        "mesh": "generated:1x1x2"}
    gs, at_g = grab("UnitTestKokkosMEGold.h", "hex8_scv_grad_op")
    gss, at_s = grab("UnitTestKokkosMEGold.h", "hex8_scv_shifted_grad_op")
    usrc = open(os.path.join(ut, "UnitTestUtils.C")).read()
    k = usrc.index("case stk::topology::HEXAHEDRON_8:", usrc.index("create_one_perturbed_element(stk::mesh::BulkData"))
    blk = usrc[k:usrc.index("break;", k)]
    coords = [float(x) for x in re.findall(r"[-+]?\d*\.\d+", blk)]
    assert len(coords) == 24
    g["hex8_scv_grad_op"] = {"gradop": gs, "shifted_gradop": gss, "coords": coords, "tol": 1.0e-10,
                             "at": [at_g, at_s, "unit_tests/UnitTestUtils.C:%d" % (usrc.count("\n", 0, k) + 1)]}
    g["hex8_scv_volume_unit_cube"] = {"volume": [0.125] * 8, "tol": 2.220446049250313e-16,
                                      "at": "unit_tests/UnitTestHexSCVDeterminant.C:60-75"}
    # time terms: BDF1 with dt 0.1 (gamma 1, -1, 0); the fixtures fill state
    # N+1 only (density 1, trig velocity / dpdx), state N stays 0
    time = {"dt": 0.1, "gamma1": 1.0, "gamma2": -1.0, "gamma3": 0.0,
            "fields": "density np1 = 1, n = nm1 = 0; velocity np1 = trig, n = nm1 = 0; dpdx = trig"}
    csrc = open(os.path.join(ut, "kernels/UnitTestContinuityMassElem.C")).read()
    for key, test in [("continuity_mass", "density_time_derivative)"),
                      ("continuity_mass_lumped", "density_time_derivative_lumped)")]:
        k = csrc.index(test)
        m = re.compile(r"expect_all_near\(helperObjs\.linsys->rhs_,\s*([-+\d.eE]+)\)").search(csrc, k)
        at = "unit_tests/kernels/UnitTestContinuityMassElem.C:%d" % (csrc.count("\n", 0, m.start()) + 1)
        g[key] = dict(time, rhs=[float(m.group(1))] * 8, lhs=[0.0] * 64, at=at, tol=1.0e-15,
                      lumped=key.endswith("lumped"))
    rhs, at_r = grab("kernels/UnitTestMomentumMassElem.C", "rhs", "momentum_time_derivative")
    lhs, at_l = grab("kernels/UnitTestMomentumMassElem.C", "lhs", "momentum_time_derivative")
    assert len(rhs) == 24 and len(lhs) == 576
    g["momentum_mass"] = dict(time, rhs=rhs, lhs=lhs, at=[at_r, at_l], tol=1.0e-15, lumped=False)
    rhs, at_r = grab("kernels/UnitTestMomentumMassElem.C", "rhs", "momentum_time_derivative_lumped")
    msrc = open(os.path.join(ut, "kernels/UnitTestMomentumMassElem.C")).read()
    m = re.search(r"lhsExact\[i\*24\+i\]\s*=\s*([-+\d.eE]+)", msrc)
    diag = float(m.group(1))
    g["momentum_mass_lumped"] = dict(time, rhs=rhs, lhs=[diag if i % 25 == 0 else 0.0 for i in range(576)],
                                     at=[at_r, "unit_tests/kernels/UnitTestMomentumMassElem.C:%d"
                                         % (msrc.count("\n", 0, m.start()) + 1)], tol=1.0e-15, lumped=True)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nalu_unit_golds.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst, "with", len(g), "golds")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
