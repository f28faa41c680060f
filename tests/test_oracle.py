"""The CPU oracle against the reference's own outputs (tests/golden).

Element-level quantities (residual, Jacobian, mat-vec, sensitivities and
adjoint products) must agree to 1e-12 norm-wise relative error; the ILU(0)
factor/apply is checked on the reference's own matrix, where it must agree
to 1e-13.  Solutions, functions and total derivatives go through GMRES on
ill-conditioned shell systems, so they are compared at 1e-7 (bounded by
cond(K) x the 1e-12 solver tolerance, not by the element arithmetic).
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import CASES, ROOT, load_case, rel

oracle = pytest.importorskip("oracle")

ELEM_TOL = 1e-12
SOLVE_TOL = 1e-7


@pytest.fixture(scope="module", params=CASES)
def case(request):
    prob, ref = load_case(request.param)
    return request.param, prob, ref, oracle.Oracle(prob)


def test_known_answers_of_reference_tests():
    """Pins from the reference's own integration tests."""
    for name in ("hex_cube", "shell_beam"):
        prob, ref = load_case(name)
        assert rel(ref["funcs"], prob["func_refs"]) < 1e-8
        o = oracle.Oracle(prob)
        r = o.static_adjoint(prob["force"], prob["gmres_m"],
                             prob["gmres_restart"], prob["rtol"])
        assert rel(r["funcs"], prob["func_refs"]) < 1e-8


def test_residual_and_jacobian(case):
    name, prob, ref, o = case
    if "u_test" not in prob:
        pytest.skip("no unit state")
    u = prob["u_test"]
    assert rel(o.assemble_res(u), ref["res"]) < ELEM_TOL
    assert rel(o.assemble_res(u, apply_bcs=False), ref["res_nobc"]) < ELEM_TOL
    jr, A = o.assemble_jac(u)
    rowp, cols, vals = o.bcsr_arrays(A)
    assert np.array_equal(rowp, ref["jac_rowp"])
    assert np.array_equal(cols, ref["jac_cols"])
    if "jac_vals" in ref:
        assert rel(vals, ref["jac_vals"]) < ELEM_TOL
    assert rel(jr, ref["jac_res"]) < ELEM_TOL
    assert rel(o.mult(A, prob["x_test"]), ref["kx"]) < ELEM_TOL
    o.free(A)


def test_ilu0_on_reference_matrix(case):
    name, prob, ref, o = case
    if "jac_vals" not in ref:
        pytest.skip("matrix not stored")
    _, A = o.assemble_jac(prob["u_test"])
    v = np.ctypeslib.as_array(A.vals, (len(ref["jac_vals"]),))
    v[:] = ref["jac_vals"]
    F, fail = o.ilu0(A)
    assert fail == 0
    assert rel(o.ilu0_apply(F, prob["x_test"]), ref["ilu_apply"]) < 1e-13
    o.free(A)
    o.free(F)


def test_point_functions_and_sensitivities(case):
    name, prob, ref, o = case
    if "u_test" not in prob:
        pytest.skip("no unit state")
    u = prob["u_test"]
    assert rel(o.eval_funcs(u), ref["funcs_test"]) < ELEM_TOL
    assert rel(o.sv_sens(u, 0), ref["dfdu_test_comp"]) < ELEM_TOL
    assert rel(o.sv_sens(u, 1), ref["dfdu_test_ks"]) < ELEM_TOL
    assert rel(o.dv_sens(u, 0), ref["dfdx_test_comp"]) < ELEM_TOL
    assert rel(o.dv_sens(u, 1), ref["dfdx_test_ks"]) < 1e-11
    assert rel(o.adj_res_product(u, prob["psi_test"]),
               ref["adjres_test"]) < ELEM_TOL


def test_static_solve_and_adjoint_gradient(case):
    name, prob, ref, o = case
    r = o.static_adjoint(prob["force"], prob.get("gmres_m", 100),
                         prob.get("gmres_restart", 2), prob.get("rtol", 1e-12))
    assert r["flag"] == 1
    assert rel(r["u"], ref["u"]) < SOLVE_TOL
    assert rel(r["funcs"], ref["funcs"]) < SOLVE_TOL
    assert rel(r["grad_comp"], ref["grad_comp"]) < SOLVE_TOL
    assert rel(r["grad_ks"], ref["grad_ks"]) < SOLVE_TOL


def test_fp64_work_constants_match_operation_counts():
    """The per-element FP64 work bench.py quotes for the reference element
    (its addJacobian) is what the operation-counting build of the
    reference's sources prints (oracle/ref/opcount.h, op_count.cpp); runs
    where that build exists (make -C oracle/ref opc)."""
    import subprocess
    exe = os.path.join(ROOT, "oracle", "_ref", "op_count")
    if not os.path.exists(exe):
        pytest.skip("operation-counting build not present")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60,
                         check=True).stdout
    rows = {" ".join(line.split()[:-6]): int(line.split()[-1])
            for line in out.splitlines()[1:] if line.strip()}
    import bench
    for kind in ("shell", "hex"):
        assert rows[f"{kind} addJacobian"] == \
            bench.FP64_FLOPS_PER_ELEMENT[kind]["reference"]
