"""Fixed-geometry assembly (tg_assembler_set_fixed_geometry) on the GPU:
the residual and Jacobian formed from per-geometry coefficient matrices
(K = t K1 + t^3 K3 for the shell, t K1 for the hex) against the
reference's own outputs (golden fixtures) and the CPU oracle, at the
element-level tolerance 1e-12 (norm-wise, every Jacobian entry):

* every golden case (curved, warped, random and reference-axis shells,
  hex blocks and distorted hexes), with and without constraints;
* scaled-down copies of the benchmark workloads against the oracle;
* the same model with the cache off and on agree to rounding;
* the cache follows the design: new thicknesses after the build;
* set_nodes invalidates the cache: after moving nodes the results are
  those of the new geometry (oracle), not the old;
* a uniform structured plate has one geometry class;
* the function and sensitivity kernels (compliance, KS, addSVSens,
  addDVSens, addAdjointResProducts) with the cached strain operators
  against the reference's outputs, and a batched adjoint of several meshes
  against the same computation without the cache.
"""
import numpy as np
import pytest

from conftest import CASES, load_case, rel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-12


@pytest.fixture(scope="module")
def gpu():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import problem
    return problem


def _h(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("name", CASES)
def test_fixed_geometry_matches_reference(gpu, name):
    prob, ref = load_case(name)
    if "u_test" not in prob:
        pytest.skip("no unit state in this case")
    M = gpu.GpuModel(prob)
    M.set_fixed_geometry(True)
    u = M.vec(prob["u_test"])
    assert rel(_h(M.assemble_res(u)), ref["res"]) < ELEM_TOL
    assert rel(_h(M.assemble_res(u, apply_bcs=False)), ref["res_nobc"]) < \
        ELEM_TOL
    mat = M.new_mat()
    res = M.vec()
    M.assemble_jacobian(u, mat, res, apply_bcs=False)
    if "jac_nobc_vals" in ref:
        assert rel(_h(mat.vals), ref["jac_nobc_vals"]) < ELEM_TOL
    M.assemble_jacobian(u, mat, res)
    assert rel(_h(res), ref["jac_res"]) < ELEM_TOL
    if "jac_vals" in ref:
        assert rel(_h(mat.vals), ref["jac_vals"]) < ELEM_TOL
    assert rel(_h(mat.mult(M.vec(prob["x_test"]))), ref["kx"]) < ELEM_TOL


def _shapes():
    from tacs_gb300 import meshes
    return {"plate_c2_64": (lambda: meshes.plate_c2(64, 2.0, seed=2), 1e-3),
            "hex_c3_16": (lambda: meshes.hex_c3(16, 16, 8, seed=3), 1e-5),
            "cylinder_c5_48": (lambda: meshes.cylinder_c5(48, 32), 1e-4)}


@pytest.mark.parametrize("name", sorted(_shapes()))
def test_fixed_geometry_on_workload_shapes(gpu, name):
    import oracle
    build, scale = _shapes()[name]
    prob = build()
    o = oracle.Oracle(prob)
    M = gpu.GpuModel(prob)
    rng = np.random.default_rng(13)
    u = scale * rng.standard_normal(M.ndof)
    ud = M.vec(u)
    # cache off: the element kernels
    mat0, res0 = M.new_mat(), M.vec()
    M.assemble_jacobian(ud, mat0, res0)
    M.set_fixed_geometry(True)
    mat, res = M.new_mat(), M.vec()
    M.assemble_jacobian(ud, mat, res)
    r_ref, A = o.assemble_jac(u)
    _, _, vals = o.bcsr_arrays(A)
    o.free(A)
    assert rel(_h(res), r_ref) < ELEM_TOL
    assert rel(_h(mat.vals), vals) < ELEM_TOL
    assert rel(_h(mat.vals), _h(mat0.vals)) < 1e-13
    assert rel(_h(res), _h(res0)) < 1e-13
    assert rel(_h(M.assemble_res(ud, lam=0.5)),
               o.assemble_res(u, lam=0.5)) < ELEM_TOL
    info = M.fixed_geometry_info()
    assert info["classes"] >= 1 and info["table_bytes"] > 0
    if name == "hex_c3_16":  # uniform 1/8 spacing: a single geometry
        assert info["classes"] == 1


def test_fixed_geometry_follows_design_and_nodes(gpu):
    import oracle
    from tacs_gb300 import meshes
    rng = np.random.default_rng(21)
    prob = meshes.plate_c2(16, 0.5, seed=4)  # spacing 1/32: one class
    M = gpu.GpuModel(prob)
    M.set_fixed_geometry(True)
    u = 1e-3 * rng.standard_normal(M.ndof)
    ud = M.vec(u)
    mat, res = M.new_mat(), M.vec()
    M.assemble_jacobian(ud, mat, res)
    assert M.fixed_geometry_info()["classes"] == 1
    # new thicknesses: the cache holds no t
    t2 = rng.uniform(0.004, 0.03, prob["nelem"])
    M.set_design_vars(torch.as_tensor(t2, device="cuda"))
    M.assemble_jacobian(ud, mat, res)
    p2 = dict(prob)
    p2["thick"] = t2
    o2 = oracle.Oracle(p2)
    r_ref, A = o2.assemble_jac(u)
    _, _, vals = o2.bcsr_arrays(A)
    o2.free(A)
    assert rel(_h(mat.vals), vals) < ELEM_TOL
    assert rel(_h(res), r_ref) < ELEM_TOL
    # move the nodes (a warped surface): set_nodes invalidates the cache
    X = prob["xpts"].reshape(-1, 3).copy()
    X[:, 2] = 0.02 * np.sin(3.0 * X[:, 0]) * np.cos(2.0 * X[:, 1])
    M.set_nodes(torch.as_tensor(X.ravel(), device="cuda"))
    M.assemble_jacobian(ud, mat, res)
    p3 = dict(p2)
    p3["xpts"] = X.ravel()
    o3 = oracle.Oracle(p3)
    r_ref3, A3 = o3.assemble_jac(u)
    _, _, vals3 = o3.bcsr_arrays(A3)
    o3.free(A3)
    assert rel(_h(mat.vals), vals3) < ELEM_TOL
    assert rel(_h(res), r_ref3) < ELEM_TOL
    assert rel(vals3, vals) > 1e-6  # the geometry did change
    assert M.fixed_geometry_info()["classes"] > 1


@pytest.mark.parametrize("name", CASES)
def test_fixed_geometry_functions_and_sensitivities(gpu, name):
    prob, ref = load_case(name)
    if "u_test" not in prob:
        pytest.skip("no unit state in this case")
    M = gpu.GpuModel(prob)
    M.set_fixed_geometry(True)
    u = M.vec(prob["u_test"])
    assert rel(M.eval_functions(u), ref["funcs_test"]) < ELEM_TOL
    dc, dk = M.vec(), M.vec()
    M.add_sv_sens(u, [0, 1], [dc, dk])
    assert rel(_h(dc), ref["dfdu_test_comp"]) < ELEM_TOL
    assert rel(_h(dk), ref["dfdu_test_ks"]) < ELEM_TOL
    xc, xk = M.dv_vec(), M.dv_vec()
    M.add_dv_sens(u, [0, 1], [xc, xk])
    assert rel(_h(xc), ref["dfdx_test_comp"]) < ELEM_TOL
    assert rel(_h(xk), ref["dfdx_test_ks"]) < 1e-11
    xa = M.dv_vec()
    M.add_adjoint_res_products(u, [M.vec(prob["psi_test"])], [xa])
    assert rel(_h(xa), ref["adjres_test"]) < ELEM_TOL


def test_fixed_geometry_batched_adjoint(gpu):
    from tacs_gb300 import _lib, meshes
    bp = meshes.batch_plates(count=4, nmax=24, seed=8)
    out = []
    for fixed in (False, True):
        M = gpu.GpuModel(bp)
        if fixed:
            M.set_fixed_geometry(True)
        F = gpu.batch_loads(M)
        r = gpu.batched_adjoint(M, F, m=60, nrestart=40, rtol=1e-12,
                                func=_lib.FUNC_KS_FAILURE)
        assert r["flags_fwd"].all() and r["flags_adj"].all()
        out.append((r["funcs"], _h(r["grads"])))
    assert rel(out[1][0], out[0][0]) < 1e-9
    assert rel(out[1][1], out[0][1]) < 1e-7

