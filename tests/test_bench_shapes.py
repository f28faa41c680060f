"""GPU parity on scaled-down copies of the benchmark workloads, against the
CPU oracle (a restatement of the reference's element, assembly and function
code, itself pinned to the reference's outputs by tests/test_oracle.py).

The shapes keep what makes each workload distinct -- the simply supported
2 m plate with its sin x sin pressure field and seeded thicknesses, the SIMP
hex block (element scale t = rho^3) with its clamped face and traction
patch, the clamped cylinder with its axial edge load and internal pressure
-- at sizes the oracle assembles in well under a second.

Tolerances (norm-wise max|a-b| / max|b|): element-level results (residual,
every Jacobian entry, mat-vec, functions, state and design sensitivities,
adjoint products) 1e-12, the KS design sensitivity 1e-11 (its exponential
weights amplify rounding); solution, functions at the solution and the
adjoint gradients 1e-7 (two different exact solvers: the GPU multifrontal
factorisation against a symmetric sparse factorisation of the oracle's
matrix on the host).
"""
import numpy as np
import pytest

from conftest import exact_solve, rel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-12
KS_DV_TOL = 1e-11
SOLVE_TOL = 1e-7


def _shapes():
    from tacs_gb300 import meshes
    return {
        # 2 m plate of the 512 x 512 workload at 64 x 64
        "plate_c2_64": (lambda: meshes.plate_c2(64, 2.0, seed=2), 1e-3),
        # 128 x 128 x 64 SIMP block at 16 x 16 x 8 (four traction elements)
        "hex_c3_16": (lambda: meshes.hex_c3(16, 16, 8, seed=3), 1e-5),
        # 384 x 256 cylinder at 48 x 32
        "cylinder_c5_48": (lambda: meshes.cylinder_c5(48, 32), 1e-4),
    }


SHAPES = sorted(_shapes())


@pytest.fixture(scope="module")
def gpu():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import problem
    return problem


def _h(t):
    return t.detach().cpu().numpy()


def _bc_zero(prob, v):
    """Zero the constrained entries of a node-major vector (the reference's
    TACSBVec::applyBCs with zero values)."""
    vpn = 6 if prob["elem_type"] == 0 else 3
    out = np.array(v, np.float64).reshape(-1, vpn)
    for node, mask in zip(prob["bc_nodes"], prob["bc_masks"]):
        for k in range(vpn):
            if mask & (1 << k):
                out[node, k] = 0.0
    return out.ravel()


@pytest.mark.parametrize("name", SHAPES)
def test_element_level_parity_on_workload_shape(gpu, name):
    import oracle
    build, scale = _shapes()[name]
    prob = build()
    o = oracle.Oracle(prob)
    M = gpu.GpuModel(prob)
    rng = np.random.default_rng(11)
    u = scale * rng.standard_normal(M.ndof)
    x = rng.standard_normal(M.ndof)
    psi = rng.standard_normal(M.ndof)
    ud = M.vec(u)

    assert rel(_h(M.assemble_res(ud)), o.assemble_res(u)) < ELEM_TOL
    assert rel(_h(M.assemble_res(ud, apply_bcs=False)),
               o.assemble_res(u, apply_bcs=False)) < ELEM_TOL
    mat = M.new_mat()
    res = M.vec()
    M.assemble_jacobian(ud, mat, res)
    r_ref, A = o.assemble_jac(u)
    rowp, cols, vals = o.bcsr_arrays(A)
    assert np.array_equal(_h(mat.rowp), rowp)
    assert np.array_equal(_h(mat.cols), cols)
    assert rel(_h(res), r_ref) < ELEM_TOL
    # every Jacobian entry, not a sum or a product
    assert rel(_h(mat.vals), vals) < ELEM_TOL
    assert rel(_h(mat.mult(M.vec(x))), o.mult(A, x)) < ELEM_TOL
    o.free(A)

    assert rel(M.eval_functions(ud), o.eval_funcs(u)) < ELEM_TOL
    dc, dk = M.vec(), M.vec()
    M.add_sv_sens(ud, [0, 1], [dc, dk])
    assert rel(_h(dc), o.sv_sens(u, 0)) < ELEM_TOL
    assert rel(_h(dk), o.sv_sens(u, 1)) < ELEM_TOL
    xc, xk = M.dv_vec(), M.dv_vec()
    M.add_dv_sens(ud, [0, 1], [xc, xk])
    assert rel(_h(xc), o.dv_sens(u, 0)) < ELEM_TOL
    assert rel(_h(xk), o.dv_sens(u, 1)) < KS_DV_TOL
    xa = M.dv_vec()
    M.add_adjoint_res_products(ud, [M.vec(psi)], [xa])
    assert rel(_h(xa), o.adj_res_product(u, psi)) < ELEM_TOL


def _checker_adjoint(prob):
    """Static solve and adjoint gradients on the CPU: the oracle's matrix,
    residual, functions and element sensitivities, with an exact sparse
    solve (conftest.exact_solve) as the solver, in the order of the
    reference harness (K and R at
    u = 0, u = -K^-1 (R - f), psi = K^-1 dfdu with the row-BC matrix,
    grad = dfdx - psi^T dR/dx)."""
    import oracle
    from scipy import sparse
    o = oracle.Oracle(prob)
    n = o.ndof
    r0, A = o.assemble_jac(np.zeros(n))
    rowp, cols, vals = o.bcsr_arrays(A)
    b = o.vpn
    K = sparse.bsr_matrix((vals.reshape(-1, b, b), cols, rowp),
                          shape=(n, n)).tocsr()
    o.free(A)
    f = _bc_zero(prob, prob["force"])
    u = -exact_solve(K, r0 - f, prob)
    funcs = o.eval_funcs(u)
    grads = []
    for w in (0, 1):
        dfdu = _bc_zero(prob, o.sv_sens(u, w))
        psi = exact_solve(K, dfdu, prob)
        grads.append(o.dv_sens(u, w) + o.adj_res_product(u, psi, -1.0))
    return u, funcs, grads


@pytest.mark.direct
@pytest.mark.parametrize("name", SHAPES)
def test_solution_and_gradients_on_workload_shape(gpu, name):
    build, _ = _shapes()[name]
    prob = build()
    u_ref, f_ref, g_ref = _checker_adjoint(prob)
    M = gpu.GpuModel(prob)
    r = gpu.static_adjoint(M, prob["force"], direct=True)
    assert r["flag"] == 1
    assert rel(_h(r["u"]), u_ref) < SOLVE_TOL
    assert rel(r["funcs"], f_ref) < SOLVE_TOL
    assert rel(_h(r["grads"][0]), g_ref[0]) < SOLVE_TOL
    assert rel(_h(r["grads"][1]), g_ref[1]) < SOLVE_TOL
    if "rho" in prob:
        # SIMP: t = rho^3, so df/drho = 3 rho^2 df/dt
        drho = 3.0 * prob["rho"] ** 2 * _h(r["grads"][0])
        assert rel(drho, 3.0 * prob["rho"] ** 2 * g_ref[0]) < SOLVE_TOL
