"""Block ILU(k) (TACSAdditiveSchwarz(mat, levFill, fill) with levFill > 0,
the BCSRMat::computeILUk pattern, src/bpmat/BCSRMat.cpp:625).

* the oracle's ILU(1) / ILU(2) applies on the reference's own matrix
  against the reference's (CPU; 1e-13, same arithmetic order);
* the GPU factor's block count against the oracle's pattern, and its
  applies on the reference's matrix against the reference: 1e-9, or 20x
  the spread that a rounding-level change of K causes in the reference's
  own apply when that is larger (thin-shell factors amplify last-bit
  differences; the same bar as ILU(0));
* GMRES with ILU(1) / ILU(3) on a thin clamped plate where ILU(0)
  stalls: fewer iterations with more fill, true residual 1e-10 and the
  solution against a sparse direct solve (1e-5), FP64 and with the FP32
  factor inside FP64 GMRES.
"""
import numpy as np
import pytest

from conftest import CASES, load_case, rel

ILUK_CASES = [c for c in CASES if "ilu1_apply" in load_case(c)[1]]
MAT_CASES = [c for c in ILUK_CASES if "jac_vals" in load_case(c)[1]]


def _oracle_on_reference_matrix(prob, ref):
    import oracle
    o = oracle.Oracle(prob)
    _, A = o.assemble_jac(prob["u_test"])
    v = np.ctypeslib.as_array(A.vals, (len(ref["jac_vals"]),))
    v[:] = ref["jac_vals"]
    return o, A


@pytest.mark.parametrize("name", MAT_CASES)
@pytest.mark.parametrize("lev", [1, 2])
def test_oracle_iluk_on_reference_matrix(name, lev):
    prob, ref = load_case(name)
    o, A = _oracle_on_reference_matrix(prob, ref)
    F, fail = o.iluk(A, lev)
    assert fail == 0
    assert rel(o.ilu0_apply(F, prob["x_test"]), ref[f"ilu{lev}_apply"]) < 1e-13
    # the random-element cases are separate dense elements: no fill
    if "rand" not in name:
        assert F.rowp[F.nrows] > A.rowp[A.nrows]
    o.free(A)
    o.free(F)


def test_oracle_iluk_zero_fill_is_ilu0():
    prob, ref = load_case("shell_plate8")
    o, A = _oracle_on_reference_matrix(prob, ref)
    F0, _ = o.ilu0(A)
    Fk, _ = o.iluk(A, 0)
    assert Fk.rowp[Fk.nrows] == A.rowp[A.nrows]
    assert rel(o.ilu0_apply(Fk, prob["x_test"]),
               o.ilu0_apply(F0, prob["x_test"])) == 0.0


# ------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import _lib, problem
    return problem, _lib, torch


@pytest.mark.gpu
@pytest.mark.parametrize("name", MAT_CASES)
@pytest.mark.parametrize("lev", [1, 2])
def test_iluk_apply_on_reference_matrix(gpu, name, lev):
    problem, L, torch = gpu
    prob, ref = load_case(name)
    M = problem.GpuModel(prob)
    mat = M.new_mat()
    mat.vals.copy_(torch.as_tensor(ref["jac_vals"], device="cuda"))
    pc = problem.Pc(mat, lev_fill=lev)
    pc.factor()
    y = pc.apply(M.vec(prob["x_test"])).cpu().numpy()
    o, A = _oracle_on_reference_matrix(prob, ref)
    F, _ = o.iluk(A, lev)
    assert pc.fill() == (lev, F.rowp[F.nrows])
    # the reference's own sensitivity to a rounding-level change of K
    _, A2 = o.assemble_jac(prob["u_test"])
    F2, _ = o.iluk(A2, lev)
    spread = rel(o.ilu0_apply(F2, prob["x_test"]), ref[f"ilu{lev}_apply"])
    assert rel(y, ref[f"ilu{lev}_apply"]) < max(1e-9, 20.0 * spread)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["shell", "hex"])
def test_iluk_apply_matches_oracle(gpu, kind):
    """Same matrix (the oracle's) in both factors, levels 1-3."""
    problem, L, torch = gpu
    import oracle
    from tacs_gb300 import meshes
    prob = meshes.clamped_plate(12) if kind == "shell" else \
        meshes.hex_c3(8, 8, 4)
    o = oracle.Oracle(prob)
    _, A = o.assemble_jac(np.zeros(o.ndof))
    M = problem.GpuModel(prob)
    mat = M.new_mat()
    nv = mat.vals.numel()
    mat.vals.copy_(torch.as_tensor(
        np.ctypeslib.as_array(A.vals, (nv,)).copy(), device="cuda"))
    x = np.random.default_rng(3).standard_normal(o.ndof)
    for lev in (1, 2, 3):
        pc = problem.Pc(mat, lev_fill=lev)
        pc.factor()
        y = pc.apply(M.vec(x)).cpu().numpy()
        F, _ = o.iluk(A, lev)
        assert pc.fill()[1] == F.rowp[F.nrows]
        assert rel(y, o.ilu0_apply(F, x)) < 1e-10, lev


@pytest.mark.gpu
def test_gmres_iluk_thin_plate(gpu):
    """A thin clamped plate (32 x 32, t = 5 mm) in the natural order: the
    ILU(0) factor is unstable there (|M^-1 b| ~ 1e17 |x|, GMRES stalls),
    ILU(1) and ILU(3) converge (ILU(2) is unstable again: the oracle,
    restating the reference's factorisation, behaves the same).  Checked:
    convergence, fewer iterations with more fill, the true residual
    (1e-10) and the solution against a sparse direct solve (1e-5: cond(K)
    x the 1e-12 GMRES tolerance), in FP64 and with the FP32 ILU(3) inside
    FP64 GMRES."""
    problem, L, torch = gpu
    from scipy import sparse
    from scipy.sparse.linalg import spsolve
    from tacs_gb300 import meshes
    prob = meshes.clamped_plate(32, t=0.005)
    M = problem.GpuModel(prob)
    mat = M.new_mat()
    r0 = M.vec()
    M.assemble_jacobian(M.vec(), mat, r0)
    b = M.vec(prob["force"])
    M.apply_bcs(b)
    b -= r0
    bs = mat.bsize
    K = sparse.bsr_matrix((mat.vals.cpu().numpy().reshape(-1, bs, bs),
                           mat.cols.cpu().numpy(), mat.rowp.cpu().numpy()),
                          shape=(M.ndof, M.ndof)).tocsc()
    bh = b.cpu().numpy()
    x_ref = spsolve(K, bh)

    def check(x):
        assert np.linalg.norm(K @ x - bh) < 1e-10 * np.linalg.norm(bh)
        assert rel(x, x_ref) < 1e-5

    flags, iters = {}, {}
    for lev in (0, 1, 3):
        pc = problem.Pc(mat, lev_fill=lev)
        pc.factor()
        # ILU(0) only has to show that it does not converge quickly
        ksm = problem.Ksm(mat, pc, 200, 2 if lev == 0 else 50)
        ksm.set_tolerances(1e-12)
        x, flags[lev] = ksm.solve(b)
        iters[lev] = ksm.iters
        if lev > 0:
            assert flags[lev] == 1, (flags, iters)
            check(x.cpu().numpy())
    assert iters[3] < iters[1] < 600 <= iters[0], iters
    pc = problem.Pc(mat, L.PC_ILU0, L.PREC_FP32, lev_fill=3)
    pc.factor()
    ksm = problem.Ksm(mat, pc, 200, 50, mixed=True)
    ksm.set_tolerances(1e-12)
    x, flag = ksm.solve(b)
    assert flag == 1
    check(x.cpu().numpy())
