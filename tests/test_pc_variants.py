"""Preconditioner variants and matrix orientation on the GPU:
block Jacobi (diagonal-block inverses, BMatComputeInverse) against host
inverses, block-Jacobi GMRES against the ILU(0) solution, the transpose
assembly (TACS_MAT_TRANSPOSE) against the normal one, and the BCSR
mat-vec against a host product over the same blocks.  Tolerances: 1e-11
for the block inverses (different pivot order than numpy), 1e-7 for the
solutions (two preconditioners, both solved to 1e-12), exact for
the transpose assembly (the element matrices are assembled symmetric,
mirrored tiles) and 1e-13 for the mat-vec (summation order)."""
import numpy as np
import pytest

from conftest import load_case, rel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import _lib, problem
    return problem, _lib


def _h(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("name", ["hex_block", "shell_plate8"])
def test_block_jacobi_apply(gpu, name):
    problem, L = gpu
    prob, _ = load_case(name)
    M = problem.GpuModel(prob)
    mat = M.new_mat()
    M.assemble_jacobian(M.vec(prob["u_test"]), mat, M.vec())
    pc = problem.Pc(mat, L.PC_BLOCK_JACOBI)
    pc.factor()
    x = M.vec(prob["x_test"])
    y = _h(pc.apply(x))
    bs = mat.bsize
    rowp, cols = _h(mat.rowp), _h(mat.cols)
    vals = _h(mat.vals).reshape(-1, bs, bs)
    xx = prob["x_test"].reshape(-1, bs)
    expect = np.zeros_like(xx)
    for i in range(mat.nrows):
        j = rowp[i] + int(np.nonzero(cols[rowp[i]:rowp[i + 1]] == i)[0][0])
        expect[i] = np.linalg.solve(vals[j], xx[i])
    assert rel(y, expect.ravel()) < 1e-11


def test_block_jacobi_gmres_matches_ilu(gpu):
    problem, L = gpu
    prob, _ = load_case("hex_block")
    M = problem.GpuModel(prob)
    sols = []
    for kind in (L.PC_BLOCK_JACOBI, L.PC_ILU0):
        mat = M.new_mat()
        M.assemble_jacobian(M.vec(), mat, M.vec())
        pc = problem.Pc(mat, kind)
        pc.factor()
        ksm = problem.Ksm(mat, pc, 200, 40)
        ksm.set_tolerances(1e-12)
        b = M.vec(prob["force"])
        M.apply_bcs(b)
        x, flag = ksm.solve(b)
        assert flag == 1
        sols.append(_h(x))
    assert rel(sols[0], sols[1]) < 1e-7


@pytest.mark.parametrize("name", ["shell_rand", "hex_rand", "shell_plate8"])
def test_transpose_assembly_equals_normal(gpu, name):
    problem, L = gpu
    prob, _ = load_case(name)
    M = problem.GpuModel(prob)
    u = M.vec(prob["u_test"])
    A, B = M.new_mat(), M.new_mat()
    M.assemble_jacobian(u, A, M.vec())
    M.assemble_jacobian(u, B, M.vec(), transpose=True)
    assert torch.equal(A.vals, B.vals)


@pytest.mark.parametrize("name", ["shell_rand", "hex_rand"])
def test_matvec_against_host_bcsr(gpu, name):
    problem, L = gpu
    prob, _ = load_case(name)
    M = problem.GpuModel(prob)
    mat = M.new_mat()
    M.assemble_jacobian(M.vec(prob["u_test"]), mat, M.vec())
    x = M.vec(prob["x_test"])
    y = _h(mat.mult(x))
    bs = mat.bsize
    rowp, cols = _h(mat.rowp), _h(mat.cols)
    vals = _h(mat.vals).reshape(-1, bs, bs)
    xx = prob["x_test"].reshape(-1, bs)
    expect = np.zeros_like(xx)
    for i in range(mat.nrows):
        for j in range(rowp[i], rowp[i + 1]):
            expect[i] += vals[j] @ xx[cols[j]]
    assert rel(y, expect.ravel()) < 1e-13
