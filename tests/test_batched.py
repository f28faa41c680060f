"""Batched solves on the GPU: several right-hand sides and several
independent meshes (element / row segments) in one GMRES, checked against
one-at-a-time GPU solves (themselves pinned to the reference through
test_gpu_parity) and, for the multi-RHS case, a host direct solve.

Tolerances: states, function values and gradients 1e-7 relative (the
solver tolerance times the conditioning of the clamped plates)."""
import numpy as np
import pytest

from conftest import rel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-7


@pytest.fixture(scope="module")
def gpu():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import problem
    return problem


def _h(t):
    return t.detach().cpu().numpy()


def _dense(mat):
    bs, nr = mat.bsize, mat.nrows
    rowp, cols = _h(mat.rowp), _h(mat.cols)
    vals = _h(mat.vals).reshape(-1, bs, bs)
    A = np.zeros((nr * bs, nr * bs))
    for i in range(nr):
        for j in range(rowp[i], rowp[i + 1]):
            c = cols[j]
            A[i * bs:(i + 1) * bs, c * bs:(c + 1) * bs] = vals[j]
    return A


# An FP32 ILU(0) factor is only a preconditioner where its rounding is not
# amplified: the natural-order block factors of thin shells (thickness well
# below the element size) amplify last-bit changes by up to ~1e9 (the
# reference's own FP64 factors, see test_gpu_parity), so the FP32 cases
# below use plates with thickness comparable to the element size.
@pytest.mark.parametrize("mixed", [False, True])
def test_multi_rhs_matches_direct_solve(gpu, mixed):
    from tacs_gb300 import _lib, meshes
    rng = np.random.default_rng(7)
    p = meshes.clamped_plate(10, thick=rng.uniform(0.06, 0.12, 100))
    M = gpu.GpuModel(p)
    mat = M.new_mat()
    M.assemble_jacobian(M.vec(), mat, M.vec())
    pc = gpu.Pc(mat, _lib.PC_ILU0,
                _lib.PREC_FP32 if mixed else _lib.PREC_FP64)
    pc.factor()
    ksm = gpu.Ksm(mat, pc, 60, 40, mixed)
    ksm.set_tolerances(1e-10)
    B = torch.zeros(3, M.ndof, dtype=torch.float64, device="cuda")
    B[0] = -M.assemble_res(M.vec(), apply_bcs=False)
    B[1, 6 * 60 + 2] = 1e3
    B[2] = torch.as_tensor(rng.standard_normal(M.ndof), device="cuda")
    for lc in range(3):
        M.apply_bcs(B[lc])
    X, it, fl, rn, rc = ksm.solve_multi(B)
    assert rc == 1 and fl.all()
    A = _dense(mat)
    Xd = np.linalg.solve(A, _h(B).T).T
    for lc in range(3):
        assert rel(_h(X[lc]), Xd[lc]) < TOL
    # the same systems one at a time give the same iterates' answer
    for lc in range(3):
        x1, f1 = ksm.solve(B[lc].clone())
        assert f1 == 1
        assert rel(_h(x1), Xd[lc]) < TOL


@pytest.mark.parametrize("pc_kind,mixed,tmin,tmax", [
    (0, False, 0.004, 0.02), (2, False, 0.004, 0.02), (2, True, 0.004, 0.02),
    (0, True, 0.05, 0.1)])
def test_batched_meshes_match_independent_solves(gpu, pc_kind, mixed, tmin,
                                                 tmax):
    from tacs_gb300 import _lib, meshes
    bp = meshes.batch_plates(count=3, seed=4, nmin=12, nmax=20, tmin=tmin,
                             tmax=tmax)
    M = gpu.GpuModel(bp)
    F = gpu.batch_loads(M)
    # m above the plates' free dof count: no restarted-GMRES stagnation
    r = gpu.batched_adjoint(M, F, m=1500, nrestart=2, rtol=1e-10,
                            pc_kind=pc_kind, mixed=mixed,
                            func=_lib.FUNC_KS_FAILURE)
    assert r["flags_fwd"].all(), (r["flags_fwd"], r["iters_fwd"],
                                  r["resnorm_fwd"])
    assert r["flags_adj"].all(), (r["flags_adj"], r["iters_adj"],
                                  r["resnorm_adj"])
    nseg = len(bp["plate_n"])
    nptr, eptr = bp["seg_node_ptr"], bp["seg_elem_ptr"]
    for g in range(nseg):
        n = int(bp["plate_n"][g])
        pg = meshes.clamped_plate(n, thick=bp["thick"][eptr[g]:eptr[g + 1]])
        Mg = gpu.GpuModel(pg)
        mat = Mg.new_mat()
        Mg.assemble_jacobian(Mg.vec(), mat, Mg.vec())
        pc = gpu.Pc(mat, _lib.PC_ILU0)
        pc.factor()
        ksm = gpu.Ksm(mat, pc, 1500, 2)
        ksm.set_tolerances(1e-12)
        sl = slice(6 * nptr[g], 6 * nptr[g + 1])
        for lc in range(F.shape[0]):
            f = F[lc, sl].clone()
            Mg.apply_bcs(f)
            u, fl = ksm.solve(f)
            assert fl == 1
            assert rel(_h(r["u"][lc, sl]), _h(u)) < TOL
            ks = Mg.eval_functions(u, [_lib.FUNC_KS_FAILURE])[0]
            assert abs(r["funcs"][lc, g] - ks) < TOL * abs(ks)
            dfdu = Mg.vec()
            Mg.add_sv_sens(u, [_lib.FUNC_KS_FAILURE], [dfdu])
            Mg.apply_bcs(dfdu)
            psi, fl = ksm.solve(dfdu)
            assert fl == 1
            gr = Mg.dv_vec()
            Mg.add_total_derivative(u, _lib.FUNC_KS_FAILURE, psi, gr, 1.0,
                                    -1.0)
            assert rel(_h(r["grads"][lc, eptr[g]:eptr[g + 1]]), _h(gr)) < TOL


@pytest.mark.gpu
def test_restart_cycle_runs_as_one_graph():
    """Each GMRES restart cycle is one graph whose WHILE node repeats the
    Arnoldi step on the device (tg_ksm_get_graph_info), in FP64 and mixed
    precision, and the solves it runs meet their tolerance.  The plate is
    12 x 12 at t = 0.05: GMRES(30) with ILU(0) in natural order converges
    there (22 iterations on the oracle); on thinner plates it stagnates in
    either precision."""
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import _lib, meshes, problem
    prob = meshes.clamped_plate(12, t=0.05)
    M = problem.GpuModel(prob)
    mat = M.new_mat()
    r0 = M.vec()
    M.assemble_jacobian(M.vec(), mat, r0)
    b = -r0
    for mixed in (False, True):
        pc = problem.Pc(mat, _lib.PC_ILU0,
                        _lib.PREC_FP32 if mixed else _lib.PREC_FP64)
        pc.factor()
        ksm = problem.Ksm(mat, pc, 30, 20, mixed)
        ksm.set_tolerances(1e-10)
        x, flag = ksm.solve(b)
        info = ksm.graph_info()
        assert flag == 1
        assert info["cycle_graph"] and info["step_launches"] > 0
        assert (info["step_launches_fp32"] > 0) == mixed
        r = mat.mult(x) - b
        assert float(r.norm() / b.norm()) < 1e-9



def test_segment_ks_save_restore(gpu):
    """The per-range KS statistics saved after one state's evaluation and
    restored after another's give that state's total derivative bitwise
    (tg_segment_ks_save / tg_segment_ks_restore); restoring without a
    saved buffer of the right kind is refused before any evaluation."""
    from tacs_gb300 import _lib, meshes
    bp = meshes.batch_plates(count=3, seed=4, nmin=8, nmax=12)
    M = gpu.GpuModel(bp)
    M.set_segments(bp["seg_elem_ptr"])
    g = torch.Generator(device="cuda").manual_seed(11)
    U = 1e-4 * torch.randn(2, M.ndof, dtype=torch.float64, device="cuda",
                           generator=g)
    psi = torch.randn(M.ndof, dtype=torch.float64, device="cuda",
                      generator=g)
    f = _lib.FUNC_KS_FAILURE
    M.eval_functions_segments(U[0], f)
    ks0 = M.segment_ks_save()
    ref = M.dv_vec()
    M.add_total_derivative_segments(U[0], f, psi, ref, 1.0, -1.0)
    M.eval_functions_segments(U[1], f)  # another state's statistics
    M.segment_ks_restore(ks0)
    got = M.dv_vec()
    M.add_total_derivative_segments(U[0], f, psi, got, 1.0, -1.0)
    assert torch.equal(got, ref)
    M2 = gpu.GpuModel(bp)
    M2.set_segments(bp["seg_elem_ptr"])
    with pytest.raises(_lib.TacsGpuError):
        M2.segment_ks_save()
