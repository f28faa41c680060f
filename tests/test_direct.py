"""The direct factorisation on the GPU (tg_direct: nested dissection,
supernodes, level-by-level multifrontal block Cholesky; the host analysis
and the kernels are also checked on the CPU in test_direct_symbolic.py).

* static solves K u = f - R(0) against the reference's own solutions
  (golden fixtures): 1e-7, the GMRES tolerance of the reference's solve
  times cond(K);
* a thin simply supported plate, where ILU(0)-GMRES stalls: the true
  residual at rounding level (1e-13 of |K| |u|) and agreement with an exact
  sparse solve on the host (conftest.exact_solve: constrained dofs
  removed, unit-diagonal scaling, symmetric factorisation) within 1e-8 or
  10x the rounding spread of that solve (its distance between two
  elimination orders), whichever is larger;
* both orders (node coordinates and level structures) and refactoring
  after new matrix values;
* the reference harness's adjoint gradients with both solves direct.
"""
import numpy as np
import pytest

from conftest import exact_and_spread, load_case, rel

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu, pytest.mark.direct]


@pytest.fixture(scope="module")
def gpu():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import problem
    return problem


def _host_matrix(mat, ndof):
    from scipy import sparse
    bs = mat.bsize
    return sparse.bsr_matrix((mat.vals.cpu().numpy().reshape(-1, bs, bs),
                              mat.cols.cpu().numpy(), mat.rowp.cpu().numpy()),
                             shape=(ndof, ndof)).tocsc()


def _rhs(M, prob, mat):
    r0 = M.vec()
    M.assemble_jacobian(M.vec(), mat, r0)
    f = M.vec(prob["force"])
    M.apply_bcs(f)
    return f - r0


@pytest.mark.parametrize("name", ["shell_plate8", "shell_c1", "hex_block",
                                  "shell_cyl"])
@pytest.mark.parametrize("coords", [True, False])
def test_direct_static_solve_matches_reference(gpu, name, coords):
    prob, ref = load_case(name)
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    b = _rhs(M, prob, mat)
    d = gpu.Direct(mat, use_coords=coords)
    d.factor()
    u = d.solve(b)
    assert rel(u.cpu().numpy(), ref["u"]) < 1e-7
    st = d.stats()
    assert st["supernodes"] > 0 and st["levels"] > 0


def test_direct_thin_plate_where_ilu_stalls(gpu):
    from tacs_gb300 import meshes
    n = 48
    prob = meshes.plate(n, n, 2.0, 2.0, t=0.002)
    e = meshes.plate_edges(n, n).astype(np.int32)
    prob["bc_nodes"], prob["bc_masks"] = e, np.full(len(e), 0x07, np.int32)
    prob["pres_elems"] = np.arange(n * n, dtype=np.int32)
    prob["pres_vals"] = np.full(4 * n * n, 1e3)
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    b = _rhs(M, prob, mat)
    d = gpu.Direct(mat)
    d.factor()
    u = d.solve(b).cpu().numpy()
    K = _host_matrix(mat, M.ndof)
    bh = b.cpu().numpy()
    Kinf = abs(K).sum(axis=1).max()
    assert np.abs(K @ u - bh).max() < 1e-13 * Kinf * np.abs(u).max()
    x_ref, spread, spread_c = exact_and_spread(K, bh, prob)
    assert rel(u, x_ref) < max(1e-8, 10.0 * spread)
    assert abs(bh @ u - bh @ x_ref) / abs(bh @ x_ref) < max(1e-12,
                                                            10.0 * spread_c)


def test_direct_refactor_after_new_values(gpu):
    from tacs_gb300 import meshes
    rng = np.random.default_rng(3)
    prob = meshes.clamped_plate(16, thick=rng.uniform(0.005, 0.02, 256))
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    b = _rhs(M, prob, mat)
    d = gpu.Direct(mat)
    d.factor()
    u1 = d.solve(b)
    # new thicknesses: same pattern, new values, same analysis
    M.set_design_vars(torch.as_tensor(rng.uniform(0.005, 0.02, 256),
                                      device="cuda"))
    b2 = _rhs(M, prob, mat)
    d.factor()
    u2 = d.solve(b2)
    r = mat.mult(u2) - b2
    assert (r.abs().max() / b2.abs().max()).item() < 1e-9
    assert not torch.equal(u1, u2)


@pytest.mark.parametrize("name", ["shell_plate8", "hex_block", "shell_cyl"])
def test_direct_adjoint_gradients_match_reference(gpu, name):
    """The reference harness's static solve and adjoint with both solves
    direct: functions, design and node-coordinate gradients against the
    reference's (1e-7)."""
    prob, ref = load_case(name)
    M = gpu.GpuModel(prob)
    r = gpu.static_adjoint(M, prob["force"], direct=True)
    assert rel(r["u"].cpu().numpy(), ref["u"]) < 1e-7
    assert rel(r["funcs"], ref["funcs"]) < 1e-7
    assert rel(r["grads"][0].cpu().numpy(), ref["grad_comp"]) < 1e-7
    assert rel(r["grads"][1].cpu().numpy(), ref["grad_ks"]) < 1e-7
    for k, key in ((0, "comp"), (1, "ks")):
        M.eval_functions(r["u"], [k])
        g = M.node_vec()
        M.add_total_xpt_derivative(r["u"], k, r["psis"][k], g, 1.0, -1.0)
        assert rel(g.cpu().numpy(), ref["grad_xpt_" + key]) < 1e-7


def test_direct_batched_adjoint_matches_gmres(gpu):
    """Independent plates x 4 load cases: the batched KS adjoint with the
    complete factorisation against the batched GMRES + ILU(0) one (both to
    their tolerances: 1e-6 on the gradients)."""
    from tacs_gb300 import meshes
    bp = meshes.batch_plates(count=5, nmin=8, nmax=24)
    M = gpu.GpuModel(bp)
    F = gpu.batch_loads(M)
    a = gpu.batched_adjoint(M, F, rtol=1e-12, direct=True)
    b = gpu.batched_adjoint(M, F, m=200, nrestart=100, rtol=1e-12)
    assert int(b["flags_fwd"].sum()) == b["flags_fwd"].size
    assert rel(a["funcs"], b["funcs"]) < 1e-8
    assert rel(a["grads"].cpu().numpy(), b["grads"].cpu().numpy()) < 1e-6


@pytest.mark.parametrize("func", [0, 1])
def test_direct_autograd_matches_reference_adjoint(gpu, func):
    """torch.autograd through the direct solves: the reference's adjoint
    gradient (1e-7)."""
    from tacs_gb300 import autograd as ag
    prob, ref = load_case("shell_plate8")
    M = gpu.GpuModel(prob)
    solver = ag.StaticSolver(M, prob["force"], direct=True)
    x = np.zeros(M.ndv)
    x[np.asarray(prob["dvnum"])] = prob["thick"]
    x = torch.as_tensor(x, device="cuda").requires_grad_(True)
    f = ag.static_functional(x, solver, func)
    assert abs(f.item() - ref["funcs"][func]) < 1e-7 * abs(ref["funcs"][func])
    f.sum().backward()
    g_ref = ref["grad_comp"] if func == 0 else ref["grad_ks"]
    assert rel(x.grad.cpu().numpy(), g_ref) < 1e-7


@pytest.mark.parametrize("name", ["shell_plate8", "hex_block"])
def test_mixed_direct_adjoint_gradients(gpu, name):
    """FP32 factorisation with FP64 refinement of every solve: the
    reference's functions and gradients (1e-7) and the all-FP64 direct
    gradients (1e-8)."""
    prob, ref = load_case(name)
    M = gpu.GpuModel(prob)
    r = gpu.static_adjoint(M, prob["force"], direct="mixed")
    r64 = gpu.static_adjoint(M, prob["force"], direct=True)
    assert rel(r["funcs"], ref["funcs"]) < 1e-7
    assert rel(r["grads"][0].cpu().numpy(), ref["grad_comp"]) < 1e-7
    assert rel(r["grads"][1].cpu().numpy(), ref["grad_ks"]) < 1e-7
    for k in range(2):
        assert rel(r["grads"][k].cpu().numpy(),
                   r64["grads"][k].cpu().numpy()) < 1e-8


def test_direct_as_gmres_preconditioner(gpu):
    """The complete factorisation as a GMRES preconditioner (TG_PC_DIRECT):
    one or two iterations in FP64; in FP32 inside FP64 flexible GMRES with
    refinement (GMRES-IR) on a thin simply supported plate, where the
    requested true residual (1e-12 |r0|) lies below what FP64 attains
    (cond(K) ~ 1e12): converged at the FP64 accuracy floor, the true
    residual at rounding level, and the FP64 solution within 10x the
    rounding spread of an exact solve."""
    from tacs_gb300 import _lib, meshes
    n = 32
    prob = meshes.plate(n, n, 2.0, 2.0, t=0.002)
    e = meshes.plate_edges(n, n).astype(np.int32)
    prob["bc_nodes"], prob["bc_masks"] = e, np.full(len(e), 0x07, np.int32)
    prob["pres_elems"] = np.arange(n * n, dtype=np.int32)
    prob["pres_vals"] = np.full(4 * n * n, 1e3)
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    b = _rhs(M, prob, mat)
    pc = gpu.Pc(mat, _lib.PC_DIRECT)
    pc.factor()
    ksm = gpu.Ksm(mat, pc, 20, 2)
    ksm.set_tolerances(1e-12)
    x64, flag = ksm.solve(b)
    assert flag == 1 and ksm.iters <= 3
    pc32 = gpu.Pc(mat, _lib.PC_DIRECT, _lib.PREC_FP32)
    pc32.factor()
    ksm32 = gpu.Ksm(mat, pc32, 50, 10, mixed=True)
    ksm32.set_tolerances(1e-12)
    x32, flag = ksm32.solve(b)
    assert flag == 1
    K = _host_matrix(mat, M.ndof)
    bh, xh = b.cpu().numpy(), x32.cpu().numpy()
    Kinf = abs(K).sum(axis=1).max()
    assert np.abs(K @ xh - bh).max() < 1e-13 * Kinf * np.abs(xh).max()
    _, spread, spread_c = exact_and_spread(K, bh, prob)
    x64h = x64.cpu().numpy()
    assert rel(xh, x64h) < max(1e-8, 10.0 * spread)
    assert abs(bh @ xh - bh @ x64h) / abs(bh @ x64h) < max(1e-12,
                                                            10.0 * spread_c)


@pytest.mark.parametrize("thin", [False, True], ids=["t10mm", "t2mm"])
def test_mixed_direct_stops_on_backward_error_or_falls_back(gpu, thin):
    """FP32 factorisation + FP64 refinement converges when the normwise
    backward error reaches eps sqrt(N) (and refines on while the steps halve
    it); where it cannot (refinement stagnates, cond(K) near 2^24) the
    solve is done by GMRES preconditioned by the FP32 factorisation
    (GMRES-IR), and where the FP32 Cholesky breaks down by an FP64
    factorisation.  Every way the result has the FP64 backward error
    (1e-13) and is the FP64 direct solution to within 10x the rounding
    spread of an exact solve (1e-8 where that is smaller)."""
    from tacs_gb300 import _lib, meshes
    n = 48
    prob = meshes.plate(n, n, 2.0, 2.0, t=0.002 if thin else 0.01)
    e = meshes.plate_edges(n, n).astype(np.int32)
    prob["bc_nodes"], prob["bc_masks"] = e, np.full(len(e), 0x07, np.int32)
    prob["pres_elems"] = np.arange(n * n, dtype=np.int32)
    prob["pres_vals"] = np.full(4 * n * n, 1e3)
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    b = _rhs(M, prob, mat)
    d64 = gpu.Direct(mat)
    d64.factor()
    x64 = d64.solve(b)
    d32 = gpu.Direct(mat, precision=_lib.PREC_FP32)
    d32.factor()
    x = d32.solve(b)
    st = d32.stats()
    tol = 2.0 ** -53 * np.sqrt(M.ndof)
    assert (st["fell_back_to_fp64"] or st["fp32_mode"] == "gmres_ir"
            or st["last_backward_error"] <= tol)
    if not thin:
        assert not st["fell_back_to_fp64"] and st["fp32_mode"] == "refine"
        # refinement runs on while a step halves the backward error
        assert 1 <= st["last_refinement_steps"] <= 30
    K = _host_matrix(mat, M.ndof)
    bh, xh, x64h = b.cpu().numpy(), x.cpu().numpy(), x64.cpu().numpy()
    _, spread, spread_c = exact_and_spread(K, bh, prob)
    assert rel(xh, x64h) < max(1e-8, 10.0 * spread)
    assert abs(bh @ xh - bh @ x64h) / abs(bh @ x64h) < max(1e-12,
                                                            10.0 * spread_c)
    r = (mat.mult(x) - b).abs().max().item()
    Kinf = abs(K).sum(axis=1).max()
    assert r < 1e-13 * (Kinf * x.abs().max().item() + b.abs().max().item())


@pytest.mark.parametrize("nrhs", [3, 4, 6])
@pytest.mark.parametrize("case", ["shell_c1", "plate_c2_128"])
def test_direct_multi_rhs(gpu, nrhs, case):
    """Several right-hand sides per pass over the factor
    (tg_direct_solve_multi, tg_direct_solve_refined_multi): FP64 solutions
    are bitwise those of single solves; the FP32 factorisation refines all
    of them together with a stopping test per right-hand side, and each
    ends within 1e-10 of the FP64 solution, as a single refined solve
    does.  On the C1 fixture and on a 128 x 128 plate (fronts solved by
    one CTA up to 768 rows and by thread-block clusters above)."""
    from tacs_gb300 import _lib, meshes
    if case == "plate_c2_128":  # fronts of up to ~1,500 rows: the one-CTA
        # solves' largest workspace and the cluster solves
        prob = meshes.plate_c2(128, 0.5, seed=2)
        M = gpu.GpuModel(prob)
        mat = M.new_mat()
        b0 = M.vec()
        M.assemble_jacobian(M.vec(), mat, b0)
        b0 = -b0
    else:
        prob, _ = load_case(case)
        M = gpu.GpuModel(prob)
        mat = M.new_mat()
        b0 = _rhs(M, prob, mat)
    g = torch.Generator(device="cuda").manual_seed(nrhs)
    B = torch.randn(nrhs, M.ndof, dtype=torch.float64, device="cuda",
                    generator=g)
    B[0] = b0
    for r in range(nrhs):
        M.apply_bcs(B[r])
    d = gpu.Direct(mat)
    d.factor()
    if case == "plate_c2_128":
        assert d.stats()["cluster_fronts"] > 0
    X = d.solve(B)
    for r in range(nrhs):
        assert torch.equal(X[r], d.solve(B[r].clone()))
    d32 = gpu.Direct(mat, precision=_lib.PREC_FP32)
    d32.factor()
    X32 = d32.solve(B)
    assert not d32.stats()["fell_back_to_fp64"]
    for r in range(nrhs):
        assert rel(X32[r].cpu().numpy(), X[r].cpu().numpy()) < 1e-10
        x1 = d32.solve(B[r].clone())
        assert rel(x1.cpu().numpy(), X32[r].cpu().numpy()) < 1e-13


def test_mixed_direct_forward_tolerance(gpu):
    """Refinement with the forward test (ftol): every right-hand side stops
    once a correction is at most ftol |x|, in no more steps than refinement
    to FP64 rounding, and lies within 10 ftol of the FP64 solution."""
    from tacs_gb300 import _lib, meshes
    prob = meshes.clamped_plate(24, t=0.01)
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    r0 = M.vec()
    M.assemble_jacobian(M.vec(), mat, r0)
    g = torch.Generator(device="cuda").manual_seed(3)
    B = torch.randn(4, M.ndof, dtype=torch.float64, device="cuda",
                    generator=g)
    B[0] = -r0
    for r in range(4):
        M.apply_bcs(B[r])
    d = gpu.Direct(mat)
    d.factor()
    X = d.solve(B)
    d32 = gpu.Direct(mat, precision=_lib.PREC_FP32)
    d32.factor()
    d32.solve(B)
    full = d32.stats()["last_refinement_steps"]
    for ftol in (1e-8, 1e-10):
        Xf = d32.solve(B, ftol=ftol)
        assert not d32.stats()["fell_back_to_fp64"]
        assert d32.stats()["last_refinement_steps"] <= full
        for r in range(4):
            assert rel(Xf[r].cpu().numpy(), X[r].cpu().numpy()) < 10 * ftol


def test_fp64_direct_refined_to_relative_residual(gpu):
    """An FP64 factorisation refined in FP64 (rtol) on a thin simply
    supported plate: every right-hand side ends with a residual at most
    rtol |b|, or at the FP64 floor eps sqrt(n) (|K| |u| + |b|) where rtol
    |b| lies below the rounding of K u itself (max norms; |K| |u| >> |b|
    here, as the Krylov solves' floor acceptance), and the refined
    solution stays within 1e-8 of the single solve."""
    from tacs_gb300 import meshes
    prob = meshes.plate_c2(64, 2.0 * 64 / 512, seed=2)
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    r0 = M.vec()
    M.assemble_jacobian(M.vec(), mat, r0)
    g = torch.Generator(device="cuda").manual_seed(5)
    B = torch.randn(3, M.ndof, dtype=torch.float64, device="cuda",
                    generator=g)
    B[0] = -r0
    for r in range(3):
        M.apply_bcs(B[r])
    d = gpu.Direct(mat)
    d.factor()
    X1 = d.solve(B)
    K = _host_matrix(mat, M.ndof)
    knorm = float(abs(K).sum(axis=1).max())
    floor_tol = 2.0 ** -53 * np.sqrt(M.ndof)
    for rtol in (1e-10, 1e-12):
        X = d.solve(B, rtol=rtol)
        assert d.stats()["last_refinement_steps"] >= 1
        for r in range(3):
            res = float((mat.mult(X[r]) - B[r]).abs().max())
            bn = float(B[r].abs().max())
            floor = floor_tol * (knorm * float(X[r].abs().max()) + bn)
            assert res <= max(rtol * bn, floor)
            assert rel(X[r].cpu().numpy(), X1[r].cpu().numpy()) < 1e-8


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_direct_first_factor_launches_later_ones_replay_graph(gpu, prec):
    """The first factorisation of a Direct launches its kernels directly;
    the second captures them as one CUDA graph and the later ones replay
    it.  All three give the same factor: the same solution to rounding, on
    a plate whose large fronts take panel steps."""
    from tacs_gb300 import _lib, meshes
    prob = meshes.plate_c2(128)
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    r0 = M.vec()
    M.assemble_jacobian(M.vec(), mat, r0)
    b = -r0
    d = gpu.Direct(mat, precision=(_lib.PREC_FP64 if prec == "fp64"
                                   else _lib.PREC_FP32), autotune=False)
    assert d.stats()["max_front"] > 768  # scalar rows: panel steps run
    xs = []
    for _ in range(3):
        d.factor()
        xs.append(d.solve(b).cpu().numpy())
    assert rel(xs[1], xs[0]) < 1e-12
    assert rel(xs[2], xs[0]) < 1e-12
    # normwise backward error at rounding level (a thin plate: |A| |x| is
    # far above |b|, so the residual relative to |b| is not)
    A = _host_matrix(mat, M.ndof)
    bh = b.cpu().numpy()
    eta = np.abs(A @ xs[0] - bh).max() / (
        abs(A).sum(axis=1).max() * np.abs(xs[0]).max() + np.abs(bh).max())
    assert eta < 1e-13, eta


def test_direct_autotune(gpu):
    """The solves' launch-shape autotuner (tg_direct_autotune, run at the
    second factorisation of a Direct): it times a solve per cluster
    threshold and keeps one of the candidates; another Direct of the same
    matrix shape takes the cached choice at its first factorisation without
    timing; the solution is the same to rounding whatever the threshold."""
    from tacs_gb300 import meshes
    # a shape no other test factors (the choice is cached per shape)
    prob = meshes.plate_c2(120, 0.5, seed=2)
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    r0 = M.vec()
    M.assemble_jacobian(M.vec(), mat, r0)
    b = -r0
    d = gpu.Direct(mat)
    d.factor()
    # a first factorisation solves with the default shapes; the second
    # (the factorisation reused) tunes them
    assert d.stats()["tuned"] is None
    assert d.stats()["cluster_threshold"] == 768
    d.factor()
    t = d.stats()["tuned"]
    assert t["cluster_threshold"] in t["candidates"]
    assert all(ms > 0 for ms in t["solve_ms"])
    assert d.stats()["cluster_threshold"] == t["cluster_threshold"]
    x = d.solve(b)
    d2 = gpu.Direct(mat)
    d2.factor()
    t2 = d2.stats()["tuned"]
    assert t2["cluster_threshold"] == t["cluster_threshold"]
    assert all(ms == 0 for ms in t2["solve_ms"])  # cached
    d3 = gpu.Direct(mat, autotune=False)
    d3.factor()
    assert d3.stats()["cluster_threshold"] == 768
    assert rel(x.cpu().numpy(), d3.solve(b).cpu().numpy()) < 1e-10


def test_mixed_direct_gmres_ir(gpu):
    """Where refinement with the FP32 factorisation does not reach the
    tolerance (here forced: one step allowed), the FP32 Direct solves by
    GMRES preconditioned by its own factorisation (tg_pc_create_direct,
    GMRES-IR) instead of factoring in FP64, and later solves go there
    directly; the solutions match the FP64 factorisation's to the GMRES
    tolerance, for one and for several right-hand sides."""
    from tacs_gb300 import _lib, meshes
    prob = meshes.plate_c2(64, 2.0 * 64 / 512, seed=2)
    M = gpu.GpuModel(prob)
    mat = M.new_mat()
    r0 = M.vec()
    M.assemble_jacobian(M.vec(), mat, r0)
    b = -r0
    d64 = gpu.Direct(mat)
    d64.factor()
    x64 = d64.solve(b)
    d32 = gpu.Direct(mat, precision=_lib.PREC_FP32)
    d32.factor()
    x = d32.solve(b, steps=1, rtol=1e-12)
    st = d32.stats()
    assert st["fp32_mode"] == "gmres_ir"
    assert not st["fell_back_to_fp64"] and not st["gmres_ir_fp64_factor"]
    assert st["last_gmres_iters"] >= 1
    assert rel(x.cpu().numpy(), x64.cpu().numpy()) < 1e-8
    g = torch.Generator(device="cuda").manual_seed(5)
    B = torch.randn(3, M.ndof, dtype=torch.float64, device="cuda",
                    generator=g)
    for r in range(3):
        M.apply_bcs(B[r])
    X = d32.solve(B, rtol=1e-12)  # straight to GMRES-IR: no refinement
    assert d32.stats()["last_refinement_steps"] == 0
    X64 = d64.solve(B)
    for r in range(3):
        assert rel(X[r].cpu().numpy(), X64[r].cpu().numpy()) < 1e-8
    # a new factorisation of changed values keeps the mode and refreshes
    # the preconditioner's FP32 copy of the matrix
    t2 = torch.as_tensor(1.3 * np.asarray(prob["thick"]), device="cuda")
    M.set_design_vars(t2)
    M.assemble_jacobian(M.vec(), mat, r0)
    d32.factor()
    d64.factor()
    x2 = d32.solve(b, rtol=1e-12)
    assert rel(x2.cpu().numpy(), d64.solve(b).cpu().numpy()) < 1e-8
