"""torch.autograd.Function over the GPU solve -> functional path.

* gradients against the reference's own adjoint gradients (the golden
  fixtures, tests/golden/make_golden.py) at the solver tolerance, 1e-7;
* gradients against central finite differences of the forward functional
  (h = 1e-4 x, error 1e-5 of the largest gradient entry: the h^2 truncation
  of a t^-3-like functional is ~1e-8 relative, while the functional's
  rounding through a 1e-12 GMRES solve, ~1e-10 relative, divided by h stays
  below 1e-5; with h = 1e-6 x that rounding term alone reaches ~1e-3);
* SIMP-style chaining (x -> x^3 in torch) through autograd;
* node-coordinate gradients against the reference's complex-step shape
  derivative and against central differences along a shape mode;
* several load cases and several meshes in one functional call against the
  batched adjoint gradients.
"""
import numpy as np
import pytest

from conftest import load_case, rel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-7
FD_TOL = 1e-5


@pytest.fixture(scope="module")
def gpu():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import autograd, problem
    return problem, autograd


def _dv_vector(prob, ndv):
    x = np.zeros(ndv)
    x[np.asarray(prob["dvnum"])] = prob["thick"]
    return torch.as_tensor(x, device="cuda")


@pytest.mark.parametrize("name", ["shell_plate8", "shell_cyl", "hex_block",
                                  "shell_c1"])
@pytest.mark.parametrize("func", [0, 1])
def test_autograd_matches_reference_adjoint(gpu, name, func):
    problem, ag = gpu
    prob, ref = load_case(name)
    M = problem.GpuModel(prob)
    solver = ag.StaticSolver(M, prob["force"], m=prob.get("gmres_m", 100),
                             nrestart=50, rtol=prob.get("rtol", 1e-12))
    x = _dv_vector(prob, M.ndv).requires_grad_(True)
    f = ag.static_functional(x, solver, func)
    assert abs(f.item() - ref["funcs"][func]) < TOL * abs(ref["funcs"][func])
    f.sum().backward()
    g_ref = ref["grad_comp"] if func == 0 else ref["grad_ks"]
    assert rel(x.grad.cpu().numpy(), g_ref) < TOL


@pytest.mark.parametrize("func", [0, 1])
def test_autograd_central_differences(gpu, func):
    problem, ag = gpu
    from tacs_gb300 import meshes
    rng = np.random.default_rng(11)
    p = meshes.clamped_plate(8, thick=rng.uniform(0.005, 0.02, 64))
    M = problem.GpuModel(p)
    solver = ag.StaticSolver(M, np.zeros(M.ndof), m=80, nrestart=50,
                             rtol=1e-12)
    x0 = torch.as_tensor(p["thick"], device="cuda")
    x = x0.clone().requires_grad_(True)
    f = ag.static_functional(x, solver, func)
    f.sum().backward()
    g = x.grad.cpu().numpy()
    for d in rng.choice(64, 6, replace=False):
        h = 1e-4 * float(x0[d])
        xp, xm = x0.clone(), x0.clone()
        xp[d] += h
        xm[d] -= h
        fp = ag.static_functional(xp, solver, func).item()
        fm = ag.static_functional(xm, solver, func).item()
        fd = (fp - fm) / (2 * h)
        assert abs(fd - g[d]) <= FD_TOL * np.abs(g).max(), (d, fd, g[d])


@pytest.mark.parametrize("name", ["shell_plate8", "hex_block"])
def test_autograd_node_coordinates(gpu, name):
    """Gradient with respect to the node coordinates: against the
    reference's complex-step total shape derivative (1e-7), and, for a
    torch-side parametrisation X(s) = X0 + s V, against central differences
    of the functional in s."""
    problem, ag = gpu
    prob, ref = load_case(name)
    M = problem.GpuModel(prob)
    solver = ag.StaticSolver(M, prob["force"], m=prob.get("gmres_m", 100),
                             nrestart=50, rtol=prob.get("rtol", 1e-12))
    x = _dv_vector(prob, M.ndv)
    X0 = torch.as_tensor(prob["xpts"], device="cuda")
    X = X0.clone().requires_grad_(True)
    f = ag.static_functional(x, solver, 0, xpts=X)
    f.sum().backward()
    assert rel(X.grad.cpu().numpy(), ref["grad_xpt_comp"]) < TOL
    # a smooth shape mode: in-plane (x) bulge of the interior
    V = torch.zeros_like(X0).reshape(-1, 3)
    P = X0.reshape(-1, 3)
    V[:, 0] = torch.sin(np.pi * P[:, 0] / P[:, 0].max()) * \
        torch.sin(np.pi * P[:, 1] / P[:, 1].max())
    V = V.reshape(-1)
    s = torch.zeros((), dtype=torch.float64, device="cuda",
                    requires_grad=True)
    f = ag.static_functional(x, solver, 0, xpts=X0 + s * V)
    (dfds,) = torch.autograd.grad(f.sum(), s)
    h = 1e-5
    fp = ag.static_functional(x, solver, 0, xpts=X0 + h * V).item()
    fm = ag.static_functional(x, solver, 0, xpts=X0 - h * V).item()
    fd = (fp - fm) / (2 * h)
    assert abs(fd - dfds.item()) < FD_TOL * abs(dfds.item()) + 1e-12


def test_autograd_simp_chain_rule(gpu):
    """t = rho^3 on a hex block: d f / d rho = 3 rho^2 d f / d t."""
    problem, ag = gpu
    from tacs_gb300 import meshes
    rng = np.random.default_rng(3)
    p = meshes.hex_block(4, 3, 2)
    face = np.where(p["xpts"].reshape(-1, 3)[:, 0] == 0.0)[0]
    p["bc_nodes"] = face.astype(np.int32)
    p["bc_masks"] = np.full(len(face), 7, np.int32)
    f = np.zeros(3 * p["nnodes"])
    tip = np.where(p["xpts"].reshape(-1, 3)[:, 0] == 2.0)[0]
    f[3 * tip + 2] = -1e4
    M = problem.GpuModel(p)
    solver = ag.StaticSolver(M, f, m=100, nrestart=50, rtol=1e-13)
    rho = torch.as_tensor(rng.uniform(0.1, 1.0, M.ndv),
                          device="cuda").requires_grad_(True)
    c = ag.static_functional(rho ** 3, solver, 0)
    c.sum().backward()
    t = (rho.detach() ** 3).requires_grad_(True)
    c2 = ag.static_functional(t, solver, 0)
    c2.sum().backward()
    expect = 3 * rho.detach() ** 2 * t.grad
    assert rel(rho.grad.cpu().numpy(), expect.cpu().numpy()) < 1e-12


def test_autograd_batched_load_cases_and_meshes(gpu):
    problem, ag = gpu
    from tacs_gb300 import _lib, meshes
    bp = meshes.batch_plates(count=3, seed=4, nmin=6, nmax=12)
    M = problem.GpuModel(bp)
    F = problem.batch_loads(M)
    ref = problem.batched_adjoint(M, F, m=1000, nrestart=2, rtol=1e-12,
                                  func=_lib.FUNC_KS_FAILURE)
    # the element pressure is already in F[0]: no element loads on top
    solver = ag.StaticSolver(M, F, m=1000, nrestart=2, rtol=1e-12,
                             include_element_loads=False, segments=True)
    x = torch.as_tensor(bp["thick"], device="cuda").requires_grad_(True)
    f = ag.static_functional(x, solver, _lib.FUNC_KS_FAILURE)
    assert rel(f.detach().cpu().numpy(), ref["funcs"]) < TOL
    w = torch.as_tensor(np.random.default_rng(5).standard_normal(f.shape),
                        device="cuda")
    (f * w).sum().backward()
    expect = (w.cpu().numpy()[:, :, None] *
              np.stack([[np.where((np.arange(M.nelem) >= bp["seg_elem_ptr"][g])
                                  & (np.arange(M.nelem) < bp["seg_elem_ptr"][g + 1]),
                                  ref["grads"][lc].cpu().numpy(), 0.0)
                         for g in range(3)] for lc in range(F.shape[0])])
              ).sum(axis=(0, 1))
    assert rel(x.grad.cpu().numpy(), expect) < TOL


def test_autograd_hex_simp_central_differences(gpu):
    """The hex8 SIMP workload's form (density rho, E rho^3, x = 0 face
    clamped, traction patch on x = 2) at 8 x 4 x 2 elements: d compliance /
    d rho from the adjoint backward against central differences with
    h = 1e-6 on 32 seeded elements.  Tolerance 5e-5 of the largest entry:
    the forward solves reach ~1e-13 relative, and that rounding over 2h is
    ~1e-7 of the compliance, ~1e-6 of a per-element gradient here."""
    problem, ag = gpu
    from tacs_gb300 import meshes
    p = meshes.hex_c3(8, 4, 2, seed=3, half=0.5)
    M = problem.GpuModel(p)
    solver = ag.StaticSolver(M, np.zeros(M.ndof), m=200, nrestart=20,
                             rtol=1e-14)
    rho0 = torch.as_tensor(p["rho"], device="cuda")
    rho = rho0.clone().requires_grad_(True)
    c = ag.static_functional(rho ** 3, solver, 0)
    c.sum().backward()
    g = rho.grad.cpu().numpy()
    rng = np.random.default_rng(33)
    h = 1e-6
    for e in rng.choice(M.nelem, 32, replace=False):
        rp, rm = rho0.clone(), rho0.clone()
        rp[e] += h
        rm[e] -= h
        fp = ag.static_functional(rp ** 3, solver, 0).item()
        fm = ag.static_functional(rm ** 3, solver, 0).item()
        fd = (fp - fm) / (2 * h)
        assert abs(fd - g[e]) <= 5e-5 * np.abs(g).max(), (e, fd, g[e])
