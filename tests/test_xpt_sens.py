"""Node-coordinate (shape) sensitivities: TACSAssembler::addXptSens and
addAdjointResXptSensProducts (src/TACSAssembler.cpp:4858,5136).

The fixtures hold the reference's complex-step values (its complex build,
dh = 1e-30, i.e. exact derivatives); the GPU kernels differentiate in dual
arithmetic, so the bar is rounding level:
  element-level dfdX and psi^T dR/dX: 1e-10 (norm-wise);
  total derivatives df/dX - psi^T dR/dX at the reference solution and
  adjoints: 1e-7 (the two terms cancel by up to 1e6);
  GPU against the central-difference oracle: 1e-7, KS 5e-6 (difference
  truncation and rounding of the oracle);
  the oracle against the fixtures (CPU): 1e-8, KS 5e-6;
  GPU total derivative against central differences of GPU static solves:
  1e-5 of the largest gradient entry.
"""
import numpy as np
import pytest

from conftest import CASES, load_case, rel

XPT_TOL = 1e-10
TOTAL_TOL = 1e-7
FD_TOL, FD_KS_TOL = 1e-7, 5e-6

XPT_CASES = [c for c in CASES if "u_test" in load_case(c)[0]]


# ------------------------------------------------------------ CPU: oracle
@pytest.mark.parametrize("name", XPT_CASES)
def test_oracle_xpt_against_reference(name):
    import oracle
    prob, ref = load_case(name)
    o = oracle.Oracle(prob)
    u = prob["u_test"]
    assert rel(o.xpt_sens(u, 0), ref["dfdX_test_comp"]) < 1e-8
    assert rel(o.xpt_sens(u, 1), ref["dfdX_test_ks"]) < FD_KS_TOL
    assert rel(o.adj_res_xpt_product(u, prob["psi_test"]),
               ref["adjxpt_test"]) < 1e-8


# ------------------------------------ CPU: the two exact derivative forms
@pytest.fixture(scope="module")
def sx(tmp_path_factory):
    """tacs_gb300/csrc/shell_xpt.cuh compiled for the host
    (tests/cpp/shell_xpt_check.cpp)."""
    import ctypes as C
    import os
    import shutil
    import subprocess
    from conftest import ROOT
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("sx") / "libsx.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "tacs_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "shell_xpt_check.cpp"),
                    "-o", out], check=True)
    lib = C.CDLL(out)
    P = C.c_void_p
    lib.sx_derivatives.argtypes = [P, P, P, P, C.c_double, P, C.c_int,
                                   C.c_int, P, P, P, P]
    lib.sx_mesh.argtypes = [C.c_int, P, P, P, P, P, P, P, C.c_int, P, P,
                            C.c_int, P]
    return lib


def _sx_elements(rng, n):
    """Random shell elements: warped squares and patches of a cylinder."""
    for k in range(n):
        if k % 2:
            X = (np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 1, 1, 0], float)
                 * rng.uniform(0.3, 3.0) + rng.normal(0, 0.15, 12))
        else:
            R, th0, dth = rng.uniform(0.5, 3), rng.uniform(0, 6), 0.3
            z0, dz = rng.uniform(-1, 1), rng.uniform(0.1, 0.5)
            X = np.array([[R * np.cos(th0 + dth * i), R * np.sin(th0 + dth * i),
                           z0 + dz * j] for j in (0, 1) for i in (0, 1)])
            X = X.ravel() + rng.normal(0, 0.01, 12)
        yield X


@pytest.mark.parametrize("transform", [0, 1])
@pytest.mark.parametrize("flags,func", [(1, -1), (3, -1), (0, 0), (0, 1),
                                        (3, 0), (1, 1)])
def test_shell_reverse_sweep_equals_dual_derivative(sx, transform, flags,
                                                    func):
    """The reverse (adjoint) sweep of shell_xpt.cuh gives the dual-number
    derivative of every coordinate to rounding (1e-12 of the largest
    entry): with and without the adjoint term (flags bit 0) and the
    pressure load (bit 1), for no function, compliance and KS failure,
    both transforms, on warped and curved elements."""
    import ctypes as C
    rng = np.random.default_rng(17 + 10 * transform + flags + 100 * (func + 1))
    P = C.c_void_p

    def ptr(a):
        return a.ctypes.data_as(P)

    for X in _sx_elements(rng, 12):
        u = rng.normal(0, 2e-4, 24)
        w = rng.normal(0, 1, 24)
        pres = rng.uniform(5e2, 2e3, 4)
        # reference axis near the element's first edge (never along its
        # normal, where the transform is undefined)
        axis = X[3:6] - X[0:3] + rng.normal(0, 0.1, 3)
        axis /= np.linalg.norm(axis)
        p = np.array([70e9, 0.3, 2.7e8, transform, *axis])
        ks = np.array([0.05, 1.3, 100.0])
        s = np.array([0.7, -1.3, 0.9])
        f, r = np.zeros(12), np.zeros(12)
        sx.sx_derivatives(ptr(p), ptr(np.ascontiguousarray(X)), ptr(u),
                          ptr(w), rng.uniform(0.002, 0.02), ptr(pres), flags,
                          func, ptr(ks), ptr(s), ptr(f), ptr(r))
        assert np.abs(f).max() > 0
        assert np.abs(f - r).max() < 1e-12 * np.abs(f).max()


@pytest.fixture(scope="module")
def hx(tmp_path_factory):
    """tacs_gb300/csrc/hex_xpt.cuh compiled for the host
    (tests/cpp/hex_xpt_check.cpp)."""
    import ctypes as C
    import os
    import shutil
    import subprocess
    from conftest import ROOT
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("hx") / "libhx.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "tacs_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "hex_xpt_check.cpp"),
                    "-o", out], check=True)
    lib = C.CDLL(out)
    P = C.c_void_p
    lib.hx_derivatives.argtypes = [P, P, P, P, C.c_double, C.c_int, C.c_int,
                                   P, P, C.c_int, P, P, P, P]
    lib.hx_mesh.argtypes = [C.c_int, P, P, P, P, P, P, P, P, P, C.c_int, P, P,
                            C.c_int, P]
    return lib


@pytest.mark.parametrize("has_psi,func", [(1, -1), (0, 0), (0, 1), (1, 0),
                                          (1, 1)])
def test_hex_reverse_sweep_equals_dual_derivative(hx, has_psi, func):
    """The hex8 reverse sweep of hex_xpt.cuh gives the dual-number
    derivative of all 24 coordinates to rounding (1e-12 of the largest
    entry), with face tractions on all six faces, on distorted bricks."""
    import ctypes as C
    rng = np.random.default_rng(5 + 3 * has_psi + 10 * (func + 1))
    P = C.c_void_p

    def ptr(a):
        return a.ctypes.data_as(P)

    cube = np.array([[(m & 1), (m >> 1) & 1, (m >> 2) & 1] for m in range(8)],
                    float)
    for _ in range(12):
        X = (cube * rng.uniform(0.2, 2.0, 3) + rng.normal(0, 0.05, (8, 3)))
        X = np.ascontiguousarray(X.ravel())
        u = rng.normal(0, 1e-4, 24)
        w = rng.normal(0, 1, 24)
        faces = np.arange(6, dtype=np.int32)
        tv = rng.normal(0, 1e4, 18)
        p = np.array([70e9, 0.3, 2.7e8])
        ks = np.array([0.05, 1.3, 100.0])
        s = np.array([0.7, -1.3, 0.9])
        f, r = np.zeros(24), np.zeros(24)
        hx.hx_derivatives(ptr(p), ptr(X), ptr(u), ptr(w),
                          rng.uniform(0.1, 1.0), has_psi, 6, ptr(faces),
                          ptr(tv), func, ptr(ks), ptr(s), ptr(f), ptr(r))
        assert np.abs(f).max() > 0
        assert np.abs(f - r).max() < 1e-12 * np.abs(f).max()


def _host_mesh_xpt(sx, hx, prob, func, psi, s, reverse):
    """The element functions of shell_xpt.cuh / hex_xpt.cuh compiled for
    the host, summed over the mesh as the kernels scatter them (loads
    staged as tg_assembler_set_pressure / _set_traction stage them)."""
    import ctypes as C
    P = C.c_void_p

    def ptr(a):
        return None if a is None else a.ctypes.data_as(P)

    ne, nn = int(prob["nelem"]), int(prob["nnodes"])
    conn = np.ascontiguousarray(prob["conn"], np.int32).ravel()
    xpts = np.ascontiguousarray(prob["xpts"], np.float64).ravel()
    thick = np.ascontiguousarray(prob["thick"], np.float64)
    _, E, nu, ys = [float(v) for v in prob["mat"]]
    u = np.ascontiguousarray(prob["u_test"], np.float64)
    w = None if psi is None else np.ascontiguousarray(psi, np.float64)
    ks = np.array([0.0, 1.0, 100.0])
    s = np.asarray(s, np.float64)
    out = np.zeros(3 * nn)
    if int(prob["elem_type"]) == 0:
        axis = np.asarray(prob.get("ref_axis", [1.0, 0.0, 0.0]), float)
        axis = axis / np.linalg.norm(axis)
        p = np.array([E, nu, ys, int(prob.get("transform", 0)), *axis])
        pres = None
        if len(prob.get("pres_elems", [])):
            pres = np.zeros(4 * ne)
            for k, e in enumerate(np.asarray(prob["pres_elems"])):
                pres[4 * e:4 * e + 4] += prob["pres_vals"][4 * k:4 * k + 4]
        sx.sx_mesh(ne, ptr(conn), ptr(xpts), ptr(thick), ptr(pres), ptr(u),
                   ptr(w), ptr(p), func, ptr(ks), ptr(s), reverse, ptr(out))
    else:
        p = np.array([E, nu, ys])
        tp = tf = tv = None
        te = np.asarray(prob.get("trac_elems", []), np.int64)
        if len(te):
            order = np.argsort(te, kind="stable")
            tp = np.zeros(ne + 1, np.int32)
            np.add.at(tp, te + 1, 1)
            tp = np.cumsum(tp).astype(np.int32)
            tf = np.asarray(prob["trac_faces"], np.int32)[order].copy()
            tv = np.asarray(prob["trac_vals"], np.float64).reshape(-1, 3)
            tv = np.ascontiguousarray(tv[order]).ravel()
        hx.hx_mesh(ne, ptr(conn), ptr(xpts), ptr(thick), ptr(tp), ptr(tf),
                   ptr(tv), ptr(u), ptr(w), ptr(p), func, ptr(ks), ptr(s),
                   reverse, ptr(out))
    return out


@pytest.mark.parametrize("reverse", [0, 1], ids=["dual", "reverse"])
@pytest.mark.parametrize("name", XPT_CASES)
def test_host_element_derivatives_against_reference(sx, hx, name, reverse):
    """The element derivative code the GPU kernels run, compiled for the
    host: the compliance derivative and psi^T dR/dX summed over the mesh
    equal the reference's complex-step values (1e-10), in both forms."""
    prob, ref = load_case(name)
    dc = _host_mesh_xpt(sx, hx, prob, 0, None, (1.0, 0.0, 0.0), reverse)
    assert rel(dc, ref["dfdX_test_comp"]) < XPT_TOL
    xa = _host_mesh_xpt(sx, hx, prob, -1, prob["psi_test"], (0.0, 1.0, 1.0),
                        reverse)
    assert rel(xa, ref["adjxpt_test"]) < XPT_TOL


# ------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import problem
    return problem


def _h(t):
    return t.detach().cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("name", XPT_CASES)
def test_xpt_element_level(gpu, name):
    prob, ref = load_case(name)
    M = gpu.GpuModel(prob)
    u = M.vec(prob["u_test"])
    M.eval_functions(u)
    dc, dk = M.node_vec(), M.node_vec()
    M.add_xpt_sens(u, [0, 1], [dc, dk])
    assert rel(_h(dc), ref["dfdX_test_comp"]) < XPT_TOL
    assert rel(_h(dk), ref["dfdX_test_ks"]) < XPT_TOL
    xa = M.node_vec()
    M.add_adjoint_res_xpt_products(u, [M.vec(prob["psi_test"])], [xa])
    assert rel(_h(xa), ref["adjxpt_test"]) < XPT_TOL
    # coefficients scale linearly, contributions add
    xb = M.node_vec()
    M.add_adjoint_res_xpt_products(u, [M.vec(prob["psi_test"])], [xb],
                                   scale=-2.0)
    M.add_xpt_sens(u, [0], [xb], coef=3.0)
    expect = 3.0 * ref["dfdX_test_comp"] - 2.0 * ref["adjxpt_test"]
    assert rel(_h(xb), expect) < XPT_TOL


@pytest.mark.gpu
@pytest.mark.late
@pytest.mark.parametrize("name", XPT_CASES)
def test_reverse_kernel_matches_reference(gpu, name):
    """The reverse-sweep kernels (tg_set_xpt_mode TG_XPT_REVERSE, shell and
    hex): the reference's complex-step values at element level (1e-10) and
    the forward kernels' results (1e-12)."""
    prob, ref = load_case(name)
    M = gpu.GpuModel(prob)
    u = M.vec(prob["u_test"])
    M.eval_functions(u)
    psi = M.vec(prob["psi_test"])
    out = {}
    for reverse in (False, True):
        M.set_xpt_mode(reverse)
        dc, dk, xa = M.node_vec(), M.node_vec(), M.node_vec()
        M.add_xpt_sens(u, [0, 1], [dc, dk])
        M.add_adjoint_res_xpt_products(u, [psi], [xa])
        out[reverse] = [_h(dc), _h(dk), _h(xa)]
    M.set_xpt_mode(True)
    for got, key in zip(out[True], ("dfdX_test_comp", "dfdX_test_ks",
                                    "adjxpt_test")):
        assert rel(got, ref[key]) < XPT_TOL
    for a, b in zip(out[True], out[False]):
        assert rel(a, b) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_xpt_total_at_reference_solution(gpu, name):
    prob, ref = load_case(name)
    M = gpu.GpuModel(prob)
    u = M.vec(ref["u"])
    M.eval_functions(u)
    for fn, key in ((0, "comp"), (1, "ks")):
        g = M.node_vec()
        M.add_total_xpt_derivative(u, fn, M.vec(ref["psi_" + key]), g,
                                   1.0, -1.0)
        assert rel(_h(g), ref["grad_xpt_" + key]) < TOTAL_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["shell", "hex"])
def test_xpt_against_oracle(gpu, kind):
    import oracle
    from tacs_gb300 import meshes
    if kind == "shell":
        prob = meshes.clamped_plate(12)
        prob["xpts"] = prob["xpts"].copy()
        rng = np.random.default_rng(11)
        prob["xpts"][2::3] += 0.01 * rng.standard_normal(prob["nnodes"])
    else:
        prob = meshes.hex_c3(8, 8, 4, traction=-1e6, half=0.3)
    rng = np.random.default_rng(5)
    vpn = 6 if prob["elem_type"] == meshes.SHELL else 3
    n = vpn * prob["nnodes"]
    u = 1e-3 * rng.standard_normal(n)
    psi = rng.standard_normal(n)
    o = oracle.Oracle(prob)
    M = gpu.GpuModel(prob)
    uu = M.vec(u)
    M.eval_functions(uu)
    dc, dk, xa = M.node_vec(), M.node_vec(), M.node_vec()
    M.add_xpt_sens(uu, [0, 1], [dc, dk])
    M.add_adjoint_res_xpt_products(uu, [M.vec(psi)], [xa], lam=0.5)
    assert rel(_h(dc), o.xpt_sens(u, 0)) < FD_TOL
    assert rel(_h(dk), o.xpt_sens(u, 1)) < FD_KS_TOL
    assert rel(_h(xa), o.adj_res_xpt_product(u, psi, lam=0.5)) < FD_TOL


@pytest.mark.gpu
def test_shape_derivative_against_solves(gpu):
    """d f/dX of a clamped plate under pressure, from one adjoint solve,
    against central differences of two full GPU static solves per
    coordinate."""
    import torch
    from tacs_gb300 import meshes
    prob = meshes.clamped_plate(8)
    M = gpu.GpuModel(prob)
    r = gpu.static_adjoint(M, prob["force"], 100, 4, 1e-13)
    assert r["flag"] == 1
    grads = []
    for k in range(2):
        g = M.node_vec()
        M.add_total_xpt_derivative(r["u"], k, r["psis"][k], g, 1.0, -1.0)
        grads.append(_h(g))
    x0 = torch.as_tensor(prob["xpts"], device="cuda").clone()
    h = 1e-5
    for node, d in ((30, 0), (40, 1), (22, 0)):
        j = 3 * node + d
        fvals = []
        for sgn in (1.0, -1.0):
            x = x0.clone()
            x[j] += sgn * h
            M.set_nodes(x)
            rr = gpu.static_adjoint(M, prob["force"], 100, 4, 1e-13)
            fvals.append(rr["funcs"])
        M.set_nodes(x0)
        fd = (fvals[0] - fvals[1]) / (2 * h)
        for k in range(2):
            err = abs(fd[k] - grads[k][j]) / np.abs(grads[k]).max()
            assert err < 1e-5, (node, d, k, fd[k], grads[k][j])


def test_element_derivatives_in_bounds_under_sanitizers(tmp_path):
    """The element derivative code the kernels run (both forms, shell and
    hex) makes no out-of-bounds access and no undefined operation: the
    host checks above, with the check libraries built with
    AddressSanitizer and UndefinedBehaviorSanitizer (any finding aborts),
    run in a child process that preloads the sanitizer runtimes."""
    import os
    import shutil
    import subprocess
    import sys
    from conftest import ROOT
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    rt = [subprocess.run([cxx, f"-print-file-name={lib}"], capture_output=True,
                         text=True).stdout.strip()
          for lib in ("libasan.so", "libubsan.so")]
    if not all(os.path.isabs(p) and os.path.exists(p) for p in rt):
        pytest.skip("sanitizer runtimes not found")
    libs = {}
    for name in ("shell_xpt_check", "hex_xpt_check"):
        out = str(tmp_path / f"lib{name}.so")
        r = subprocess.run([cxx, "-O1", "-g", "-std=c++17",
                            "-fsanitize=address,undefined",
                            "-fno-sanitize-recover=all", "-shared", "-fPIC",
                            "-I", os.path.join(ROOT, "tacs_gb300", "csrc"),
                            os.path.join(ROOT, "tests", "cpp", name + ".cpp"),
                            "-o", out], capture_output=True, text=True)
        if r.returncode:
            pytest.skip("sanitizer build failed: " + r.stderr[-200:])
        libs[name] = out
    child = f"""
import ctypes as C, sys
sys.path[:0] = [{os.path.join(ROOT, "tests")!r}, {ROOT!r}]
import test_xpt_sens as T
P = C.c_void_p
sx = C.CDLL({libs["shell_xpt_check"]!r})
sx.sx_derivatives.argtypes = [P, P, P, P, C.c_double, P, C.c_int, C.c_int,
                              P, P, P, P]
sx.sx_mesh.argtypes = [C.c_int, P, P, P, P, P, P, P, C.c_int, P, P, C.c_int,
                       P]
hx = C.CDLL({libs["hex_xpt_check"]!r})
hx.hx_derivatives.argtypes = [P, P, P, P, C.c_double, C.c_int, C.c_int, P, P,
                              C.c_int, P, P, P, P]
hx.hx_mesh.argtypes = [C.c_int, P, P, P, P, P, P, P, P, P, C.c_int, P, P,
                       C.c_int, P]
n = 0
for tr in (0, 1):
    for flags, func in [(1, -1), (3, -1), (0, 0), (0, 1), (3, 0), (1, 1)]:
        T.test_shell_reverse_sweep_equals_dual_derivative(sx, tr, flags,
                                                          func)
        n += 1
for hp, func in [(1, -1), (0, 0), (0, 1), (1, 0), (1, 1)]:
    T.test_hex_reverse_sweep_equals_dual_derivative(hx, hp, func)
    n += 1
for name in T.XPT_CASES:
    for rev in (0, 1):
        T.test_host_element_derivatives_against_reference(sx, hx, name, rev)
        n += 1
print("checked", n)
"""
    env = dict(os.environ, LD_PRELOAD=":".join(rt),
               ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([sys.executable, "-c", child], capture_output=True,
                       text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "checked 33" in r.stdout
