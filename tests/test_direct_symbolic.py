"""Host analysis of the direct factorisation (tacs_gb300/csrc/direct_symbolic.h:
nested-dissection order, elimination tree, fundamental supernodes, fronts,
extend-add and assembly maps), checked on the CPU: a dense multifrontal
block Cholesky driven by the analysis (tests/cpp/direct_check.cpp) must
solve the assembled stiffness matrices to rounding (backward error 1e-14
of |K| |x|, and within 1e-5 of a sparse LU solve: cond(K) x eps, with
SIMP densities down to 1e-3 in the solid case), for
shells, solids, a closed cylinder and independent
meshes in one matrix; the order must be a permutation, and the nested
dissection must fill less than the natural order."""
import ctypes as C
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, load_case, rel

SRC = os.path.join(ROOT, "tests", "cpp", "direct_check.cpp")
INC = os.path.join(ROOT, "tacs_gb300", "csrc")


@pytest.fixture(scope="module")
def dc(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("dc") / "libdc.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-shared", "-fPIC",
                    "-I", INC, SRC, "-o", out], check=True)
    lib = C.CDLL(out)
    P = C.c_void_p
    lib.dc_analyse.argtypes = [C.c_int, P, P, P, C.c_int, C.c_int, P, P]
    lib.dc_solve.argtypes = [C.c_int, C.c_int, P, P, P, P, P, C.c_int, P]
    lib.dc_plan.argtypes = [C.c_int, P, P, C.c_int, P, P]
    lib.dc_nd.argtypes = [C.c_int, P, P, C.c_int, P, C.c_int, P]
    return lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _matrix(prob):
    import oracle
    o = oracle.Oracle(prob)
    _, A = o.assemble_jac(np.zeros(o.ndof))
    n, bs = A.nrows, A.bsize
    nnz = A.rowp[n]
    rowp = np.ctypeslib.as_array(A.rowp, (n + 1,)).astype(np.int32).copy()
    cols = np.ctypeslib.as_array(A.cols, (nnz,)).astype(np.int32).copy()
    vals = np.ctypeslib.as_array(A.vals, (nnz * bs * bs,)).copy()
    o.free(A)
    return n, bs, rowp, cols, vals


def _problems():
    from tacs_gb300 import meshes
    rng = np.random.default_rng(9)
    yield "plate 16", meshes.clamped_plate(16, thick=rng.uniform(0.004, 0.02,
                                                                 256))
    yield "plate 24 thin", meshes.clamped_plate(24, t=0.002)
    yield "hex 6x5x4", meshes.hex_c3(6, 5, 4)
    yield "cylinder", load_case("shell_cyl")[0]
    yield "4 plates", meshes.batch_plates(count=4, nmin=6, nmax=20)
    yield "separate shells", load_case("shell_rand")[0]
    yield "separate solids", load_case("hex_rand")[0]


@pytest.mark.parametrize("name,prob", list(_problems()),
                         ids=[p[0] for p in _problems()])
@pytest.mark.parametrize("leaf,coords", [(1, False), (8, False),
                                         (64, False), (8, True)])
def test_multifrontal_solve_is_exact(dc, name, prob, leaf, coords):
    """The assembled K carries the reference's row boundary conditions
    (identity rows, columns kept): K = [[K_ff, K_fb], [0, I]].  Its
    symmetric part Kt = K_ff + I (boundary columns zeroed too) is what the
    Cholesky factors; K x = b is then x = Kt^-1 (b - (K - Kt) b)."""
    from scipy import sparse
    from scipy.sparse.linalg import spsolve
    n, bs, rowp, cols, vals = _matrix(prob)
    K = sparse.bsr_matrix((vals.reshape(-1, bs, bs), cols, rowp),
                          shape=(n * bs, n * bs)).tocsr()
    K.eliminate_zeros()
    d = K.diagonal()
    bc = np.flatnonzero((np.diff(K.indptr) == 1) & (d == 1.0))
    keep = np.ones(n * bs)
    keep[bc] = 0.0
    E = K @ sparse.diags(1.0 - keep) - sparse.diags(1.0 - keep)
    Kt = K - E
    assert abs(Kt - Kt.T).max() <= 1e-9 * abs(Kt).max()
    # Kt's values in K's block pattern (zeroed blocks stay stored)
    vals_t = np.zeros_like(vals).reshape(-1, bs, bs)
    Ktd = Kt.tolil()
    for i in range(n):
        for j in range(rowp[i], rowp[i + 1]):
            r0, c0 = bs * i, bs * cols[j]
            vals_t[j] = Ktd[r0:r0 + bs, c0:c0 + bs].toarray()
    b = np.random.default_rng(1).standard_normal(n * bs)
    x = np.zeros_like(b)
    bb = b - E @ b
    xyz = np.ascontiguousarray(prob["xpts"], np.float64) if coords else None
    rc = dc.dc_solve(n, bs, _ptr(rowp), _ptr(cols), _ptr(vals_t.ravel()),
                     _ptr(bb), _ptr(x), leaf, _ptr(xyz))
    assert rc == 0
    # backward error at rounding level; forward error within cond(K) x eps
    # of the sparse LU's
    Kinf = abs(K).sum(axis=1).max()
    assert np.abs(K @ x - b).max() < 1e-14 * Kinf * np.abs(x).max()
    assert rel(x, spsolve(K.tocsc(), b)) < 1e-5


def _pattern(prob):
    """Block pattern (every node coupled with the nodes of its elements)
    and node coordinates of a mesh, without assembling it."""
    from scipy import sparse
    conn = np.asarray(prob["conn"]).reshape(prob["nelem"], -1)
    n, k = prob["nnodes"], conn.shape[1]
    A = sparse.csr_matrix((np.ones(conn.size * k),
                           (np.repeat(conn, k, axis=1).ravel(),
                            np.tile(conn, (1, k)).ravel())), shape=(n, n))
    A.sum_duplicates()
    A.sort_indices()
    return (n, A.indptr.astype(np.int32), A.indices.astype(np.int32),
            np.ascontiguousarray(prob["xpts"], np.float64))


def _nd_cases():
    from tacs_gb300 import meshes
    yield "plate 200", meshes.plate_c2(200)
    yield "cylinder 192x96", meshes.cylinder_c5(192, 96)
    yield "hex 32x32x16", meshes.hex_c3(32, 32, 16)
    yield "8 plates", meshes.batch_plates(count=8, nmin=60, nmax=90)


@pytest.mark.parametrize("name,prob", list(_nd_cases()),
                         ids=[p[0] for p in _nd_cases()])
def test_nested_dissection_order_independent_of_threads(dc, name, prob):
    """The two sides of each cut at the top of the recursion are ordered on
    two threads; the order is the sequential one for every thread count,
    by coordinates and by level structures."""
    n, rowp, cols, xyz = _pattern(prob)
    for coords in (xyz, None):
        ref = np.zeros(n, np.int32)
        assert dc.dc_nd(n, _ptr(rowp), _ptr(cols), 64, _ptr(coords), 1,
                        _ptr(ref)) == 0
        assert np.array_equal(np.sort(ref), np.arange(n))
        for threads in (2, 3, 8, 16):
            p = np.zeros(n, np.int32)
            assert dc.dc_nd(n, _ptr(rowp), _ptr(cols), 64, _ptr(coords),
                            threads, _ptr(p)) == 0
            assert np.array_equal(p, ref), (threads, coords is None)


def test_nested_dissection_threads_race_free(tmp_path):
    """ThreadSanitizer finds no data race in the threaded nested dissection
    (16 threads, by coordinates and by level structures; one plate, and
    separate plates ordered on threads side by side)."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    tsan = subprocess.run([cxx, "-print-file-name=libtsan.so"],
                          capture_output=True, text=True).stdout.strip()
    if not os.path.isabs(tsan):
        pytest.skip("ThreadSanitizer runtime unavailable")
    lib = str(tmp_path / "libdc_tsan.so")
    r = subprocess.run([cxx, "-O1", "-g", "-std=c++17", "-pthread",
                        "-fsanitize=thread", "-shared", "-fPIC", "-I", INC,
                        SRC, "-o", lib], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("ThreadSanitizer build failed: " + r.stderr[-200:])
    from tacs_gb300 import meshes
    files = []
    for k, prob in enumerate((meshes.plate_c2(160),
                              meshes.batch_plates(count=6, nmin=40,
                                                  nmax=60))):
        n, rowp, cols, xyz = _pattern(prob)
        files.append(str(tmp_path / f"pat{k}.npz"))
        np.savez(files[-1], rowp=rowp, cols=cols, xyz=xyz)
    code = f"""
import ctypes as C, numpy as np
lib = C.CDLL({lib!r})
P = C.c_void_p
lib.dc_nd.argtypes = [C.c_int, P, P, C.c_int, P, C.c_int, P]
for f in {files!r}:
    d = np.load(f)
    rowp, cols, xyz = d["rowp"], d["cols"], d["xyz"]
    n = len(rowp) - 1
    for coords in (xyz, None):
        p = np.zeros(n, np.int32)
        cp = coords.ctypes.data_as(P) if coords is not None else None
        assert lib.dc_nd(n, rowp.ctypes.data_as(P), cols.ctypes.data_as(P),
                         64, cp, 16, p.ctypes.data_as(P)) == 0
        assert np.array_equal(np.sort(p), np.arange(n))
print("ok")
"""
    env = dict(os.environ, LD_PRELOAD=tsan,
               TSAN_OPTIONS="halt_on_error=1 exitcode=66 "
                            "report_signal_unsafe=0")
    r = subprocess.run([sys.executable, "-c", code], env=env,
                       capture_output=True, text=True, timeout=600)
    assert "ThreadSanitizer" not in r.stderr, r.stderr[-3000:]
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]


def test_nested_dissection_fills_less(dc):
    from tacs_gb300 import meshes
    n, bs, rowp, cols, vals = _matrix(meshes.clamped_plate(96))
    nd, nat = np.zeros(5), np.zeros(5)
    assert dc.dc_analyse(n, _ptr(rowp), _ptr(cols), None, 64, bs, None,
                         _ptr(nd)) == 0
    ident = np.arange(n, dtype=np.int32)
    assert dc.dc_analyse(n, _ptr(rowp), _ptr(cols), _ptr(ident), 64, bs,
                         None, _ptr(nat)) == 0
    # factor blocks and flops
    assert nd[2] < 0.5 * nat[2]
    assert nd[4] < 0.3 * nat[4]
    # the natural order of a plate is one chain: few, wide supernodes but
    # as many tree levels as supernodes; dissection gives a shallow tree
    assert nd[1] < nat[1]


@pytest.mark.parametrize("name,prob", list(_problems()),
                         ids=[p[0] for p in _problems()])
def test_storage_plan_has_no_overlap(dc, name, prob):
    """Update matrices live from their supernode's level to their parent's:
    no two live at the same level may share pool blocks, and the pool is
    no larger than needed by more than the first-fit slack (2x the busiest
    level)."""
    n, bs, rowp, cols, vals = _matrix(prob)
    out = np.zeros(4)
    assert dc.dc_plan(n, _ptr(rowp), _ptr(cols), 8, None, _ptr(out)) == 0
    l_total, peak, busiest, bad = out
    assert bad == 0
    assert busiest <= peak <= 2 * busiest + 1


# ------------------------------------------------------------------------
# The GPU kernels of the numeric phase, run on the CPU (one thread per CTA,
# tests/cpp/direct_emul.cpp) through the launch sequence of tg_direct.cu,
# on the assembled matrices with their row boundary conditions.
EMUL = os.path.join(ROOT, "tests", "cpp", "direct_emul.cpp")


@pytest.fixture(scope="module")
def de(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("de") / "libde.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-shared", "-fPIC",
                    "-I", INC, EMUL, "-o", out], check=True)
    lib = C.CDLL(out)
    P = C.c_void_p
    lib.de_solve.argtypes = [C.c_int, C.c_int, P, P, P, P, P, C.c_int,
                             C.c_int, P, P]
    lib.de_solve_multi.argtypes = [C.c_int, C.c_int, P, P, P, P, P, C.c_int,
                                   C.c_int, C.c_int, P, P]
    return lib


def _bcmask(prob):
    m = np.zeros(int(prob["nnodes"]), np.int32)
    for node, mask in zip(prob["bc_nodes"], prob["bc_masks"]):
        m[int(node)] |= int(mask)
    return m


@pytest.mark.parametrize("name,prob", list(_problems()),
                         ids=[p[0] for p in _problems()])
@pytest.mark.parametrize("small_max,coords", [(256, True), (512, True),
                                              (0, True), (1 << 30, False)])
def test_gpu_kernels_on_cpu_solve_assembled_system(de, name, prob, small_max,
                                                   coords):
    """small_max 0 sends every front through the panel + trailing-tile
    path, 1 << 30 every front through the one-CTA kernel."""
    from scipy import sparse
    from scipy.sparse.linalg import spsolve
    n, bs, rowp, cols, vals = _matrix(prob)
    K = sparse.bsr_matrix((vals.reshape(-1, bs, bs), cols, rowp),
                          shape=(n * bs, n * bs)).tocsr()
    b = np.random.default_rng(2).standard_normal(n * bs)
    x = np.zeros_like(b)
    xyz = np.ascontiguousarray(prob["xpts"], np.float64) if coords else None
    rc = de.de_solve(n, bs, _ptr(rowp), _ptr(cols), _ptr(vals),
                     _ptr(_bcmask(prob)), _ptr(xyz), small_max, 0, _ptr(b),
                     _ptr(x))
    assert rc == 0
    Kinf = abs(K).sum(axis=1).max()
    assert np.abs(K @ x - b).max() < 1e-14 * Kinf * np.abs(x).max()
    assert rel(x, spsolve(K.tocsc(), b)) < 1e-5


def _random_spd(n, bs, deg, seed):
    """A random symmetric block pattern (random geometric graph in 3D plus
    a few long-range edges) with symmetric positive definite values."""
    rng = np.random.default_rng(seed)
    xyz = rng.random((n, 3))
    rows = [set([i]) for i in range(n)]
    order = np.argsort(xyz[:, 0])
    for k, i in enumerate(order):
        for j in order[k + 1:k + 1 + deg]:
            if rng.random() < 0.6:
                rows[i].add(int(j))
                rows[int(j)].add(int(i))
    for _ in range(n // 10):
        i, j = rng.integers(0, n, 2)
        rows[i].add(int(j))
        rows[j].add(int(i))
    rowp = np.zeros(n + 1, np.int32)
    cols = []
    for i in range(n):
        c = sorted(rows[i])
        cols += c
        rowp[i + 1] = len(cols)
    cols = np.array(cols, np.int32)
    vals = np.zeros((len(cols), bs, bs))
    for i in range(n):
        for k in range(rowp[i], rowp[i + 1]):
            j = cols[k]
            if j > i:
                blk = rng.standard_normal((bs, bs))
                vals[k] = blk
                kk = rowp[j] + np.searchsorted(cols[rowp[j]:rowp[j + 1]], i)
                vals[kk] = blk.T
    for i in range(n):  # diagonal dominance
        k = rowp[i] + np.searchsorted(cols[rowp[i]:rowp[i + 1]], i)
        s = np.abs(vals[rowp[i]:rowp[i + 1]]).sum() + 1.0
        g = rng.standard_normal((bs, bs))
        vals[k] = s * np.eye(bs) + 0.1 * (g + g.T)
    return rowp, cols, vals.ravel(), xyz.ravel().copy()


@pytest.mark.parametrize("n,bs,deg,seed", [(200, 3, 6, 1), (300, 6, 10, 2),
                                           (500, 2, 20, 3), (64, 1, 40, 4)])
@pytest.mark.parametrize("small_max,coords", [(256, True), (0, True),
                                              (1 << 30, False)])
def test_gpu_kernels_on_cpu_random_spd(de, n, bs, deg, seed, small_max,
                                       coords):
    """Random patterns (uneven degrees, long-range couplings, many
    children per supernode) beyond the finite-element meshes."""
    from scipy import sparse
    rowp, cols, vals, xyz = _random_spd(n, bs, deg, seed)
    K = sparse.bsr_matrix((vals.reshape(-1, bs, bs), cols, rowp),
                          shape=(n * bs, n * bs)).tocsr()
    b = np.random.default_rng(seed).standard_normal(n * bs)
    x = np.zeros_like(b)
    rc = de.de_solve(n, bs, _ptr(rowp), _ptr(cols), _ptr(vals),
                     _ptr(np.zeros(n, np.int32)),
                     _ptr(xyz if coords else None), small_max, 0, _ptr(b),
                     _ptr(x))
    assert rc == 0
    assert rel(K @ x, b) < 1e-12



@pytest.mark.parametrize("name,prob", list(_problems())[:4],
                         ids=[p[0] for p in _problems()][:4])
@pytest.mark.parametrize("small_max", [256, 0])
def test_gpu_kernels_on_cpu_fp32_factor(de, name, prob, small_max):
    """The FP32 factorisation: one FP32 solve is backward stable at FP32
    level (|K x - b| <= 1e-5 |K| |x|), and iterative refinement with FP64
    residuals and FP32 corrections reaches the FP64 solution (1e-10, and
    the backward error of FP64, 1e-14 |K| |x|) within 6 steps.  The plain
    relative residual cannot show this: these matrices have |K| |x| up to
    1e9 |b|."""
    from scipy import sparse
    n, bs, rowp, cols, vals = _matrix(prob)
    K = sparse.bsr_matrix((vals.reshape(-1, bs, bs), cols, rowp),
                          shape=(n * bs, n * bs)).tocsr()
    b = np.random.default_rng(5).standard_normal(n * bs)
    xyz = np.ascontiguousarray(prob["xpts"], np.float64)
    mask = _bcmask(prob)

    def solve(r, prec):
        r = np.ascontiguousarray(r, np.float64)
        y = np.zeros_like(r)
        assert de.de_solve(n, bs, _ptr(rowp), _ptr(cols), _ptr(vals),
                           _ptr(mask), _ptr(xyz), small_max, prec, _ptr(r),
                           _ptr(y)) == 0
        return y

    Kinf = abs(K).sum(axis=1).max()

    def eta(x):
        return np.abs(K @ x - b).max() / (Kinf * np.abs(x).max())

    x = solve(b, 1)
    assert eta(x) < 1e-5
    x64 = solve(b, 0)
    for _ in range(6):
        x = x + solve(b - K @ x, 1)
    assert rel(x, x64) < 1e-10
    assert eta(x) < 1e-14


def _write_system(path, n, bs, rowp, cols, vals, mask, b, xyz):
    """The binary layout the sanitizer driver of direct_emul.cpp reads."""
    with open(path, "wb") as f:
        np.array([n, bs, len(cols), xyz is not None], np.int32).tofile(f)
        rowp.astype(np.int32).tofile(f)
        cols.astype(np.int32).tofile(f)
        vals.astype(np.float64).tofile(f)
        mask.astype(np.int32).tofile(f)
        b.astype(np.float64).tofile(f)
        if xyz is not None:
            np.asarray(xyz, np.float64).ravel().tofile(f)


def test_gpu_kernels_in_bounds_under_sanitizers(tmp_path):
    """Every load and store the numeric kernels make stays inside the
    buffers tg_direct.cu allocates: the emulation, with its buffers sized
    exactly as on the device, built with AddressSanitizer and
    UndefinedBehaviorSanitizer (any finding aborts), over meshes, a
    disconnected set of solids and a random pattern, both front paths, FP64
    and FP32.  The kernels' thread loops are all strided, so one thread per
    CTA visits exactly the GPU's index set."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    exe = str(tmp_path / "de_san")
    r = subprocess.run([cxx, "-O1", "-g", "-std=c++17",
                        "-fsanitize=address,undefined",
                        "-fno-sanitize-recover=all", "-pthread", "-DDE_MAIN",
                        "-I", INC,
                        EMUL, "-o", exe], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("sanitizer runtime unavailable: " + r.stderr[-200:])
    from tacs_gb300 import meshes
    cases = []
    for prob in (meshes.clamped_plate(12), meshes.hex_c3(4, 3, 3),
                 load_case("hex_rand")[0]):
        n, bs, rowp, cols, vals = _matrix(prob)
        cases.append((n, bs, rowp, cols, vals, _bcmask(prob),
                      np.asarray(prob["xpts"], np.float64)))
    rowp, cols, vals, xyz = _random_spd(120, 3, 12, 7)
    cases.append((120, 3, rowp, cols, vals, np.zeros(120, np.int32), xyz))
    sysf = str(tmp_path / "sys.bin")
    for n, bs, rowp, cols, vals, mask, xyz in cases:
        b = np.random.default_rng(n).standard_normal(n * bs)
        _write_system(sysf, n, bs, rowp, cols, vals, mask, b, xyz)
        for small_max in ("96", "0", str(1 << 30)):
            r = subprocess.run([exe, sysf, small_max], capture_output=True,
                               text=True, timeout=300)
            assert r.returncode == 0, r.stdout + r.stderr[-3000:]
            assert len(r.stdout.split()) == 4


@pytest.mark.parametrize("name,prob", list(_problems())[:3],
                         ids=[p[0] for p in _problems()][:3])
@pytest.mark.parametrize("nrhs", [2, 3, 4, 7])
@pytest.mark.parametrize("prec", [0, 1])
def test_gpu_kernels_on_cpu_multi_rhs(de, name, prob, nrhs, prec):
    """Several right-hand sides per pass over the factor (passes of 4, 2
    and 1, interleaved vectors): each right-hand side's solution is bitwise
    the one a single solve gives it, in FP64 and FP32."""
    n, bs, rowp, cols, vals = _matrix(prob)
    N = n * bs
    B = np.random.default_rng(nrhs).standard_normal((nrhs, N))
    xyz = np.ascontiguousarray(prob["xpts"], np.float64)
    mask = _bcmask(prob)
    X = np.zeros_like(B)
    assert de.de_solve_multi(n, bs, _ptr(rowp), _ptr(cols), _ptr(vals),
                             _ptr(mask), _ptr(xyz), 64, prec, nrhs, _ptr(B),
                             _ptr(X)) == 0
    for r in range(nrhs):
        b = np.ascontiguousarray(B[r])
        x = np.zeros(N)
        assert de.de_solve(n, bs, _ptr(rowp), _ptr(cols), _ptr(vals),
                           _ptr(mask), _ptr(xyz), 64, prec, _ptr(b),
                           _ptr(x)) == 0
        assert np.array_equal(X[r], x)
