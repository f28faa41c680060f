"""The allocation-free entry point tg_eval_functions_noalloc, called
through the C ABI, against the allocating path (tg_eval_functions).

Callers that cannot allocate device memory (a host framework that hands
out views of its own pre-allocated arena, or a loop that has frozen its
memory footprint) use this entry point.  The test file sorts after every
other test (tests/conftest.py orders it last), so that a run stopping at its
first failure has already run the rest; it must also pass alone in a fresh
process, where the first call on the device performs the scratch-address
set-up.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12  # the same element arithmetic and reductions as the reference path


def _meshes():
    from tacs_gb300 import meshes
    rng = np.random.default_rng(101)
    sh = meshes.plate(24, 20, 1.2, 1.0,
                      zfun=lambda X, Y: 0.05 * np.sin(2 * X) * np.cos(Y),
                      thick=0.004 + 0.01 * rng.random(480))
    sh["transform"], sh["ref_axis"] = 1, np.array([1.0, 0.3, 0.0])
    hx = meshes.hex_block(6, 5, 4, 1.5, 1.2, 1.0,
                          thick=0.1 + 0.9 * rng.random(120))
    return [(sh, 1e-3), (hx, 1e-4)]


def _noalloc(L, prob, u, out):
    d = lambda a, dt: torch.as_tensor(np.asarray(a, dt), device="cuda")  # noqa
    conn = d(prob["conn"], np.int32)
    xpts = d(prob["xpts"], np.float64)
    thick = d(prob["thick"], np.float64)
    axis = np.ascontiguousarray(prob.get("ref_axis", [1.0, 0, 0]), np.float64)
    _, E, nu, ys = [float(v) for v in prob["mat"]]
    rc = L.tg_eval_functions_noalloc(
        int(prob["elem_type"]), int(prob["nelem"]),
        C.c_void_p(conn.data_ptr()), C.c_void_p(xpts.data_ptr()),
        C.c_void_p(thick.data_ptr()), E, nu, ys, int(prob.get("transform", 0)),
        axis.ctypes.data, C.c_void_p(u.data_ptr()), float(prob["ks_weight"]),
        C.c_void_p(out.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc


def test_noalloc_matches_allocating_path_twice():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required")
    from tacs_gb300 import _lib, problem
    L = _lib.lib()
    for prob, scale in _meshes():
        M = problem.GpuModel(prob)
        rng = np.random.default_rng(7)
        for call in range(2):  # two calls in a row, different states
            u = M.vec(scale * rng.standard_normal(M.ndof))
            ref = M.eval_functions(u, (0, 1))
            out = torch.full((2,), np.nan, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            assert _noalloc(L, prob, u, out) == 0, L.tg_last_error()
            if call == 1:
                # the first call may load kernel modules; the second one
                # must leave the device's free memory exactly as it was
                assert torch.cuda.mem_get_info()[0] == free0
            got = out.cpu().numpy()
            assert rel(got, ref) < TOL, (call, got, ref)


def test_noalloc_rejects_oversized_mesh():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required")
    from tacs_gb300 import _lib
    L = _lib.lib()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = L.tg_eval_functions_noalloc(
        0, 32768 + 1, C.c_void_p(dummy.data_ptr()), C.c_void_p(dummy.data_ptr()),
        C.c_void_p(dummy.data_ptr()), 70e9, 0.3, 2.7e8, 0, None,
        C.c_void_p(dummy.data_ptr()), 100.0, C.c_void_p(dummy.data_ptr()), None)
    assert rc == -1
    assert b"TG_NOALLOC_MAX_ELEMENTS" in L.tg_last_error()
