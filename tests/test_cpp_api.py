"""The C++ interface (include/tacs_gb300.hpp): tests/cpp/plate_adjoint.cpp
drives a static analysis with adjoint gradients through the reference-named
C++ classes; it must compile against the headers (CPU) and reproduce the
reference's own outputs for the same 32 x 32 clamped plate (GPU; the golden
case shell_c1) at the solver tolerance, 1e-7."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_case, rel

SRC = os.path.join(ROOT, "tests", "cpp", "plate_adjoint.cpp")
CUDA_INC = "/usr/local/cuda/include"


def _compiler():
    return shutil.which("g++") or shutil.which("c++")


def test_cpp_header_compiles():
    cxx = _compiler()
    if not cxx or not os.path.isdir(CUDA_INC):
        pytest.skip("no C++ compiler or CUDA headers")
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall",
                        "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC,
                        SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["gmres", pytest.param(
    "direct", marks=pytest.mark.direct)])
def test_cpp_driver_matches_reference(tmp_path, mode):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    cxx = _compiler()
    lib_dir = os.path.join(ROOT, "tacs_gb300")
    exe = str(tmp_path / "plate_adjoint")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I",
                        os.path.join(ROOT, "include"), "-I", CUDA_INC, SRC,
                        "-o", exe, "-L", lib_dir, "-ltacs_gb300",
                        "-L/usr/local/cuda/lib64", "-lcudart",
                        f"-Wl,-rpath,{lib_dir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe] + (["direct"] if mode == "direct" else []),
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    d = json.loads(out.stdout)
    prob, ref = load_case("shell_c1")
    assert d["flag"] == 1
    assert rel(d["funcs"], ref["funcs"]) < 1e-7
    assert rel(np.array(d["grad0"]), ref["grad_comp"]) < 1e-7
    assert rel(np.array(d["grad1"]), ref["grad_ks"]) < 1e-7
    assert rel(np.array(d["gradX0"]), ref["grad_xpt_comp"]) < 1e-7
    assert rel(np.array(d["gradX1"]), ref["grad_xpt_ks"]) < 1e-7
