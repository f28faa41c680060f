"""BDF ingestion (tacs_gb300.bdf): card parsing on synthetic input (CPU),
and the reference's 100-element plate model read by it, solved against the
known answers the reference's own test pins (tests/golden/known/
plate_bdf.npz, made by tests/golden/make_bdf_golden.py): by the oracle on
the CPU and by the GPU path.  Tolerance 1e-8 relative: the known answers
come from the reference's solve at its own tolerance (observed agreement
~1e-9)."""
import os

import numpy as np
import pytest

from conftest import ROOT

from tacs_gb300 import bdf, meshes

KNOWN = os.path.join(ROOT, "tests", "golden", "known", "plate_bdf.npz")
TOL = 1e-8

SMALL = """$ 2 x 1 plate, small field with a continuation
CORD2R         5       0      1.      0.      0.      1.      0.      1.+C1
+C1           2.      0.      0.
GRID           1       5      0.      0.      0.
GRID           2       5      .5      0.      0.
GRID           3       5     1.0      0.      0.
GRID           4       5      0.     1.0      0.
GRID           5       5      .5    1.+0      0.
GRID           6       5     1.0  100.-2      0.
CQUAD4        11       1       1       2       5       4
CQUAD4        12       1       2       3       6       5
SPC1           1     123       1       4
FORCE          1       6       0    10.0      0.      0.     -1.
"""

FREE = """GRID,1,,0.,0.,0.
GRID,2,,0.5,0.,0.
GRID,3,,1.,0.,0.
GRID,4,,0.,1.,0.
GRID,5,,.5,1.,0.
GRID,6,,1.,1.,0.
CQUAD4,11,1,1,2,5,4
CQUAD4,12,1,2,3,6,5
SPC1,1,123,1,4
FORCE,1,6,0,10.,0.,0.,-1.
"""


def _large_grid(gid, cp, x, y, z):
    """GRID* in large-field format: 16-character fields, the z coordinate
    on a '*' continuation line."""
    def f16(v):
        return f"{v:>16}"
    return (f"{'GRID*':<8}{f16(gid)}{f16(cp)}{f16(x)}{f16(y)}*G{gid}\n"
            f"{'*G' + str(gid):<8}{f16(z)}\n")


LARGE = "".join(_large_grid(i + 1, "", x, y, "0.25") for i, (x, y) in enumerate(
    [("0.", "0."), (".5", "0."), ("1.0", "0."), ("0.", "1.0"), (".5", "1."),
     ("1.0", "1.0")])) + """CQUAD4        11       1       1       2       5       4
CQUAD4        12       1       2       3       6       5
SPC1           1     123       1       4
FORCE          1       6       0    10.0      0.      0.     -1.
"""


@pytest.mark.parametrize("text", [SMALL, FREE, LARGE],
                         ids=["small", "free", "large"])
def test_bdf_cards(tmp_path, text):
    f = tmp_path / "m.bdf"
    f.write_text(text)
    p = bdf.read_bdf(str(f), thickness=0.01)
    ref = meshes.plate(2, 1, Lx=1.0, Ly=1.0, t=0.01)
    xyz = p["xpts"].reshape(-1, 3)
    if text is SMALL:  # CORD2R 5: origin (1, 0, 0), basic axes
        xyz = xyz - np.array([1.0, 0.0, 0.0])
    if text is LARGE:  # the plate at z = 0.25 (z on the continuation)
        xyz = xyz - np.array([0.0, 0.0, 0.25])
    assert np.allclose(xyz, ref["xpts"].reshape(-1, 3))
    assert np.array_equal(p["conn"], ref["conn"])
    assert list(p["bc_nodes"]) == [0, 3]
    assert list(p["bc_masks"]) == [7, 7]
    F = p["force"].reshape(-1, 6)
    assert F[5, 2] == -10.0 and np.count_nonzero(F) == 1
    assert list(p["elem_ids"]) == [11, 12]


def test_nastran_reals():
    assert bdf._real("1.07+7") == 1.07e7
    assert bdf._real("2.5906-4") == 2.5906e-4
    assert bdf._real("-.5") == -0.5
    assert bdf._real("1.E-5") == 1e-5
    assert bdf._real("3.") == 3.0


def _problem():
    d = np.load(KNOWN)
    p = meshes._base(meshes.SHELL, d["in_xpts"].reshape(-1, 3),
                     d["in_conn"].reshape(-1, 4), d["in_thick"],
                     d["in_dvnum"], d["in_mat"])
    p["bc_nodes"], p["bc_masks"] = d["in_bc_nodes"], d["in_bc_masks"]
    p["point_force"] = d["in_point_force"]
    p["ks_weight"] = 10.0
    ref = {k[4:]: float(d[k]) for k in d.files if k.startswith("ref_")}
    return p, ref


def _pressure(p):
    q = dict(p)
    q["pres_elems"] = np.arange(p["nelem"], dtype=np.int32)
    q["pres_vals"] = np.full(4 * p["nelem"], 100e3)
    return q


def test_known_answers_oracle():
    import oracle
    p, ref = _problem()
    o = oracle.Oracle(_pressure(p))
    r = o.static_adjoint(np.zeros(o.ndof), 200, 10, 1e-12)
    assert abs(r["funcs"][0] / ref["pressure_compliance"] - 1) < TOL
    assert abs(r["funcs"][1] / ref["pressure_ks_vmfailure"] - 1) < TOL
    o = oracle.Oracle(p)
    r = o.static_adjoint(p["point_force"], 200, 10, 1e-12)
    assert abs(r["funcs"][0] / ref["point_load_compliance"] - 1) < TOL
    assert abs(r["funcs"][1] / ref["point_load_ks_vmfailure"] - 1) < TOL


@pytest.mark.gpu
def test_known_answers_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import problem
    p, ref = _problem()
    M = problem.GpuModel(_pressure(p))
    r = problem.static_adjoint(M, np.zeros(M.ndof), 200, 10, 1e-12)
    assert abs(r["funcs"][0] / ref["pressure_compliance"] - 1) < TOL
    assert abs(r["funcs"][1] / ref["pressure_ks_vmfailure"] - 1) < TOL
    M = problem.GpuModel(p)
    r = problem.static_adjoint(M, p["point_force"], 200, 10, 1e-12)
    assert abs(r["funcs"][0] / ref["point_load_compliance"] - 1) < TOL
    assert abs(r["funcs"][1] / ref["point_load_ks_vmfailure"] - 1) < TOL
