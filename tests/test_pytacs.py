"""pyTACS-style static problems on the GPU (tacs_gb300.pytacs), driven the
way the reference's test_shell_plate_quad.py drives pytacs: the reference's
100-element plate model (written back to a BDF from the golden fixture),
the element call-back with one thickness design variable for the PLATE
component, a 100 kPa pressure case and a 10 kN point load at GRID 81,
compliance and KS failure (weight 10) against the known answers of that
test (1e-8), and the design and node-coordinate sensitivities against
central differences of the solves."""
import numpy as np
import pytest

from conftest import ROOT  # noqa: F401

KNOWN = "tests/golden/known/plate_bdf.npz"


def _bdf(tmp_path):
    from tacs_gb300 import bdf, meshes
    d = np.load(KNOWN)
    p = meshes._base(meshes.SHELL, d["in_xpts"].reshape(-1, 3),
                     d["in_conn"].reshape(-1, 4), d["in_thick"],
                     d["in_dvnum"], d["in_mat"])
    p["bc_nodes"], p["bc_masks"] = d["in_bc_nodes"], d["in_bc_masks"]
    path = str(tmp_path / "plate.bdf")
    bdf.write_bdf(path, p, {1: "PLATE"})
    ref = {k[4:]: float(d[k]) for k in d.files if k.startswith("ref_")}
    # the fixture's GRID ids are 1..121 in node order, as written here
    assert np.array_equal(d["in_grid_ids"], np.arange(1, 122))
    return path, ref


def _callback(dvNum, compID, compDescript, elemDescripts, globalDVs,
              **kwargs):
    from tacs_gb300 import constitutive, elements
    prop = constitutive.MaterialProperties(rho=2500.0, E=70e9, nu=0.3,
                                           ys=464.0e6)
    con = constitutive.IsoShellConstitutive(prop, t=0.005, tNum=dvNum)
    return elements.Quad4Shell(None, con), [100.0]


def test_pytacs_selects_components(tmp_path):
    pytest.importorskip("torch")
    from tacs_gb300 import pytacs
    path, _ = _bdf(tmp_path)
    fea = pytacs.pyTACS(path)
    assert fea.getNumComponents() == 1
    assert fea.selectCompIDs(include="PLATE") == [0]
    assert fea.selectCompIDs(include="SKIN") == []


@pytest.mark.gpu
def test_pytacs_static_problems_match_reference(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import functions, pytacs
    path, ref = _bdf(tmp_path)
    fea = pytacs.pyTACS(path)
    fea.initialize(_callback)
    probs = []
    sp = fea.createStaticProblem("point_load")
    sp.addLoadToNodes(81, np.array([0.0, 0.0, 1e4, 0.0, 0.0, 0.0]),
                      nastranOrdering=True)
    probs.append(sp)
    sp = fea.createStaticProblem("pressure")
    sp.addPressureToComponents(fea.selectCompIDs(include="PLATE"), 100e3)
    probs.append(sp)
    funcs, sens = {}, {}
    for sp in probs:
        sp.addFunction("compliance", functions.Compliance)
        sp.addFunction("ks_vmfailure", functions.KSFailure, ksWeight=10.0)
        sp.solve()
        sp.evalFunctions(funcs)
        sp.evalFunctionsSens(sens)
    for key in ("pressure_compliance", "pressure_ks_vmfailure",
                "point_load_compliance", "point_load_ks_vmfailure"):
        assert abs(funcs[key] / ref[key] - 1) < 1e-8, key
    # d compliance / d t of the single thickness variable, central FD
    sp = probs[1]
    g = sens["pressure_compliance"]["struct"][0]
    t0 = sp.getDesignVars()
    h = 1e-5 * t0[0]
    vals = []
    for s in (1.0, -1.0):
        sp.setDesignVars(t0 + s * h)
        sp.solve()
        f = {}
        sp.evalFunctions(f, ["compliance"])
        vals.append(f["pressure_compliance"])
    sp.setDesignVars(t0)
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(fd - g) < 1e-5 * abs(g)
    # node-coordinate sensitivities ("Xpts") of both functions against
    # central differences of the solves, in-plane coordinates of two nodes
    sp.solve()
    sens = {}
    sp.evalFunctionsSens(sens)
    X0 = sp.getNodes()
    h = 1e-6
    for key in ("compliance", "ks_vmfailure"):
        gx = sens["pressure_" + key]["Xpts"]
        assert gx.shape == X0.shape
        for j in (3 * 38 + 0, 3 * 50 + 1):
            vals = []
            for s in (1.0, -1.0):
                X = X0.copy()
                X[j] += s * h
                sp.setNodes(X)
                sp.solve()
                f = {}
                sp.evalFunctions(f, [key])
                vals.append(f["pressure_" + key])
            sp.setNodes(X0)
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - gx[j]) < 1e-5 * np.abs(gx).max(), (key, j)


@pytest.mark.gpu
@pytest.mark.direct
def test_pytacs_direct_solve_matches_reference(tmp_path):
    """The same problems solved by the complete factorisation (option
    directSolve): the known answers (1e-8) and the same sensitivities as
    the iterative solves (1e-7)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import functions, pytacs
    path, ref = _bdf(tmp_path)
    fea = pytacs.pyTACS(path)
    fea.initialize(_callback)
    out = {}
    for direct in (False, True):
        sp = fea.createStaticProblem("pressure",
                                     options={"directSolve": direct})
        sp.addPressureToComponents(fea.selectCompIDs(include="PLATE"), 100e3)
        sp.addFunction("compliance", functions.Compliance)
        sp.addFunction("ks_vmfailure", functions.KSFailure, ksWeight=10.0)
        sp.solve()
        funcs, sens = {}, {}
        sp.evalFunctions(funcs)
        sp.evalFunctionsSens(sens)
        out[direct] = (funcs, sens)
    funcs, sens = out[True]
    for key in ("pressure_compliance", "pressure_ks_vmfailure"):
        assert abs(funcs[key] / ref[key] - 1) < 1e-8, key
        for part in ("struct", "Xpts"):
            a, b = sens[key][part], out[False][1][key][part]
            assert np.abs(a - b).max() < 1e-7 * np.abs(b).max(), (key, part)
