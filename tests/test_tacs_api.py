"""The reference-style Python interface (tacs_gb300.TACS / elements /
constitutive / functions): a static analysis with adjoint gradients (design
variables and node coordinates) written the way the reference's
integration tests drive tacs.TACS
(tests/integration_tests/static_analysis_base_test.py:359-427), checked
against the reference's own outputs (golden fixtures)."""
import numpy as np
import pytest

from conftest import load_case, rel

TOL = 1e-7

API = {
    "Assembler": ["create", "setElementConnectivity", "setElements", "addBCs",
                  "initialize", "createVec", "createNodeVec",
                  "createDesignVec", "createMat", "createSchurMat", "setNodes",
                  "setDesignVars", "setVariables", "getVariables",
                  "zeroVariables", "setAuxElements", "assembleRes",
                  "assembleJacobian", "applyBCs", "evalFunctions",
                  "addSVSens", "addDVSens", "addAdjointResProducts",
                  "addXptSens", "addAdjointResXptSensProducts"],
    "Vec": ["getArray", "zeroEntries", "copyValues", "scale", "axpy",
            "axpby", "norm", "dot", "setRand", "getVarsPerNode", "getSize"],
    "Mat": ["zeroEntries", "mult", "getMat"],
    "Pc": ["factor", "applyFactor"],
    "KSM": ["setTolerances", "solve", "getIterCount", "getResidualNorm"],
    "AuxElements": ["addElement"],
}


def test_api_names_match_reference():
    pytest.importorskip("torch")
    from tacs_gb300 import TACS, constitutive, elements, functions
    for cls, meths in API.items():
        c = getattr(TACS, cls)
        for m in meths:
            assert hasattr(c, m), f"TACS.{cls}.{m}"
    for name in ("Quad4Shell", "ShellNaturalTransform", "ShellRefAxisTransform",
                 "Element3D", "LinearElasticity3D", "LinearHexaBasis",
                 "Traction3D"):
        assert hasattr(elements, name)
    for name in ("MaterialProperties", "IsoShellConstitutive",
                 "SolidConstitutive"):
        assert hasattr(constitutive, name)
    for name in ("Compliance", "KSFailure"):
        assert hasattr(functions, name)


def _build(prob):
    from tacs_gb300 import TACS, constitutive, elements
    rho, E, nu, ys = [float(v) for v in prob["mat"]]
    props = constitutive.MaterialProperties(rho=rho, E=E, nu=nu, ys=ys)
    ne, nn = int(prob["nelem"]), int(prob["nnodes"])
    shell = int(prob["elem_type"]) == 0
    npe = 4 if shell else 8
    if shell:
        tr = (elements.ShellRefAxisTransform(prob["ref_axis"])
              if int(prob.get("transform", 0)) else
              elements.ShellNaturalTransform())
        elems = [elements.Quad4Shell(tr, constitutive.IsoShellConstitutive(
            props, t=float(prob["thick"][e]), tNum=int(prob["dvnum"][e])))
            for e in range(ne)]
    else:
        basis = elements.LinearHexaBasis()
        elems = [elements.Element3D(
            elements.LinearElasticity3D(constitutive.SolidConstitutive(
                props, t=float(prob["thick"][e]), tNum=int(prob["dvnum"][e]))),
            basis) for e in range(ne)]
    assembler = TACS.Assembler.create(None, 6 if shell else 3, nn, ne)
    assembler.setElementConnectivity(np.arange(0, npe * ne + 1, npe),
                                      prob["conn"])
    assembler.setElements(elems)
    for node, mask in zip(prob["bc_nodes"], prob["bc_masks"]):
        assembler.addBCs(np.array([node], np.int32),
                         np.array([k for k in range(6) if (mask >> k) & 1],
                                  np.int32))
    aux = TACS.AuxElements()
    for k, e in enumerate(prob.get("pres_elems", [])):
        aux.addElement(int(e), elements.ShellPressure(
            prob["pres_vals"][4 * k:4 * k + 4]))
    for k, e in enumerate(prob.get("trac_elems", [])):
        aux.addElement(int(e), elems[int(e)].createElementTraction(
            int(prob["trac_faces"][k]), prob["trac_vals"][3 * k:3 * k + 3]))
    assembler.setAuxElements(aux)
    assembler.initialize()
    X = assembler.createNodeVec()
    X.getArray()[:] = prob["xpts"]
    assembler.setNodes(X)
    return assembler


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["shell_c1", "shell_plate8", "hex_block",
                                  "shell_cyl"])
@pytest.mark.parametrize("schur", [False, pytest.param(
    True, marks=pytest.mark.direct)])
def test_static_adjoint_through_reference_api(name, schur):
    """schur=True: createSchurMat with the default Pc, the reference's
    direct solve (here the complete multifrontal factorisation)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from tacs_gb300 import TACS, functions
    prob, ref = load_case(name)
    assembler = _build(prob)
    res, ans = assembler.createVec(), assembler.createVec()
    mat = assembler.createSchurMat() if schur else assembler.createMat()
    assembler.zeroVariables()
    assembler.assembleJacobian(1.0, 0.0, 0.0, res, mat)
    pc = TACS.Pc(mat)
    pc.factor()
    gmres = TACS.KSM(mat, pc, int(prob.get("gmres_m", 100)), 50)
    gmres.setTolerances(float(prob.get("rtol", 1e-12)), 1e-30)
    f = assembler.createVec()
    f.getArray()[:] = prob["force"]
    assembler.applyBCs(f)
    res.axpy(-1.0, f)
    assert gmres.solve(res, ans) == 1
    ans.scale(-1.0)
    assembler.setVariables(ans)
    assert rel(ans.getArray(), ref["u"]) < TOL
    funcs = [functions.Compliance(assembler),
             functions.KSFailure(assembler,
                                 ksWeight=float(prob.get("ks_weight", 100.0)))]
    fvals = assembler.evalFunctions(funcs)
    assert rel(fvals, ref["funcs"]) < TOL
    grads = []
    for k, fn in enumerate(funcs):
        dfdu = assembler.createVec()
        assembler.addSVSens([fn], [dfdu])
        assembler.applyBCs(dfdu)
        psi = assembler.createVec()
        assert gmres.solve(dfdu, psi) == 1
        dfdx = assembler.createDesignVec()
        assembler.addDVSens([fn], [dfdx])
        assembler.addAdjointResProducts([psi], [dfdx], -1.0)
        dfdX = assembler.createNodeVec()
        assembler.addXptSens([fn], [dfdX])
        assembler.addAdjointResXptSensProducts([psi], [dfdX], -1.0)
        grads.append((dfdx.getArray().copy(), dfdX.getArray().copy()))
    assert rel(grads[0][0], ref["grad_comp"]) < TOL
    assert rel(grads[1][0], ref["grad_ks"]) < TOL
    assert rel(grads[0][1], ref["grad_xpt_comp"]) < TOL
    assert rel(grads[1][1], ref["grad_xpt_ks"]) < TOL
