"""pyTACS and StaticProblem for the GPU path, with the reference's call
pattern (tacs/pytacs.py, tacs/problems/static.py):

    fea = pyTACS(bdf_file)
    fea.initialize(elemCallBack)          # callback(dvNum, compID, ...)
    sp = fea.createStaticProblem("pressure")
    sp.addPressureToComponents(fea.selectCompIDs(include="PLATE"), 100e3)
    sp.addLoadToNodes(81, [0, 0, 1e4, 0, 0, 0], nastranOrdering=True)
    sp.addFunction("compliance", functions.Compliance)
    sp.addFunction("ks", functions.KSFailure, ksWeight=10.0)
    sp.solve()
    funcs, sens = {}, {}
    sp.evalFunctions(funcs)               # funcs["pressure_compliance"]
    sp.evalFunctionsSens(sens)            # sens[...]["struct"]: d f / d x
                                          # sens[...]["Xpts"]: d f / d X

Models come from tacs_gb300.bdf (one element type per model); the element
call-back returns tacs_gb300.elements objects over one material.  Functions
are Compliance and KSFailure, with design-variable ("struct") and
node-coordinate ("Xpts", 3 per node in the BDF's node order)
sensitivities.  Every solve, function and sensitivity runs on the GPU.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, bdf
from . import elements as _el
from . import functions as _fn
from .problem import Direct, GpuModel, Ksm, Pc


class pyTACS:
    """Model set-up from a BDF file (pyTACS(fileName, comm, options))."""

    def __init__(self, fileName, comm=None, options=None):
        self.bdfName = fileName
        self.options = dict(options or {})
        self.record = bdf.read_bdf(fileName)
        pids = self.record["elem_pids"]
        self._pids = sorted(set(int(x) for x in pids))
        self._names = self.record["pid_names"]
        self.elements = None
        self.ndv = 0

    # --------------------------------------------------------- components
    def getNumComponents(self):
        return len(self._pids)

    def getComponentDescripts(self):
        return [self._names.get(p, "") for p in self._pids]

    def selectCompIDs(self, include=None, exclude=None):
        """Component indices whose description contains one of include
        (all if None) and none of exclude (case-insensitive)."""
        def as_list(v):
            return [v] if isinstance(v, str) else list(v or [])
        inc, exc = as_list(include), as_list(exclude)
        out = []
        for c, p in enumerate(self._pids):
            d = self._names.get(p, "").upper()
            if inc and not any(s.upper() in d for s in inc):
                continue
            if any(s.upper() in d for s in exc):
                continue
            out.append(c)
        return out

    def initialize(self, elemCallBack):
        """elemCallBack(dvNum, compID, compDescript, elemDescripts,
        globalDVs, **kwargs) -> element (or (element, scales)); dvNum counts
        up over the components, as in pyTACS."""
        pids = self.record["elem_pids"]
        shell = int(self.record["elem_type"]) == 0
        self.elements = [None] * len(pids)
        dv = 0
        for c, pid in enumerate(self._pids):
            r = elemCallBack(dvNum=dv, compID=c,
                             compDescript=self._names.get(pid, ""),
                             elemDescripts=["CQUAD4" if shell else "CHEXA"],
                             globalDVs={}, propID=pid)
            elem = r[0] if isinstance(r, (tuple, list)) else r
            for e in np.nonzero(pids == pid)[0]:
                self.elements[e] = elem
            if elem.con.tNum >= 0:
                dv = max(dv, elem.con.tNum + 1)
        self.ndv = dv
        e0 = self.elements[0]
        props = e0.con.props
        rec = self.record
        rec["thick"] = np.array([e.con.t for e in self.elements])
        rec["dvnum"] = np.array([e.con.tNum for e in self.elements], np.int32)
        rec["mat"] = np.array([props.rho, props.E, props.nu, props.ys])
        if shell:
            tr = e0.transform
            rec["transform"] = tr.kind
            rec["ref_axis"] = np.asarray(tr.axis, np.float64)

    def getOrigDesignVars(self):
        x = np.zeros(self.ndv)
        for e in self.elements:
            if e.con.tNum >= 0:
                x[e.con.tNum] = e.con.t
        return x

    def createStaticProblem(self, name, options=None):
        if self.elements is None:
            raise RuntimeError("call initialize() first")
        return StaticProblem(name, self, options)


class _DirectSolves:
    """The solve interface of Ksm over a Direct factorisation."""

    def __init__(self, direct):
        self.direct = direct

    def solve(self, b):
        return self.direct.solve(b), 1


class StaticProblem:
    """Linear static analysis (tacs/problems/static.py) on the GPU."""

    # The reference factors the matrix completely (PCFillLevel 1000 on a
    # Schur matrix, tacs/problems/static.py:59,329); the GPU path has no
    # direct factorisation, so the fill level is capped at MAX_FILL (block
    # ILU(5)) and the Krylov space is larger than the reference's 10.
    MAX_FILL = 5
    # "directSolve" (an extension) solves both systems by the complete
    # multifrontal factorisation instead, as the reference's default does
    defaults = {"subSpaceSize": 100, "nRestarts": 20,
                "L2ConvergenceRel": 1e-12, "L2Convergence": 1e-30,
                "PCFillLevel": 1000, "directSolve": False}

    def __init__(self, name, fea, options=None):
        self.name, self.fea = name, fea
        self.options = dict(self.defaults)
        self.options.update(options or {})
        rec = fea.record
        self.vpn = 6 if int(rec["elem_type"]) == 0 else 3
        self.nnodes, self.nelem = int(rec["nnodes"]), int(rec["nelem"])
        self.F = np.zeros(self.vpn * self.nnodes)
        self.pressure = np.zeros(self.nelem)
        self.has_pressure = False
        self.functionList = {}
        self.x = fea.getOrigDesignVars()
        self._model = None
        self._xpts = None
        self.u = None

    def setOption(self, name, value):
        self.options[name] = value

    def getDesignVars(self):
        return self.x.copy()

    def setDesignVars(self, x):
        self.x = np.asarray(x, np.float64).copy()

    def getNodes(self):
        """Node coordinates, 3 per node (TACSProblem.getNodes)."""
        return np.asarray(self.fea.record["xpts"], np.float64).copy() \
            if self._xpts is None else self._xpts.copy()

    def setNodes(self, Xpts):
        """New node coordinates for this problem (TACSProblem.setNodes)."""
        self._xpts = np.asarray(Xpts, np.float64).ravel().copy()
        if self._model is not None:
            self._model.set_nodes(torch.as_tensor(self._xpts, device="cuda"))

    # -------------------------------------------------------------- loads
    def _node_index(self, ids, nastranOrdering):
        ids = np.atleast_1d(ids)
        if not nastranOrdering:
            return ids.astype(int)
        gid = self.fea.record["grid_ids"]
        pos = {int(g): k for k, g in enumerate(gid)}
        return np.array([pos[int(i)] for i in ids])

    def addLoadToNodes(self, nodeIDs, F, nastranOrdering=False):
        idx = self._node_index(nodeIDs, nastranOrdering)
        F = np.asarray(F, np.float64).reshape(-1, self.vpn)
        if F.shape[0] == 1:
            F = np.repeat(F, len(idx), axis=0)
        for k, n in enumerate(idx):
            self.F[self.vpn * n:self.vpn * (n + 1)] += F[k]

    def addPressureToComponents(self, compIDs, pressures, faceIndex=0):
        pids = self.fea.record["elem_pids"]
        p = np.broadcast_to(np.asarray(pressures, np.float64),
                            (len(np.atleast_1d(compIDs)),))
        for c, pc in zip(np.atleast_1d(compIDs), p):
            self.pressure[pids == self.fea._pids[int(c)]] += pc
        self.has_pressure = True
        self._model = None

    def addPressureToElements(self, elemIDs, pressures, faceIndex=0,
                              nastranOrdering=False):
        ids = np.atleast_1d(elemIDs)
        if nastranOrdering:
            pos = {int(e): k for k, e in enumerate(self.fea.record["elem_ids"])}
            ids = np.array([pos[int(e)] for e in ids])
        p = np.broadcast_to(np.asarray(pressures, np.float64), (len(ids),))
        self.pressure[ids] += p
        self.has_pressure = True
        self._model = None

    # ---------------------------------------------------------- functions
    def addFunction(self, funcName, funcHandle, compIDs=None, **kwargs):
        if funcHandle not in (_fn.Compliance, _fn.KSFailure):
            raise NotImplementedError(
                f"{getattr(funcHandle, '__name__', funcHandle)} is not on the "
                "GPU path (Compliance and KSFailure are)")
        if compIDs is not None:
            raise NotImplementedError("functions over a component subset")
        ksw = float(kwargs.get("ksWeight", 80.0))
        self.functionList[funcName] = (funcHandle.kind, ksw)

    # -------------------------------------------------------------- solve
    def _ensure_model(self):
        if self._model is None:
            rec = dict(self.fea.record)
            if self.has_pressure:
                pe = np.nonzero(self.pressure)[0]
                rec["pres_elems"] = pe.astype(np.int32)
                rec["pres_vals"] = np.repeat(self.pressure[pe], 4)
            if self._xpts is not None:
                rec["xpts"] = self._xpts
            self._model = GpuModel(rec)
            self._mat = self._model.new_mat()
            if self.options["directSolve"]:
                self._pc = Direct(self._mat)
                self._ksm = _DirectSolves(self._pc)
            else:
                lev = max(0, min(int(self.options["PCFillLevel"]),
                                 self.MAX_FILL))
                self._pc = Pc(self._mat, lev_fill=lev)
                self._ksm = Ksm(self._mat, self._pc,
                                self.options["subSpaceSize"],
                                self.options["nRestarts"])
                self._ksm.set_tolerances(self.options["L2ConvergenceRel"],
                                         self.options["L2Convergence"])
        return self._model

    def solve(self, Fext=None):
        M = self._ensure_model()
        if self.fea.ndv:
            M.set_design_vars(torch.as_tensor(self.x, device="cuda"))
        r0 = M.vec()
        M.assemble_jacobian(M.vec(), self._mat, r0)
        self._pc.factor()
        f = M.vec(self.F if Fext is None else self.F + np.asarray(Fext))
        M.apply_bcs(f)
        u, flag = self._ksm.solve(f - r0)
        if flag != 1:
            raise _lib.TacsGpuError(f"{self.name}: GMRES did not converge")
        self.u = u
        return flag

    def getVariables(self):
        return self.u.cpu().numpy()

    def evalFunctions(self, funcs, evalFuncs=None, ignoreMissing=False):
        names = sorted(self.functionList if evalFuncs is None else evalFuncs)
        for f in names:
            if f not in self.functionList:
                if ignoreMissing:
                    continue
                raise KeyError(f"function '{f}' was not added")
            kind, ksw = self.functionList[f]
            funcs[f"{self.name}_{f}"] = float(self._model.eval_functions(
                self.u, [kind], ks_weight=ksw)[0])

    def evalFunctionsSens(self, funcsSens, evalFuncs=None,
                          includeDVSens=True, includeXptSens=True):
        M = self._model
        names = sorted(self.functionList if evalFuncs is None else evalFuncs)
        for f in names:
            kind, ksw = self.functionList[f]
            M.eval_functions(self.u, [kind], ks_weight=ksw)
            dfdu = M.vec()
            M.add_sv_sens(self.u, [kind], [dfdu])
            M.apply_bcs(dfdu)
            psi, flag = self._ksm.solve(dfdu)
            if flag != 1:
                raise _lib.TacsGpuError(f"{self.name}: adjoint GMRES did not "
                                        "converge")
            out = {}
            if includeDVSens:
                g = M.dv_vec()
                M.add_total_derivative(self.u, kind, psi, g, 1.0, -1.0)
                out["struct"] = g.cpu().numpy()
            if includeXptSens:
                gx = M.node_vec()
                M.add_total_xpt_derivative(self.u, kind, psi, gx, 1.0, -1.0)
                out["Xpts"] = gx.cpu().numpy()
            funcsSens[f"{self.name}_{f}"] = out
