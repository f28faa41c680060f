"""The reference's Python interface (tacs/TACS.pyx) for the hot path, backed
by libtacs_gb300 on the GPU.

Class and method names, argument order and defaults follow tacs.TACS:
Assembler (create, setElementConnectivity, setElements, addBCs,
initialize, createVec / createNodeVec / createDesignVec / createMat,
setNodes, setDesignVars, setVariables, setAuxElements, assembleRes,
assembleJacobian, applyBCs, evalFunctions, addSVSens, addDVSens,
addAdjointResProducts, addXptSens, addAdjointResXptSensProducts), Vec, Mat,
Pc, KSM and AuxElements.  Vectors live on
the GPU; getArray() returns a host copy that is written back to the device
before the vector is next used, so the reference's ``vec.getArray()[:] =``
idiom works.  A single process owns the whole model (the comm argument is
accepted and ignored).  Features outside the hot path raise
NotImplementedError rather than running on the CPU.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from . import elements as _el
from .problem import Direct as _Direct, GpuModel, Ksm as _Ksm, Pc as _Pc

NORMAL, TRANSPOSE = _lib.MAT_NORMAL, _lib.MAT_TRANSPOSE


class Vec:
    """TACSBVec: a block vector on the GPU (device tensor ``dev``)."""

    def __init__(self, n, bsize=1):
        self.dev = torch.zeros(n, dtype=torch.float64, device="cuda")
        self.bsize = bsize
        self._host = None

    def _sync(self):
        if self._host is not None:
            self.dev.copy_(torch.as_tensor(self._host))
            self._host = None
        return self.dev

    def getArray(self):
        if self._host is None:
            self._host = self.dev.cpu().numpy()
        return self._host

    def getVarsPerNode(self):
        return self.bsize

    def getSize(self):
        return self.dev.numel()

    def zeroEntries(self):
        self._host = None
        self.dev.zero_()

    def copyValues(self, vec):
        self._host = None
        self.dev.copy_(vec._sync())

    def scale(self, alpha):
        self._sync().mul_(alpha)

    def axpy(self, alpha, vec):
        self._sync().add_(vec._sync(), alpha=alpha)

    def axpby(self, alpha, beta, vec):
        d = self._sync()
        d.mul_(beta).add_(vec._sync(), alpha=alpha)

    def norm(self):
        return float(torch.linalg.vector_norm(self._sync()))

    def dot(self, vec):
        return float(torch.dot(self._sync(), vec._sync()))

    def setRand(self, lower=-1.0, upper=1.0):
        self._host = None
        self.dev.uniform_(lower, upper)


class Mat:
    """TACSParallelMat over a BCSRMat of the assembler's pattern; with
    schur=True the matrix of createSchurMat, whose Pc is the complete
    factorisation."""

    def __init__(self, assembler, schur=False):
        self.assembler = assembler
        self.schur = schur
        self.gm = assembler._model.new_mat()

    def zeroEntries(self):
        self.gm.vals.zero_()

    def mult(self, x, y):
        y._host = None
        self.gm.mult(x._sync(), y.dev)

    def getMat(self):
        """scipy BSR matrix of the values (host copy)."""
        import scipy.sparse as sparse
        bs, nr = self.gm.bsize, self.gm.nrows
        vals = self.gm.vals.cpu().numpy().reshape(-1, bs, bs)
        return sparse.bsr_matrix((vals, self.gm.cols.cpu().numpy(),
                                  self.gm.rowp.cpu().numpy()),
                                 shape=(bs * nr, bs * nr))


class Pc:
    """TACS.Pc(mat, lev_fill=..., ratio_fill=..., reorder=...).

    For a matrix from createMat the reference builds
    TACSAdditiveSchwarz(mat, 5, 10.0) whatever the keywords say (they
    configure TACSSchurPc, tacs/TACS.pyx:1106-1139), so this is block
    ILU(5) on the GPU in the natural order.  fill_level=k overrides the
    level (an extension; 0 gives ILU(0)); precision='fp32' keeps the factor
    in FP32."""

    def __init__(self, mat, *args, precision="fp64", fill_level=5,
                 **kwargs):
        self.mat = mat
        self.direct = None
        if getattr(mat, "schur", False):
            # TACSSchurPc(mat, lev_fill = 1000000 by default, ...): with one
            # process a complete factorisation; lev_fill below that is not
            # offered on this matrix
            if int(kwargs.get("lev_fill", 1000000)) < 1000:
                raise NotImplementedError("incomplete Schur factorisations "
                                          "(lev_fill < 1000)")
            self.direct = _Direct(mat.gm)
            self.pc = None
            return
        prec = _lib.PREC_FP32 if precision == "fp32" else _lib.PREC_FP64
        self.pc = _Pc(mat.gm, _lib.PC_ILU0, prec, lev_fill=int(fill_level))

    def factor(self):
        (self.direct or self.pc).factor()

    def applyFactor(self, x, y):
        y._host = None
        if self.direct is not None:
            self.direct.solve(x._sync(), y.dev)
        else:
            self.pc.apply(x._sync(), y.dev)


class KSM:
    """TACS.KSM(mat, pc, m, nrestart=1, isFlexible=0): restarted GMRES.
    mixed=True runs the FP32 preconditioner and mat-vec inside FP64 GMRES
    with iterative refinement (needs Pc(..., precision='fp32'))."""

    def __init__(self, mat, pc, m, nrestart=1, isFlexible=0, mixed=False):
        # with the complete factorisation as preconditioner GMRES converges
        # in one step; the solve applies the factorisation directly
        self.direct = pc.direct if pc is not None else None
        self.ksm = None if self.direct is not None else _Ksm(
            mat.gm, pc.pc if pc is not None else None, m, nrestart, mixed)
        self._iters, self._res = 0, 0.0

    def setTolerances(self, rtol, atol):
        if self.ksm is not None:
            self.ksm.set_tolerances(rtol, atol)

    def solve(self, b, x, zero_guess=1):
        x._host = None
        if self.direct is not None:
            self.direct.solve(b._sync(), x.dev)
            self._iters, self._res = 1, 0.0
            return 1
        _, flag = self.ksm.solve(b._sync(), x.dev, bool(zero_guess))
        self._iters, self._res = self.ksm.iters, self.ksm.resnorm
        return flag

    def getIterCount(self):
        return self._iters

    def getResidualNorm(self):
        return self._res

    def setMonitor(self, *args, **kwargs):
        return None


class AuxElements:
    """TACSAuxElements: load elements attached to element numbers."""

    def __init__(self):
        self.items = []

    def addElement(self, num, elem):
        self.items.append((int(num), elem))


class Assembler:
    """TACSAssembler for one process (src/TACSAssembler.h:83-299)."""

    def __init__(self, varsPerNode, numOwnedNodes, numElements):
        self.vpn, self.nnodes, self.nelem = varsPerNode, numOwnedNodes, \
            numElements
        self.ptr = self.conn = None
        self.elems = None
        self.bc_nodes, self.bc_masks = [], []
        self.aux = None
        self._model = None
        self._vars = None

    @staticmethod
    def create(comm, varsPerNode, numOwnedNodes, numElements,
               numDependentNodes=0):
        if numDependentNodes:
            raise NotImplementedError("dependent nodes are not on the GPU path")
        return Assembler(varsPerNode, numOwnedNodes, numElements)

    # ------------------------------------------------------------ set-up
    def setElementConnectivity(self, ptr, conn):
        self.ptr = np.asarray(ptr, np.int64)
        self.conn = np.asarray(conn, np.int64)
        return 0

    def setElements(self, elements):
        if len(elements) != self.nelem:
            raise ValueError("one element object per element")
        self.elems = list(elements)
        return 0

    def addBCs(self, nodes, vars=None, values=None):
        if values is not None and np.any(np.asarray(values) != 0.0):
            raise NotImplementedError("non-zero Dirichlet values")
        mask = (1 << self.vpn) - 1 if vars is None else \
            int(sum(1 << int(v) for v in vars))
        for n in np.atleast_1d(nodes):
            self.bc_nodes.append(int(n))
            self.bc_masks.append(mask)

    def setAuxElements(self, aux):
        self.aux = aux
        if self._model is not None:
            raise NotImplementedError("set auxiliary elements before "
                                      "initialize()")

    def initialize(self):
        e0 = self.elems[0]
        et = e0.elem_type
        npe = e0.num_nodes
        if any(e.elem_type != et for e in self.elems):
            raise NotImplementedError("one element type per assembler")
        if np.any(np.diff(self.ptr) != npe):
            raise ValueError(f"every element needs {npe} nodes")
        props = e0.con.props
        if any(e.con.props is not props for e in self.elems):
            pr = props.getMaterialProperties()
            if any(e.con.props.getMaterialProperties() != pr
                   for e in self.elems):
                raise NotImplementedError("one material per assembler")
        thick = np.array([e.con.t for e in self.elems])
        dvnum = np.array([e.con.tNum for e in self.elems], np.int32)
        prob = {
            "elem_type": et, "nnodes": self.nnodes, "nelem": self.nelem,
            "xpts": np.zeros(3 * self.nnodes),
            "conn": self.conn.astype(np.int32), "thick": thick,
            "dvnum": dvnum,
            "mat": [props.rho, props.E, props.nu, props.ys],
            "transform": getattr(e0, "transform", _el.ShellNaturalTransform).kind
            if et == 0 else 0,
            "ref_axis": np.asarray(getattr(e0, "transform",
                                           _el.ShellNaturalTransform).axis)
            if et == 0 else np.array([1.0, 0.0, 0.0]),
            "bc_nodes": np.array(self.bc_nodes, np.int32),
            "bc_masks": np.array(self.bc_masks, np.int32),
        }
        if self.aux is not None:
            pe, pv, te, tf, tv = [], [], [], [], []
            for num, el in self.aux.items:
                if isinstance(el, _el.ShellPressure):
                    pe.append(num)
                    pv.append(el.values)
                elif isinstance(el, _el.Traction3D):
                    te.append(num)
                    tf.append(el.face)
                    tv.append(el.values)
                else:
                    raise NotImplementedError(type(el).__name__)
            if pe:
                prob["pres_elems"] = np.array(pe, np.int32)
                prob["pres_vals"] = np.concatenate(pv)
            if te:
                prob["trac_elems"] = np.array(te, np.int32)
                prob["trac_faces"] = np.array(tf, np.int32)
                prob["trac_vals"] = np.concatenate(tv)
        self._model = GpuModel(prob)
        self._vars = self.createVec()
        return 1

    # ----------------------------------------------------------- vectors
    def createVec(self):
        return Vec(self.vpn * self.nnodes, self.vpn)

    def createNodeVec(self):
        return Vec(3 * self.nnodes, 3)

    def createDesignVec(self):
        return Vec(self._model.ndv, 1)

    def createMat(self):
        return Mat(self)

    def createSchurMat(self, order_type=None):
        """The matrix pyTACS solves directly (createSchurMat); its Pc is the
        complete factorisation, ordered by nested dissection of the node
        coordinates whatever order_type asks for."""
        return Mat(self, schur=True)

    def getNumOwnedNodes(self):
        return self.nnodes

    def getNumElements(self):
        return self.nelem

    def getVarsPerNode(self):
        return self.vpn

    def setNodes(self, X):
        self._model.set_nodes(X._sync())

    def setDesignVars(self, x):
        self._model.set_design_vars(x._sync())

    def setVariables(self, vec, dvec=None, ddvec=None):
        self._vars.copyValues(vec)

    def getVariables(self, vec, dvec=None, ddvec=None):
        vec.copyValues(self._vars)

    def zeroVariables(self):
        self._vars.zeroEntries()

    def applyBCs(self, vec):
        self._model.apply_bcs(vec._sync())

    # ---------------------------------------------------------- assembly
    def assembleRes(self, residual, loadScale=1.0, applyBCs=True):
        residual._host = None
        self._model.assemble_res(self._vars._sync(), loadScale, applyBCs,
                                 residual.dev)

    def assembleJacobian(self, alpha, beta, gamma, residual, A, matOr=NORMAL,
                         loadScale=1.0, applyBCs=True):
        if (alpha, beta, gamma) != (1.0, 0.0, 0.0):
            if beta != 0.0 or gamma != 0.0:
                raise NotImplementedError("static Jacobian only (beta = "
                                          "gamma = 0)")
        res = None
        if residual is not None:
            residual._host = None
            res = residual.dev
        self._model.assemble_jacobian(self._vars._sync(), A.gm, res,
                                      transpose=matOr == TRANSPOSE,
                                      apply_bcs=applyBCs, lam=loadScale)
        if alpha != 1.0:
            A.gm.vals.mul_(alpha)

    # --------------------------------------------------------- functions
    def _ksw(self, funcs):
        w = {f.ksWeight for f in funcs if hasattr(f, "ksWeight")}
        if len(w) > 1:
            raise NotImplementedError("one KS weight per call")
        return w.pop() if w else None

    def evalFunctions(self, funcs):
        return self._model.eval_functions(self._vars._sync(),
                                          [f.kind for f in funcs],
                                          ks_weight=self._ksw(funcs))

    def addSVSens(self, funcs, dfdu, alpha=1.0, beta=0.0, gamma=0.0):
        u = self._vars._sync()
        self._model.eval_functions(u, [f.kind for f in funcs],
                                   ks_weight=self._ksw(funcs))
        for d in dfdu:
            d._sync()
            d._host = None
        self._model.add_sv_sens(u, [f.kind for f in funcs],
                                [d.dev for d in dfdu], alpha)

    def addDVSens(self, funcs, dfdx, alpha=1.0):
        u = self._vars._sync()
        self._model.eval_functions(u, [f.kind for f in funcs],
                                   ks_weight=self._ksw(funcs))
        for d in dfdx:
            d._sync()
            d._host = None
        self._model.add_dv_sens(u, [f.kind for f in funcs],
                                [d.dev for d in dfdx], alpha)

    def addAdjointResProducts(self, adjoints, dfdx, alpha=1.0, loadScale=1.0):
        for d in dfdx:
            d._sync()
            d._host = None
        self._model.add_adjoint_res_products(
            self._vars._sync(), [a._sync() for a in adjoints],
            [d.dev for d in dfdx], alpha)

    def addXptSens(self, funcs, dfdXpts, alpha=1.0):
        """Assembler.addXptSens (tacs/TACS.pyx): dfdX += alpha d f / dX."""
        u = self._vars._sync()
        self._model.eval_functions(u, [f.kind for f in funcs],
                                   ks_weight=self._ksw(funcs))
        for d in dfdXpts:
            d._sync()
            d._host = None
        self._model.add_xpt_sens(u, [f.kind for f in funcs],
                                 [d.dev for d in dfdXpts], alpha)

    def addAdjointResXptSensProducts(self, adjoints, dfdXpts, alpha=1.0,
                                     loadScale=1.0):
        """Assembler.addAdjointResXptSensProducts (tacs/TACS.pyx):
        dfdX += alpha psi^T dR/dX."""
        for d in dfdXpts:
            d._sync()
            d._host = None
        self._model.add_adjoint_res_xpt_products(
            self._vars._sync(), [a._sync() for a in adjoints],
            [d.dev for d in dfdXpts], alpha, loadScale)
