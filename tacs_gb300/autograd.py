"""Linear static solve -> structural functional as a torch.autograd.Function.

Forward (for design variables x, e.g. per-element shell thickness or solid
density): set x, assemble K(x) and the load, ILU(0) + GMRES for u, evaluate
f(u, x) (compliance or the KS failure aggregate).  Backward: the adjoint
solve K^T psi = df/du with the same factorisation (K is symmetric with the
reference's row-and-column boundary conditions, so the forward matrix is
reused as TACSAssembler::assembleJacobian(..., TRANSPOSE) would produce it),
then df/dx - psi^T dR/dx from the fused addDVSens + addAdjointResProducts
kernel (and, for node coordinates, df/dX - psi^T dR/dX from the dual-number
addXptSens + addAdjointResXptSensProducts kernel).  This is the reference's
own adjoint recipe
(tests/integration_tests/static_analysis_base_test.py:359-427,
tacs/problems/static.py:1140-1279) behind torch's autograd.

Several load cases (and several independent meshes) are solved and
differentiated together when the solver holds more than one load vector:
the functional then returns one value per (load case, mesh).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .problem import Direct, Ksm, Pc


class StaticSolver:
    """State shared by the forward and backward passes of one model.

    loads: (nlc, ndof) or (ndof,) nodal forces (device or host); the
    assembler's own pressure / traction loads are added to every case when
    include_element_loads is true (as R(u) = K u - f_elem - f).
    """

    def __init__(self, model, loads, m=100, nrestart=50, rtol=1e-12,
                 atol=1e-30, pc_kind=_lib.PC_ILU0, mixed=False,
                 include_element_loads=True, segments=False, lev_fill=0,
                 direct=False):
        self.model = model
        F = torch.as_tensor(np.asarray(loads, np.float64) if not
                            torch.is_tensor(loads) else loads,
                            dtype=torch.float64, device="cuda")
        self.F = F.reshape(-1, model.ndof).clone()
        self.nlc = self.F.shape[0]
        self.include_element_loads = include_element_loads
        self.segments = segments
        if segments:
            if model.ndv != model.nelem or np.any(
                    np.asarray(model.prob["dvnum"]) != np.arange(model.nelem)):
                raise ValueError("segments need one design variable per "
                                 "element, numbered like the elements")
            model.set_segments(model.prob["seg_elem_ptr"])
        self.mat = model.new_mat()
        # direct: True / "fp64" complete factorisation, "mixed" in FP32
        # with FP64 refinement of every solve; either refined to the
        # relative residual rtol (or the FP64 floor) like the Krylov solves
        self.direct = Direct(self.mat, precision=_lib.PREC_FP32
                             if direct == "mixed" else _lib.PREC_FP64) \
            if direct else None
        self.rtol = rtol
        self.mixed_direct = direct == "mixed"
        if direct:
            self.pc = self.ksm = None
        else:
            prec = _lib.PREC_FP32 if mixed else _lib.PREC_FP64
            self.pc = Pc(self.mat, pc_kind, prec, lev_fill=lev_fill)
            self.ksm = Ksm(self.mat, self.pc, m, nrestart, mixed)
            self.ksm.set_tolerances(rtol, atol)
            if segments:
                self.ksm.set_segments(model.prob["seg_node_ptr"])
        self.u = None
        self.iters = []
        self.flags = []

    def solve(self, x, xpts=None):
        M = self.model
        if xpts is not None:
            M.set_nodes(xpts.detach().to(torch.float64).contiguous())
        M.set_design_vars(x.detach().to(torch.float64).contiguous())
        r0 = M.vec()
        M.assemble_jacobian(M.vec(), self.mat, r0)
        if self.direct is not None:
            self.direct.factor()
        else:
            self.pc.factor()
        B = self.F.clone()
        for lc in range(self.nlc):
            M.apply_bcs(B[lc])
            if self.include_element_loads:
                B[lc] -= r0
        U, it, fl, _, rc = self._solve_multi(B)
        self.u = U
        self.iters.append(it)
        self.flags.append(fl)
        if rc != 1:
            raise _lib.TacsGpuError(
                f"GMRES did not converge (flags {fl.tolist()})")
        return U

    def _solve_multi(self, B):
        """All load cases (and meshes): batched GMRES, or the complete
        factorisation one load case at a time (exact, 0 iterations)."""
        if self.direct is None:
            return self.ksm.solve_multi(B)
        X = self.direct.solve(B.contiguous(), rtol=self.rtol)
        nsys = B.shape[0] * (self.model.nseg if self.segments else 1)
        return (X, np.zeros(nsys, np.int32), np.ones(nsys, np.int32),
                np.zeros(nsys), 1)

    def functions(self, func):
        M = self.model
        if self.segments:
            return np.stack([M.eval_functions_segments(self.u[lc], func)
                             for lc in range(self.nlc)])
        return np.array([[M.eval_functions(self.u[lc], [func])[0]]
                         for lc in range(self.nlc)])

    def gradients(self, func, weights, xpts=False):
        """sum over (load case, mesh) of weights * d f / d x; with xpts, also
        the node-coordinate gradient (addXptSens +
        addAdjointResXptSensProducts) and the pair (g, gX) is returned."""
        M = self.model
        if xpts and self.segments:
            raise NotImplementedError("node-coordinate gradients of "
                                      "segmented models")
        W = np.asarray(weights, np.float64).reshape(self.nlc, -1)
        dfdu = torch.zeros_like(self.u)
        for lc in range(self.nlc):
            if self.segments:
                M.eval_functions_segments(self.u[lc], func)
                M.add_sv_sens_segments(self.u[lc], func, dfdu[lc])
            else:
                M.eval_functions(self.u[lc], [func])
                M.add_sv_sens(self.u[lc], [func], [dfdu[lc]])
            M.apply_bcs(dfdu[lc])
        if self.segments:
            # per-mesh weights: scale each mesh's rows of dfdu
            nptr = self.model.prob["seg_node_ptr"]
            vpn = M.vpn
            for lc in range(self.nlc):
                for g in range(W.shape[1]):
                    dfdu[lc, vpn * nptr[g]:vpn * nptr[g + 1]] *= W[lc, g]
        else:
            dfdu *= torch.as_tensor(W[:, 0], device="cuda")[:, None]
        Psi, it, fl, _, rc = self._solve_multi(dfdu)
        self.iters.append(it)
        self.flags.append(fl)
        if rc != 1:
            raise _lib.TacsGpuError(
                f"adjoint GMRES did not converge (flags {fl.tolist()})")
        g = M.dv_vec()
        gX = M.node_vec() if xpts else None
        for lc in range(self.nlc):
            if self.segments:
                # coefficient of df/dx per element = the mesh weight
                M.eval_functions_segments(self.u[lc], func)
                gl = M.dv_vec()
                M.add_total_derivative_segments(self.u[lc], func, Psi[lc], gl,
                                                1.0, 0.0)
                w_el = np.repeat(W[lc], np.diff(self.model.prob["seg_elem_ptr"]))
                g += gl * torch.as_tensor(w_el, device="cuda")
                M.add_total_derivative_segments(self.u[lc], func, Psi[lc], g,
                                                0.0, -1.0)
            else:
                M.eval_functions(self.u[lc], [func])
                M.add_total_derivative(self.u[lc], func, Psi[lc], g,
                                       float(W[lc, 0]), -1.0)
                if xpts:
                    M.add_total_xpt_derivative(self.u[lc], func, Psi[lc], gX,
                                               float(W[lc, 0]), -1.0)
        return (g, gX) if xpts else g


class StaticFunctional(torch.autograd.Function):
    """f = StaticFunctional.apply(x, solver, func, xpts) -> (nlc, nmesh)
    tensor; xpts (node coordinates, 3 per node) may be None."""

    @staticmethod
    def forward(ctx, x, solver, func, xpts=None):
        solver.solve(x, xpts)
        f = solver.functions(func)
        ctx.solver, ctx.func = solver, func
        ctx.x_shape, ctx.x_dtype = x.shape, x.dtype
        ctx.has_xpts = xpts is not None
        if ctx.has_xpts:
            ctx.X_shape, ctx.X_dtype = xpts.shape, xpts.dtype
        return torch.as_tensor(f, dtype=torch.float64, device=x.device)

    @staticmethod
    def backward(ctx, gout):
        w = gout.detach().cpu().numpy()
        want_X = ctx.has_xpts and ctx.needs_input_grad[3]
        if want_X:
            g, gX = ctx.solver.gradients(ctx.func, w, xpts=True)
            gX = gX.to(ctx.X_dtype).reshape(ctx.X_shape)
        else:
            g, gX = ctx.solver.gradients(ctx.func, w), None
        return g.to(ctx.x_dtype).reshape(ctx.x_shape), None, None, gX


def static_functional(x, solver, func=_lib.FUNC_COMPLIANCE, xpts=None):
    """Structural functional of the design variables x (and, when given,
    of the node coordinates xpts) through a linear static solve."""
    return StaticFunctional.apply(x, solver, func, xpts)
