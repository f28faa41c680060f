"""Device-resident model built from a problem record (tacs_gb300.meshes).

:class:`GpuModel` drives the C ABI of libtacs_gb300 with torch CUDA tensors
as device storage.  It is the plumbing under the reference-style API in
:mod:`tacs_gb300.TACS` and the object the tests and the benchmark use.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class _DevArray:
    """Exposes a raw device allocation to torch via __cuda_array_interface__."""

    def __init__(self, ptr, n, typestr="<f8"):
        self.__cuda_array_interface__ = {
            "shape": (int(n),), "typestr": typestr, "data": (int(ptr), False),
            "version": 3, "strides": None}


def device_view(ptr, n, dtype=torch.float64):
    typestr = {torch.float64: "<f8", torch.float32: "<f4",
               torch.int32: "<i4"}[dtype]
    return torch.as_tensor(_DevArray(ptr, n, typestr), device="cuda")


class Mat:
    """tg_mat: BCSR matrix with the assembler's pattern (device)."""

    def __init__(self, model):
        L = _lib.lib()
        h = C.c_void_p()
        check(L.tg_mat_create(model.handle, C.byref(h)), "tg_mat_create")
        self.handle, self.model = h, model
        bs, nr = C.c_int(), C.c_int()
        rowp, cols, vals = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(L.tg_mat_get_arrays(h, C.byref(bs), C.byref(nr), C.byref(rowp),
                                  C.byref(cols), C.byref(vals)))
        self.bsize, self.nrows = bs.value, nr.value
        self.rowp = device_view(rowp.value, self.nrows + 1, torch.int32)
        nnz = int(self.rowp[-1].item())
        self.nnz = nnz
        self.cols = device_view(cols.value, nnz, torch.int32)
        self.vals = device_view(vals.value, nnz * self.bsize ** 2)

    def mult(self, x, y=None):
        y = torch.empty_like(x) if y is None else y
        check(_lib.lib().tg_mat_mult(self.handle, _p(x), _p(y), _stream()),
              "tg_mat_mult")
        return y

    def __del__(self):
        try:
            _lib.lib().tg_mat_decref(self.handle)
        except Exception:
            pass


class Pc:
    """tg_pc: ILU(k) / block-Jacobi preconditioner, FP64 or FP32."""

    @classmethod
    def from_direct(cls, direct):
        """tg_pc_create_direct: a preconditioner sharing the factorisation
        of a Direct (factor() then only refreshes the FP32 matrix copy)."""
        h = C.c_void_p()
        check(_lib.lib().tg_pc_create_direct(direct.handle, C.byref(h)),
              "tg_pc_create_direct")
        pc = cls.__new__(cls)
        # the C object holds its own reference to the factorisation: no
        # Python reference back to the Direct (which keeps this pc), so
        # dropping the Direct frees its device memory at once
        pc.handle, pc.mat = h, direct.mat
        return pc

    def fp64_used(self):
        """True when mixed GMRES switched to an FP64 factor of the matrix."""
        u = C.c_int(0)
        check(_lib.lib().tg_pc_get_fp64_used(self.handle, C.byref(u)))
        return bool(u.value)

    def __init__(self, mat, kind=_lib.PC_ILU0, precision=_lib.PREC_FP64,
                 lev_fill=0):
        h = C.c_void_p()
        if lev_fill > 0:
            if kind != _lib.PC_ILU0:
                raise ValueError("fill levels need the natural-order ILU")
            check(_lib.lib().tg_pc_create_iluk(mat.handle, int(lev_fill),
                                               precision, C.byref(h)),
                  "tg_pc_create_iluk")
        else:
            check(_lib.lib().tg_pc_create(mat.handle, kind, precision,
                                          C.byref(h)), "tg_pc_create")
        self.handle, self.mat = h, mat

    def fill(self):
        """(level of fill, blocks in the factor)."""
        lev, nnz = C.c_int(), C.c_int()
        check(_lib.lib().tg_pc_get_fill(self.handle, C.byref(lev),
                                        C.byref(nnz)))
        return lev.value, nnz.value

    def factor(self):
        check(_lib.lib().tg_pc_factor(self.handle, _stream()), "tg_pc_factor")

    def apply(self, x, y=None):
        y = torch.empty_like(x) if y is None else y
        check(_lib.lib().tg_pc_apply(self.handle, _p(x), _p(y), _stream()),
              "tg_pc_apply")
        return y

    def schedule(self):
        """Cluster size, clusters, levels and the autotuner's timings."""
        cs, ng, nl = C.c_int(), C.c_int(), C.c_int()
        ms = np.zeros(5)
        check(_lib.lib().tg_pc_get_schedule(self.handle, C.byref(cs),
                                            C.byref(ng), C.byref(nl),
                                            ms.ctypes.data))
        return {"cluster_size": cs.value, "clusters": ng.value,
                "levels": nl.value,
                "tuned_ms": {1 << i: float(ms[i]) for i in range(5)
                             if ms[i] > 0}}

    def __del__(self):
        try:
            _lib.lib().tg_pc_decref(self.handle)
        except Exception:
            pass


class Direct:
    """tg_direct: complete multifrontal factorisation of an assembled
    matrix (the reference's direct solve), nested dissection by the node
    coordinates; solve(b) returns A^-1 b for the assembled A with its row
    boundary conditions.

    precision PREC_FP32 factors in FP32 and solves FP64 right-hand sides
    by iterative refinement (FP64 residuals, FP32 corrections) until the
    normwise backward error is at most eps sqrt(N) (the test of LAPACK's
    mixed-precision dsgesv) and a further step no longer halves it.  Where
    refinement stagnates (cond(A) near the inverse of FP32's unit
    roundoff, so that one FP32 solve contracts the error too little), the
    solve is done again by FP64 GMRES preconditioned by the same FP32
    factorisation (GMRES-IR, `mode` "gmres_ir", which later solves then
    take directly); where that fails too, or the FP32 Cholesky meets a
    non-positive pivot, the matrix is factored in FP64 instead
    (`fell_back`), from its values at that moment.

    autotune: tg_direct_autotune picks the solves' launch shapes once per
    matrix shape.  It costs about a dozen solves, so it runs at the second
    factor() of this object (a factorisation reused for a design loop), or
    at the first when this process has tuned the shape before (then it
    only applies the cached choice)."""

    _tuned_shapes = set()

    def __init__(self, mat, use_coords=True, precision=_lib.PREC_FP64,
                 autotune=True):
        h = C.c_void_p()
        check(_lib.lib().tg_direct_create(mat.handle, int(use_coords),
                                          int(precision), C.byref(h)),
              "tg_direct_create")
        self.handle, self.mat, self.precision = h, mat, precision
        self.use_coords = use_coords
        self._fp64 = None
        self.fell_back = False
        self.last_steps, self.last_eta = 0, 0.0
        # after the first factorisation: the solves' launch shapes
        # (tg_direct_autotune), then cached per matrix shape
        self.autotune = autotune
        self.tuned = None
        self.nfactor = 0
        # FP32: how FP64 right-hand sides are solved ("refine", or
        # "gmres_ir" after refinement stagnated on this matrix)
        self.mode = "refine"
        self._ir = None
        self.last_gmres_iters = 0

    def _factor_fp64(self):
        self._fp64 = Direct(self.mat, self.use_coords, _lib.PREC_FP64)
        self._fp64.factor()
        self.fell_back = True

    def _shape(self):
        m = self.mat
        return (m.nrows, m.nnz, m.bsize, self.precision,
                torch.cuda.current_device())

    def factor(self):
        self._fp64 = None
        self.fell_back = False
        self.nfactor += 1
        rc = _lib.lib().tg_direct_factor(self.handle, _stream())
        if rc == _lib.ERR_PIVOT and self.precision == _lib.PREC_FP32:
            self._factor_fp64()  # the FP32 Cholesky broke down
            return
        check(rc, "tg_direct_factor")
        if self.autotune and self.tuned is None and (
                self.nfactor >= 2 or self._shape() in Direct._tuned_shapes):
            Direct._tuned_shapes.add(self._shape())
            thr = C.c_int(0)
            ms = np.zeros(3)
            check(_lib.lib().tg_direct_autotune(self.handle, C.byref(thr),
                                                 ms.ctypes.data, _stream()),
                  "tg_direct_autotune")
            self.tuned = {"cluster_threshold": thr.value,
                          "candidates": [384, 768, 1536],
                          "solve_ms": ms.tolist()}

    def solve(self, b, x=None, steps=30, tol=None, ftol=0.0, rtol=0.0):
        """x = A^-1 b; b a vector or an (nrhs, n) tensor of right-hand sides
        (solved together, up to four per pass over the factor).  FP64
        factorisation: FP64 vectors, one solve, or with rtol > 0 refined
        in FP64 until the residual is at most rtol |b| (max norms).  FP32
        factorisation: FP32 vectors are solved in FP32, FP64 ones by
        refinement (at most `steps` steps, to the backward error `tol`,
        default eps sqrt(n), per right-hand side; with ftol > 0 or
        rtol > 0 until every given test holds: a step's correction at most
        ftol |x|, the residual at most rtol |b|), or by the FP64
        factorisation after a fallback."""
        x = torch.empty_like(b) if x is None else x
        L = _lib.lib()
        nrhs = b.shape[0] if b.dim() == 2 else 1
        if self._fp64 is not None and b.dtype == torch.float64:
            return self._fp64.solve(b, x, steps=steps, rtol=rtol)
        refine = b.dtype == torch.float64 and (
            self.precision == _lib.PREC_FP32 or rtol > 0.0)
        if refine:
            n = b.shape[-1]
            if tol is None:
                tol = 2.0 ** -53 * float(np.sqrt(n))
            if x.data_ptr() == b.data_ptr():  # in place: refine from a copy
                b = b.clone()
            f32 = self.precision == _lib.PREC_FP32
            if f32 and self.mode == "gmres_ir":
                return self._gmres_ir_or_fp64(b, x, steps, rtol)
            st = np.zeros(nrhs, np.int32)
            eta = np.zeros(nrhs)
            rc = L.tg_direct_solve_refined_multi(
                self.handle, nrhs, _p(b), _p(x), int(steps), float(tol),
                float(ftol), float(rtol), st.ctypes.data, eta.ctypes.data,
                _stream())
            self.last_steps, self.last_eta = int(st.max()), float(eta.max())
            if rc == _lib.ERR_NOCONV and f32:
                # refinement stagnated: this matrix needs GMRES-IR
                self.mode = "gmres_ir"
                return self._gmres_ir_or_fp64(b, x, steps, rtol)
            check(rc, "tg_direct_solve_refined_multi")
            return x
        if self.precision == _lib.PREC_FP32:
            if nrhs > 1:
                for r in range(nrhs):
                    self.solve(b[r], x[r])
                return x
            check(L.tg_direct_solve_f32(self.handle, _p(b), _p(x), _stream()),
                  "tg_direct_solve_f32")
            return x
        check(L.tg_direct_solve_multi(self.handle, nrhs, _p(b), _p(x),
                                      _stream()), "tg_direct_solve_multi")
        return x

    def _gmres_ir_or_fp64(self, b, x, steps, rtol):
        """FP64 flexible GMRES(30) preconditioned by this FP32
        factorisation (GMRES-IR) to the relative residual rtol (1e-12 when
        none is given), restarted up to max(steps, 10) times; the FP64
        factorisation when it does not converge."""
        n = b.shape[-1]
        if self._ir is None:
            pc = Pc.from_direct(self)
            # FP64 Arnoldi and mat-vec, the FP32 factorisation applied to
            # FP32 copies of the Krylov vectors (flexible GMRES)
            self._ir = (pc, Ksm(self.mat, pc, m=30, nrestart=max(steps, 10),
                                mixed=False))
        pc, ksm = self._ir
        pc.factor()  # the FP32 copy of the current matrix values
        ksm.set_tolerances(rtol if rtol > 0.0 else 1e-12)
        X, it, fl, rn, rc = ksm.solve_multi(b.reshape(-1, n),
                                            x.reshape(-1, n))
        self.last_gmres_iters = int(it.max())
        self.last_steps = 0
        if rc == 1:
            return x
        self._factor_fp64()
        return self._fp64.solve(b, x, steps=steps, rtol=rtol)

    def stats(self):
        st = np.zeros(9)
        check(_lib.lib().tg_direct_get_stats(self.handle, st.ctypes.data))
        return {"supernodes": int(st[0]), "levels": int(st[1]),
                "factor_bytes": st[2], "pool_bytes": st[3],
                "flops": st[4], "max_front": int(st[5]),
                "cluster_fronts": int(st[7]),
                "cluster_threshold": int(st[8]),
                "tuned": self.tuned,
                "fell_back_to_fp64": self.fell_back,
                "fp32_mode": self.mode if self.precision ==
                _lib.PREC_FP32 else None,
                "last_gmres_iters": self.last_gmres_iters,
                "gmres_ir_fp64_factor": bool(self._ir is not None
                                             and self._ir[0].fp64_used()),
                "last_refinement_steps": self.last_steps,
                "last_backward_error": self.last_eta}

    def __del__(self):
        try:
            _lib.lib().tg_direct_decref(self.handle)
        except Exception:
            pass


class Ksm:
    """tg_ksm: restarted GMRES (optionally mixed precision)."""

    def __init__(self, mat, pc, m=100, nrestart=2, mixed=False):
        h = C.c_void_p()
        check(_lib.lib().tg_ksm_create(mat.handle, pc.handle if pc else None,
                                       m, nrestart, int(mixed), C.byref(h)),
              "tg_ksm_create")
        self.handle, self.mat, self.pc = h, mat, pc
        self.iters, self.resnorm = 0, 0.0

    def set_tolerances(self, rtol, atol=1e-30):
        check(_lib.lib().tg_ksm_set_tolerances(self.handle, rtol, atol))

    def solve(self, b, x=None, zero_guess=True):
        x = torch.zeros_like(b) if x is None else x
        it, rn = C.c_int(0), C.c_double(0.0)
        flag = check(_lib.lib().tg_ksm_solve(self.handle, _p(b), _p(x),
                                             int(zero_guess), C.byref(it),
                                             C.byref(rn), _stream()),
                     "tg_ksm_solve")
        self.iters, self.resnorm = it.value, rn.value
        return x, flag

    def graph_info(self):
        """tg_ksm_get_graph_info: whether a restart cycle runs as one graph
        (device-side loop over the Arnoldi step) and the launches of one
        step."""
        cyc, n64, n32 = C.c_int(0), C.c_int(0), C.c_int(0)
        check(_lib.lib().tg_ksm_get_graph_info(self.handle, C.byref(cyc),
                                                C.byref(n64), C.byref(n32)))
        return {"cycle_graph": bool(cyc.value), "step_launches": n64.value,
                "step_launches_fp32": n32.value}

    def set_segments(self, row_ptr):
        """Independent row ranges (block-diagonal matrix): one system each."""
        rp = np.ascontiguousarray(row_ptr, np.int32)
        check(_lib.lib().tg_ksm_set_segments(self.handle, len(rp) - 1,
                                             rp.ctypes.data),
              "tg_ksm_set_segments")
        self.nseg = len(rp) - 1

    def solve_multi(self, B, X=None, zero_guess=True):
        """B: (nrhs, n) device tensor.  Returns X, per-system iterations,
        flags and residual norms (index rhs * nseg + range)."""
        B = B.contiguous()
        nrhs = B.shape[0]
        X = torch.zeros_like(B) if X is None else X
        ns = getattr(self, "nseg", 1) * nrhs
        it = np.zeros(ns, np.int32)
        fl = np.zeros(ns, np.int32)
        rn = np.zeros(ns, np.float64)
        rc = check(_lib.lib().tg_ksm_solve_multi(
            self.handle, nrhs, _p(B), _p(X), int(zero_guess), it.ctypes.data,
            fl.ctypes.data, rn.ctypes.data, _stream()), "tg_ksm_solve_multi")
        self.iters = int(it.max()) if ns else 0
        return X, it, fl, rn, rc

    def __del__(self):
        try:
            _lib.lib().tg_ksm_decref(self.handle)
        except Exception:
            pass


class GpuModel:
    """An initialised tg_assembler holding one mesh, its loads and DVs."""

    def __init__(self, prob):
        if not torch.cuda.is_available():
            raise _lib.TacsGpuError("a CUDA device is required")
        L = _lib.lib()
        self.prob = prob
        et = int(prob["elem_type"])
        self.vpn = 6 if et == 0 else 3
        self.nnodes, self.nelem = int(prob["nnodes"]), int(prob["nelem"])
        self.ndof = self.vpn * self.nnodes
        conn = np.ascontiguousarray(prob["conn"], np.int32)
        rho, E, nu, ys = [float(v) for v in prob["mat"]]
        axis = np.ascontiguousarray(prob.get("ref_axis", [1.0, 0, 0]),
                                    np.float64)
        h = C.c_void_p()
        check(L.tg_assembler_create(et, self.nnodes, self.nelem,
                                    conn.ctypes.data, rho, E, nu, ys,
                                    int(prob.get("transform", 0)),
                                    axis.ctypes.data, C.byref(h)),
              "tg_assembler_create")
        self.handle = h
        bcn = np.ascontiguousarray(prob.get("bc_nodes", []), np.int32)
        bcm = np.ascontiguousarray(prob.get("bc_masks", []), np.int32)
        check(L.tg_assembler_add_bcs(h, len(bcn), bcn.ctypes.data,
                                     bcm.ctypes.data), "add_bcs")
        thick = np.ascontiguousarray(prob["thick"], np.float64)
        dvnum = np.ascontiguousarray(prob["dvnum"], np.int32)
        check(L.tg_assembler_set_element_dvs(h, thick.ctypes.data,
                                             dvnum.ctypes.data), "dvs")
        pe = np.ascontiguousarray(prob.get("pres_elems", []), np.int32)
        if len(pe):
            pv = np.ascontiguousarray(prob["pres_vals"], np.float64)
            check(L.tg_assembler_set_pressure(h, len(pe), pe.ctypes.data,
                                              pv.ctypes.data), "pressure")
        te = np.ascontiguousarray(prob.get("trac_elems", []), np.int32)
        if len(te):
            tf = np.ascontiguousarray(prob["trac_faces"], np.int32)
            tv = np.ascontiguousarray(prob["trac_vals"], np.float64)
            check(L.tg_assembler_set_traction(h, len(te), te.ctypes.data,
                                              tf.ctypes.data, tv.ctypes.data),
                  "traction")
        check(L.tg_assembler_initialize(h), "tg_assembler_initialize")
        vpn, nn, ne, ndv, nc = (C.c_int() for _ in range(5))
        check(L.tg_assembler_get_sizes(h, C.byref(vpn), C.byref(nn),
                                       C.byref(ne), C.byref(ndv),
                                       C.byref(nc)))
        self.ndv, self.ncolors = ndv.value, nc.value
        self.xpts = torch.as_tensor(np.asarray(prob["xpts"], np.float64),
                                    device="cuda")
        check(L.tg_assembler_set_nodes(h, _p(self.xpts), _stream()),
              "set_nodes")
        self.ks_weight = float(prob.get("ks_weight", 100.0))

    def __del__(self):
        try:
            _lib.lib().tg_assembler_decref(self.handle)
        except Exception:
            pass

    # ---------------------------------------------------------------- api
    def vec(self, values=None):
        if values is None:
            return torch.zeros(self.ndof, dtype=torch.float64, device="cuda")
        return torch.as_tensor(np.asarray(values, np.float64),
                               device="cuda").clone()

    def set_nodes(self, xpts):
        """Node coordinates (3 per node, device tensor)."""
        self.xpts = xpts
        check(_lib.lib().tg_assembler_set_nodes(self.handle, _p(xpts),
                                                _stream()), "set_nodes")

    def set_fixed_geometry(self, enable=True):
        """Fixed-geometry assembly (tg_assembler_set_fixed_geometry): the
        residual and Jacobian from per-geometry coefficient matrices, built
        at the next assembly and after every set_nodes."""
        check(_lib.lib().tg_assembler_set_fixed_geometry(self.handle,
                                                         int(enable)),
              "set_fixed_geometry")

    def fixed_geometry_info(self):
        n, tb, pb = C.c_int(0), C.c_double(0.0), C.c_double(0.0)
        check(_lib.lib().tg_assembler_get_fixed_geometry(
            self.handle, C.byref(n), C.byref(tb), C.byref(pb)),
            "get_fixed_geometry")
        return {"classes": n.value, "table_bytes": tb.value,
                "plan_bytes": pb.value}

    def set_design_vars(self, dvs):
        check(_lib.lib().tg_assembler_set_design_vars(self.handle, _p(dvs),
                                                      _stream()), "set_dvs")

    def assemble_res(self, u, lam=1.0, apply_bcs=True, res=None):
        res = torch.empty(self.ndof, dtype=torch.float64,
                          device="cuda") if res is None else res
        check(_lib.lib().tg_assemble_res(self.handle, _p(u), lam,
                                         int(apply_bcs), _p(res), _stream()),
              "tg_assemble_res")
        return res

    def new_mat(self):
        return Mat(self)

    def assemble_jacobian(self, u, mat, res=None, transpose=False,
                          apply_bcs=True, lam=1.0):
        check(_lib.lib().tg_assemble_jacobian(
            self.handle, 1.0, 0.0, 0.0, _p(u), _p(res), mat.handle,
            int(transpose), lam, int(apply_bcs), _stream()),
            "tg_assemble_jacobian")
        return res

    def apply_bcs(self, x):
        check(_lib.lib().tg_apply_bcs(self.handle, _p(x), _stream()))
        return x

    def eval_functions(self, u, funcs=(0, 1), ks_weight=None):
        f = np.ascontiguousarray(funcs, np.int32)
        out = np.zeros(len(f))
        ksw = self.ks_weight if ks_weight is None else ks_weight
        check(_lib.lib().tg_eval_functions(self.handle, _p(u), len(f),
                                           f.ctypes.data, ksw,
                                           out.ctypes.data, _stream()),
              "tg_eval_functions")
        return out

    def add_sv_sens(self, u, funcs, dfdu, alpha=1.0):
        f = np.ascontiguousarray(funcs, np.int32)
        ptrs = (C.c_void_p * len(f))(*[t.data_ptr() for t in dfdu])
        check(_lib.lib().tg_add_sv_sens(self.handle, _p(u), len(f),
                                        f.ctypes.data, alpha, ptrs,
                                        _stream()), "tg_add_sv_sens")

    def add_dv_sens(self, u, funcs, dfdx, coef=1.0):
        f = np.ascontiguousarray(funcs, np.int32)
        ptrs = (C.c_void_p * len(f))(*[t.data_ptr() for t in dfdx])
        check(_lib.lib().tg_add_dv_sens(self.handle, _p(u), len(f),
                                        f.ctypes.data, coef, ptrs,
                                        _stream()), "tg_add_dv_sens")

    def add_adjoint_res_products(self, u, psis, dfdx, scale=1.0):
        pp = (C.c_void_p * len(psis))(*[t.data_ptr() for t in psis])
        dp = (C.c_void_p * len(dfdx))(*[t.data_ptr() for t in dfdx])
        check(_lib.lib().tg_add_adjoint_res_products(
            self.handle, _p(u), scale, len(psis), pp, dp, _stream()),
            "tg_add_adjoint_res_products")

    def add_total_derivative(self, u, func, psi, dfdx, coef=1.0, scale=-1.0):
        check(_lib.lib().tg_add_total_derivative(
            self.handle, _p(u), int(func), coef, _p(psi), scale, _p(dfdx),
            _stream()), "tg_add_total_derivative")

    def dv_vec(self):
        return torch.zeros(self.ndv, dtype=torch.float64, device="cuda")

    # ------------------------------------- node-coordinate sensitivities
    def node_vec(self):
        """Zero node vector, 3 per node (TACSAssembler::createNodeVec)."""
        return torch.zeros(3 * self.nnodes, dtype=torch.float64, device="cuda")

    def set_xpt_mode(self, reverse):
        """Element coordinate derivatives by the reverse (adjoint) sweep,
        one thread per element, instead of dual numbers per coordinate."""
        check(_lib.lib().tg_set_xpt_mode(
            self.handle, _lib.XPT_REVERSE if reverse else _lib.XPT_FORWARD),
            "tg_set_xpt_mode")

    def add_xpt_sens(self, u, funcs, dfdX, coef=1.0):
        """dfdX[i] += coef d f_i / dX (TACSAssembler::addXptSens)."""
        f = np.ascontiguousarray(funcs, np.int32)
        ptrs = (C.c_void_p * len(f))(*[t.data_ptr() for t in dfdX])
        check(_lib.lib().tg_add_xpt_sens(self.handle, _p(u), len(f),
                                         f.ctypes.data, coef, ptrs,
                                         _stream()), "tg_add_xpt_sens")

    def add_adjoint_res_xpt_products(self, u, psis, dfdX, scale=1.0,
                                     lam=1.0):
        """dfdX[k] += scale psi_k^T dR/dX
        (TACSAssembler::addAdjointResXptSensProducts)."""
        pp = (C.c_void_p * len(psis))(*[t.data_ptr() for t in psis])
        dp = (C.c_void_p * len(dfdX))(*[t.data_ptr() for t in dfdX])
        check(_lib.lib().tg_add_adjoint_res_xpt_products(
            self.handle, _p(u), scale, len(psis), pp, dp, lam, _stream()),
            "tg_add_adjoint_res_xpt_products")

    def add_total_xpt_derivative(self, u, func, psi, dfdX, coef=1.0,
                                 scale=-1.0):
        check(_lib.lib().tg_add_total_xpt_derivative(
            self.handle, _p(u), int(func), coef, _p(psi), scale, _p(dfdX),
            _stream()), "tg_add_total_xpt_derivative")

    # ------------------------------------------------ element segments
    def set_segments(self, elem_ptr):
        ep = np.ascontiguousarray(elem_ptr, np.int32)
        check(_lib.lib().tg_assembler_set_segments(self.handle, len(ep) - 1,
                                                   ep.ctypes.data),
              "tg_assembler_set_segments")
        self.nseg = len(ep) - 1

    def eval_functions_segments(self, u, func, ks_weight=None):
        out = np.zeros(self.nseg)
        ksw = self.ks_weight if ks_weight is None else ks_weight
        check(_lib.lib().tg_eval_functions_segments(
            self.handle, _p(u), int(func), ksw, out.ctypes.data, _stream()),
            "tg_eval_functions_segments")
        return out

    def add_sv_sens_segments(self, u, func, dfdu, alpha=1.0):
        check(_lib.lib().tg_add_sv_sens_segments(
            self.handle, _p(u), int(func), alpha, _p(dfdu), _stream()),
            "tg_add_sv_sens_segments")

    def segment_ks_save(self, ks=None):
        """The per-range KS statistics of the last
        eval_functions_segments (3 per range), into a device tensor."""
        ks = torch.empty(3 * self.nseg, dtype=torch.float64,
                         device="cuda") if ks is None else ks
        check(_lib.lib().tg_segment_ks_save(self.handle, _p(ks), _stream()),
              "tg_segment_ks_save")
        return ks

    def segment_ks_restore(self, ks):
        """Make saved per-range KS statistics current again, for the
        sensitivities of the state they were evaluated at."""
        check(_lib.lib().tg_segment_ks_restore(self.handle, _p(ks),
                                               _stream()),
              "tg_segment_ks_restore")

    def add_total_derivative_segments(self, u, func, psi, dfdx, coef=1.0,
                                      scale=-1.0):
        check(_lib.lib().tg_add_total_derivative_segments(
            self.handle, _p(u), int(func), coef, _p(psi), scale, _p(dfdx),
            _stream()), "tg_add_total_derivative_segments")


def static_adjoint(model, force, m=100, nrestart=2, rtol=1e-12, atol=1e-30,
                   pc_kind=_lib.PC_ILU0, mixed=False, funcs=(0, 1),
                   lev_fill=0, direct=False):
    """Linear static solve + adjoint gradients on the GPU, following the
    reference harness (tests/integration_tests/static_analysis_base_test.py:
    359-427): K(u=0) and R(0), ILU(0), GMRES for R - f, functions, dfdu,
    adjoint solve with the same row-BC matrix, dfdx - psi^T dR/dx.  With
    direct, both solves use the complete factorisation (Direct) instead,
    refined to the relative residual rtol (or the FP64 floor) like the
    Krylov solves; direct="mixed" factors in FP32 and refines every solve in
    FP64 to the same relative residual.  `iters`
    then counts refinement steps."""
    dev = torch.device("cuda")
    u0 = model.vec()
    res = model.vec()
    mat = model.new_mat()
    model.assemble_jacobian(u0, mat, res)
    pc = ksm = dsol = None
    if direct:
        dsol = Direct(mat, precision=_lib.PREC_FP32 if direct == "mixed"
                      else _lib.PREC_FP64)
        dsol.factor()

        class _Exact:  # the solves' interface of Ksm
            iters = 0

            def solve(self, b):
                x = dsol.solve(b, rtol=rtol)
                self.iters = dsol.last_steps
                return x, 1
        ksm = _Exact()
    else:
        prec = _lib.PREC_FP32 if mixed else _lib.PREC_FP64
        pc = Pc(mat, pc_kind, prec, lev_fill=lev_fill)
        pc.factor()
        ksm = Ksm(mat, pc, m, nrestart, mixed)
        ksm.set_tolerances(rtol, atol)
    f = torch.as_tensor(np.asarray(force, np.float64), device=dev).clone()
    model.apply_bcs(f)
    res -= f
    ans, flag = ksm.solve(res)
    u = -ans
    iters, flags = [ksm.iters], [flag]
    fvals = model.eval_functions(u, funcs)
    grads, psis = [], []
    for k, fn in enumerate(funcs):
        dfdu = model.vec()
        model.add_sv_sens(u, [fn], [dfdu])
        model.apply_bcs(dfdu)
        psi, fl = ksm.solve(dfdu)
        iters.append(ksm.iters)
        flags.append(fl)
        g = model.dv_vec()
        model.add_total_derivative(u, fn, psi, g, 1.0, -1.0)
        grads.append(g)
        psis.append(psi)
    return dict(u=u, funcs=fvals, grads=grads, psis=psis, flag=flag,
                flags=flags, iters=iters, mat=mat, pc=pc, ksm=ksm,
                direct=dsol)


def batched_adjoint(model, loads, m=100, nrestart=50, rtol=1e-10, atol=1e-30,
                    pc_kind=_lib.PC_ILU0, mixed=False, func=1, lev_fill=0,
                    direct=False, direct_solver=None, mat=None):
    """Independent meshes (element / node segments set from the problem's
    seg_elem_ptr / seg_node_ptr) under several load cases, solved and
    differentiated together: one batched GMRES for all forward solves, the
    per-mesh function of each load case, one batched GMRES for all adjoint
    solves and the per-element total derivatives.

    loads: (nlc, ndof) device tensor of nodal forces.  Returns the states
    (nlc, ndof), per-mesh function values (nlc, nseg), per-element gradients
    (nlc, ndv), per-system iteration counts and convergence flags of both
    solves (index load_case * nseg + mesh).

    direct_solver (with the matrix mat it was made for): a Direct from an
    earlier call, whose analysis (ordering, supernodes, storage) is reused
    -- the next design of an optimisation loop refactors it only.  The
    direct solves are refined to the relative residual rtol (max norms)
    like the iterative ones; with direct="mixed" also until a step's
    correction is at most rtol |x| (Direct.solve's rtol, ftol), not to
    FP64 rounding.
    """
    prob = model.prob
    model.set_segments(prob["seg_elem_ptr"])
    nlc = loads.shape[0]
    u0 = model.vec()
    if direct_solver is not None:
        if mat is None:
            raise ValueError("direct_solver needs the matrix it was made for")
    else:
        mat = model.new_mat()
    model.assemble_jacobian(u0, mat, model.vec())
    if direct:
        # one complete factorisation of the block-diagonal matrix (FP32 with
        # FP64 refinement for direct="mixed"); every load case and mesh is
        # then solved directly (reported as converged in 0 iterations)
        dsol = direct_solver if direct_solver is not None else Direct(
            mat, precision=_lib.PREC_FP32 if direct == "mixed"
            else _lib.PREC_FP64)
        dsol.factor()
        nsys = nlc * model.nseg

        def solve_multi(B):
            # both precisions to the relative residual rtol of the
            # iterative path (the FP32 factorisation by FP64 refinement)
            X = dsol.solve(B.contiguous(), rtol=rtol)
            z = np.zeros(nsys, np.int32)
            return X, z, np.ones(nsys, np.int32), np.zeros(nsys), 1
    else:
        dsol = None
        prec = _lib.PREC_FP32 if mixed else _lib.PREC_FP64
        pc = Pc(mat, pc_kind, prec, lev_fill=lev_fill)
        pc.factor()
        ksm = Ksm(mat, pc, m, nrestart, mixed)
        ksm.set_tolerances(rtol, atol)
        ksm.set_segments(prob["seg_node_ptr"])
        solve_multi = ksm.solve_multi
    F = loads.clone()
    for lc in range(nlc):
        model.apply_bcs(F[lc])
    U, it_f, fl_f, rn_f, _ = solve_multi(F)
    fvals = np.zeros((nlc, model.nseg))
    dfdu = torch.zeros_like(U)
    # each load case's KS statistics, kept for its total derivative after
    # the adjoint solve (instead of evaluating the functions again)
    ks = torch.empty(nlc, 3 * model.nseg, dtype=torch.float64, device="cuda")
    for lc in range(nlc):
        fvals[lc] = model.eval_functions_segments(U[lc], func)
        model.segment_ks_save(ks[lc])
        model.add_sv_sens_segments(U[lc], func, dfdu[lc])
        model.apply_bcs(dfdu[lc])
    Psi, it_a, fl_a, rn_a, _ = solve_multi(dfdu)
    grads = torch.zeros(nlc, model.ndv, dtype=torch.float64, device="cuda")
    for lc in range(nlc):
        model.segment_ks_restore(ks[lc])
        model.add_total_derivative_segments(U[lc], func, Psi[lc], grads[lc],
                                            1.0, -1.0)
    return dict(u=U, funcs=fvals, grads=grads, iters_fwd=it_f, flags_fwd=fl_f,
                iters_adj=it_a, flags_adj=fl_a, psi=Psi, resnorm_fwd=rn_f,
                resnorm_adj=rn_a, direct=dsol if direct else None, mat=mat,
                ksm=None if direct else ksm)


def batch_loads(model):
    """Load cases of a meshes.batch_plates problem: the consistent pressure
    load (from the residual at u = 0) and one point load per seeded node."""
    prob = model.prob
    pn = np.asarray(prob["point_nodes"])
    nlc = 1 + pn.shape[1]
    F = torch.zeros(nlc, model.ndof, dtype=torch.float64, device="cuda")
    F[0] = -model.assemble_res(model.vec(), apply_bcs=False)
    idx = torch.as_tensor(model.vpn * pn + 2, device="cuda")
    for c in range(pn.shape[1]):
        F[1 + c, idx[:, c]] = float(prob["point_load"])
    return F
