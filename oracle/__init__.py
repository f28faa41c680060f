"""CPU oracle for the TACS hot path -- test infrastructure.

``liboracle.so`` (built from ``tacs_oracle.c`` by :func:`build`) is a plain-C
restatement of the reference algorithms, pinned against the reference's own
outputs in ``tests/golden``.  Only the tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` load it; the GPU package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


def build(force=False):
    src = os.path.join(HERE, "tacs_oracle.c")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(src)):
        return LIB
    subprocess.run(["gcc", "-O3", "-std=c99", "-fPIC", "-shared", "-o", LIB,
                    src, "-lm", "-lpthread"], check=True)
    return LIB


class _Problem(C.Structure):
    _fields_ = [
        ("elem_type", C.c_int), ("nnodes", C.c_int), ("nelem", C.c_int),
        ("xpts", C.c_void_p), ("conn", C.c_void_p), ("thick", C.c_void_p),
        ("dvnum", C.c_void_p), ("rho", C.c_double), ("E", C.c_double),
        ("nu", C.c_double), ("ys", C.c_double), ("transform", C.c_int),
        ("ref_axis", C.c_double * 3), ("nbcs", C.c_int),
        ("bc_nodes", C.c_void_p), ("bc_masks", C.c_void_p),
        ("npres", C.c_int), ("pres_elems", C.c_void_p),
        ("pres_vals", C.c_void_p), ("ntrac", C.c_int),
        ("trac_elems", C.c_void_p), ("trac_faces", C.c_void_p),
        ("trac_vals", C.c_void_p), ("ks_weight", C.c_double),
        ("nthreads", C.c_int),
    ]


class _Bcsr(C.Structure):
    _fields_ = [("bsize", C.c_int), ("nrows", C.c_int),
                ("rowp", C.POINTER(C.c_int)), ("cols", C.POINTER(C.c_int)),
                ("diag", C.POINTER(C.c_int)),
                ("vals", C.POINTER(C.c_double))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Oracle:
    """Holds one problem (the dict produced by tacs_gb300.meshes)."""

    def __init__(self, prob, nthreads=1):
        L = lib()
        self.L = L
        self.keep = {}
        get = lambda k, dt: self.keep.setdefault(  # noqa: E731
            k, np.ascontiguousarray(prob[k], dtype=dt))
        P = _Problem()
        P.elem_type = int(prob["elem_type"])
        P.nnodes, P.nelem = int(prob["nnodes"]), int(prob["nelem"])
        P.xpts = _ptr(get("xpts", np.float64))
        P.conn = _ptr(get("conn", np.int32))
        P.thick = _ptr(get("thick", np.float64))
        P.dvnum = _ptr(get("dvnum", np.int32))
        rho, E, nu, ys = [float(v) for v in prob["mat"]]
        P.rho, P.E, P.nu, P.ys = rho, E, nu, ys
        P.transform = int(prob.get("transform", 0))
        ax = np.asarray(prob.get("ref_axis", [1.0, 0.0, 0.0]), np.float64)
        for i in range(3):
            P.ref_axis[i] = float(ax[i])
        bcn = get("bc_nodes", np.int32)
        P.nbcs = len(bcn)
        P.bc_nodes, P.bc_masks = _ptr(bcn), _ptr(get("bc_masks", np.int32))
        pe = get("pres_elems", np.int32)
        P.npres, P.pres_elems = len(pe), _ptr(pe)
        P.pres_vals = _ptr(get("pres_vals", np.float64))
        te = get("trac_elems", np.int32)
        P.ntrac, P.trac_elems = len(te), _ptr(te)
        P.trac_faces = _ptr(get("trac_faces", np.int32))
        P.trac_vals = _ptr(get("trac_vals", np.float64))
        P.ks_weight = float(prob.get("ks_weight", 100.0))
        P.nthreads = int(nthreads)
        self.P = P
        self.vpn = 6 if P.elem_type == 0 else 3
        self.ndof = self.vpn * P.nnodes
        self.ndv = int(np.max(self.keep["dvnum"])) + 1 if P.nelem else 0
        self.prob = prob

    # -- assembly ---------------------------------------------------------
    def assemble_res(self, vars_, lam=1.0, apply_bcs=True):
        u = np.ascontiguousarray(vars_, np.float64)
        r = np.zeros(self.ndof)
        self.L.or_assemble_res(C.byref(self.P), _ptr(u), C.c_double(lam),
                               int(apply_bcs), _ptr(r))
        return r

    def new_bcsr(self):
        A = _Bcsr()
        self.L.or_bcsr_create(C.byref(self.P), C.byref(A))
        return A

    @staticmethod
    def bcsr_arrays(A):
        n = A.nrows
        rowp = np.ctypeslib.as_array(A.rowp, (n + 1,)).copy()
        nnz = int(rowp[-1])
        cols = np.ctypeslib.as_array(A.cols, (nnz,)).copy()
        vals = np.ctypeslib.as_array(A.vals,
                                     (nnz * A.bsize * A.bsize,)).copy()
        return rowp, cols, vals

    def assemble_jac(self, vars_, A=None, transpose=False, apply_bcs=True):
        A = A or self.new_bcsr()
        u = np.ascontiguousarray(vars_, np.float64)
        r = np.zeros(self.ndof)
        self.L.or_assemble_jac(C.byref(self.P), _ptr(u), _ptr(r), C.byref(A),
                               int(transpose), int(apply_bcs))
        return r, A

    def mult(self, A, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.L.or_bcsr_mult(C.byref(A), _ptr(x), _ptr(y), self.P.nthreads)
        return y

    def ilu0(self, A):
        F = _Bcsr()
        fail = self.L.or_ilu0_factor(C.byref(A), C.byref(F))
        return F, fail

    def iluk(self, A, lev_fill):
        """ILU(lev_fill) factor (its own pattern) of A."""
        F = _Bcsr()
        fail = self.L.or_iluk_factor(C.byref(A), int(lev_fill), C.byref(F))
        return F, fail

    def ilu0_apply(self, F, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.L.or_ilu0_apply(C.byref(F), _ptr(x), _ptr(y))
        return y

    def gmres(self, A, F, b, m=100, nrestart=2, rtol=1e-12, atol=1e-30):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros_like(b)
        it = C.c_int(0)
        flag = self.L.or_gmres(C.byref(A), C.byref(F), _ptr(b), _ptr(x), m,
                               nrestart, C.c_double(rtol), C.c_double(atol),
                               C.byref(it), self.P.nthreads)
        return x, flag, it.value

    def free(self, A):
        self.L.or_bcsr_free(C.byref(A))

    # -- functions --------------------------------------------------------
    def eval_funcs(self, vars_):
        u = np.ascontiguousarray(vars_, np.float64)
        f = np.zeros(2)
        self.L.or_eval_funcs(C.byref(self.P), _ptr(u), _ptr(f))
        return f

    def sv_sens(self, vars_, which):
        u = np.ascontiguousarray(vars_, np.float64)
        d = np.zeros(self.ndof)
        self.L.or_add_sv_sens(C.byref(self.P), _ptr(u), int(which), _ptr(d))
        return d

    def dv_sens(self, vars_, which, scale=1.0):
        u = np.ascontiguousarray(vars_, np.float64)
        d = np.zeros(self.ndv)
        self.L.or_add_dv_sens(C.byref(self.P), _ptr(u), int(which),
                              C.c_double(scale), _ptr(d))
        return d

    def adj_res_product(self, vars_, psi, scale=1.0):
        u = np.ascontiguousarray(vars_, np.float64)
        ps = np.ascontiguousarray(psi, np.float64)
        d = np.zeros(self.ndv)
        self.L.or_add_adj_res_product(C.byref(self.P), _ptr(u), _ptr(ps),
                                      C.c_double(scale), _ptr(d))
        return d

    def xpt_sens(self, vars_, which, coef=1.0):
        u = np.ascontiguousarray(vars_, np.float64)
        d = np.zeros(3 * self.P.nnodes)
        self.L.or_add_xpt_sens(C.byref(self.P), _ptr(u), int(which),
                               C.c_double(coef), _ptr(d))
        return d

    def adj_res_xpt_product(self, vars_, psi, scale=1.0, lam=1.0):
        u = np.ascontiguousarray(vars_, np.float64)
        ps = np.ascontiguousarray(psi, np.float64)
        d = np.zeros(3 * self.P.nnodes)
        self.L.or_add_adj_res_xpt_product(C.byref(self.P), _ptr(u), _ptr(ps),
                                          C.c_double(scale), C.c_double(lam),
                                          _ptr(d))
        return d

    def static_adjoint(self, force, m=100, nrestart=2, rtol=1e-12,
                       atol=1e-30, grads=True):
        f = np.ascontiguousarray(force, np.float64)
        u = np.zeros(self.ndof)
        fv = np.zeros(2)
        gc = np.zeros(self.ndv) if grads else None
        gk = np.zeros(self.ndv) if grads else None
        it = (C.c_int * 3)()
        flag = self.L.or_static_adjoint(C.byref(self.P), m, nrestart,
                                        C.c_double(rtol), C.c_double(atol),
                                        _ptr(f), _ptr(u), _ptr(fv), _ptr(gc),
                                        _ptr(gk), it)
        return dict(u=u, funcs=fv, grad_comp=gc, grad_ks=gk, flag=flag,
                    iters=list(it))
