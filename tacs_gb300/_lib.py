"""ctypes binding of libtacs_gb300.so (the C ABI in include/tacs_gb300.h).

The library is loaded from the package directory; there is no fallback:
if it is missing or no CUDA device is present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtacs_gb300.so")

ELEM_MITC4, ELEM_HEX8 = 0, 1
MAT_NORMAL, MAT_TRANSPOSE = 0, 1
PC_ILU0, PC_BLOCK_JACOBI, PC_ILU0_COLORED, PC_DIRECT = 0, 1, 2, 3
XPT_FORWARD, XPT_REVERSE = 0, 1
PREC_FP64, PREC_FP32 = 0, 1
FUNC_COMPLIANCE, FUNC_KS_FAILURE = 0, 1

ERR_ARG, ERR_CUDA, ERR_STATE, ERR_PIVOT, ERR_NOCONV, ERR_NONFINITE = \
    -1, -2, -3, -4, -5, -6
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "bad call order",
          -4: "zero pivot", -5: "no convergence", -6: "non-finite value"}

# (name, restype, argtypes)
_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)
SIGNATURES = [
    ("tg_last_error", C.c_char_p, []),
    ("tg_version", _I, []),
    ("tg_assembler_create", _I, [_I, _I, _I, _P, _D, _D, _D, _D, _I, _P,
                                 C.POINTER(_P)]),
    ("tg_assembler_incref", _I, [_P]),
    ("tg_assembler_decref", _I, [_P]),
    ("tg_assembler_get_sizes", _I, [_P, _IP, _IP, _IP, _IP, _IP]),
    ("tg_assembler_add_bcs", _I, [_P, _I, _P, _P]),
    ("tg_assembler_set_element_dvs", _I, [_P, _P, _P]),
    ("tg_assembler_initialize", _I, [_P]),
    ("tg_assembler_set_nodes", _I, [_P, _P, _P]),
    ("tg_assembler_set_design_vars", _I, [_P, _P, _P]),
    ("tg_assembler_set_pressure", _I, [_P, _I, _P, _P]),
    ("tg_assembler_set_traction", _I, [_P, _I, _P, _P, _P]),
    ("tg_assembler_set_fixed_geometry", _I, [_P, _I]),
    ("tg_assembler_get_fixed_geometry", _I, [_P, _IP, _DP, _DP]),
    ("tg_assemble_res", _I, [_P, _P, _D, _I, _P, _P]),
    ("tg_assemble_jacobian", _I, [_P, _D, _D, _D, _P, _P, _P, _I, _D, _I,
                                  _P]),
    ("tg_apply_bcs", _I, [_P, _P, _P]),
    ("tg_eval_functions", _I, [_P, _P, _I, _P, _D, _P, _P]),
    ("tg_add_sv_sens", _I, [_P, _P, _I, _P, _D, _P, _P]),
    ("tg_add_dv_sens", _I, [_P, _P, _I, _P, _D, _P, _P]),
    ("tg_add_adjoint_res_products", _I, [_P, _P, _D, _I, _P, _P, _P]),
    ("tg_add_total_derivative", _I, [_P, _P, _I, _D, _P, _D, _P, _P]),
    ("tg_direct_create", _I, [_P, _I, _I, _P]),
    ("tg_direct_factor", _I, [_P, _P]),
    ("tg_direct_solve", _I, [_P, _P, _P, _P]),
    ("tg_direct_solve_multi", _I, [_P, _I, _P, _P, _P]),
    ("tg_direct_solve_f32", _I, [_P, _P, _P, _P]),
    ("tg_direct_solve_refined", _I, [_P, _P, _P, _I, _P]),
    ("tg_direct_solve_refined_tol", _I, [_P, _P, _P, _I, _D, _IP,
                                         C.POINTER(C.c_double), _P]),
    ("tg_direct_solve_refined_multi", _I, [_P, _I, _P, _P, _I, _D, _D, _D,
                                           _P, _P, _P]),
    ("tg_direct_autotune", _I, [_P, _IP, _P, _P]),
    ("tg_direct_get_stats", _I, [_P, _P]),
    ("tg_direct_decref", _I, [_P]),
    ("tg_add_xpt_sens", _I, [_P, _P, _I, _P, _D, _P, _P]),
    ("tg_set_xpt_mode", _I, [_P, _I]),
    ("tg_add_adjoint_res_xpt_products", _I, [_P, _P, _D, _I, _P, _P, _D, _P]),
    ("tg_add_total_xpt_derivative", _I, [_P, _P, _I, _D, _P, _D, _P, _P]),
    ("tg_mat_create", _I, [_P, C.POINTER(_P)]),
    ("tg_mat_decref", _I, [_P]),
    ("tg_mat_get_arrays", _I, [_P, _IP, _IP, C.POINTER(_P), C.POINTER(_P),
                               C.POINTER(_P)]),
    ("tg_mat_mult", _I, [_P, _P, _P, _P]),
    ("tg_mat_mult_f32", _I, [_P, _P, _P, _P]),
    ("tg_pc_create", _I, [_P, _I, _I, C.POINTER(_P)]),
    ("tg_pc_create_iluk", _I, [_P, _I, _I, _P]),
    ("tg_pc_create_direct", _I, [_P, C.POINTER(_P)]),
    ("tg_pc_get_fp64_used", _I, [_P, _IP]),
    ("tg_pc_get_fill", _I, [_P, _P, _P]),
    ("tg_pc_decref", _I, [_P]),
    ("tg_pc_factor", _I, [_P, _P]),
    ("tg_pc_apply", _I, [_P, _P, _P, _P]),
    ("tg_ksm_create", _I, [_P, _P, _I, _I, _I, C.POINTER(_P)]),
    ("tg_ksm_decref", _I, [_P]),
    ("tg_ksm_set_tolerances", _I, [_P, _D, _D]),
    ("tg_ksm_solve", _I, [_P, _P, _P, _I, _IP, _DP, _P]),
    ("tg_ksm_set_segments", _I, [_P, _I, _P]),
    ("tg_pc_get_schedule", _I, [_P, _IP, _IP, _IP, _P]),
    ("tg_vec_axpy", _I, [_D, _P, _P, C.c_long, _P]),
    ("tg_vec_scale", _I, [_D, _P, C.c_long, _P]),
    ("tg_vec_dot", _I, [_P, _P, C.c_long, _DP, _P]),
    ("tg_assembler_set_segments", _I, [_P, _I, _P]),
    ("tg_eval_functions_segments", _I, [_P, _P, _I, _D, _P, _P]),
    ("tg_add_sv_sens_segments", _I, [_P, _P, _I, _D, _P, _P]),
    ("tg_add_total_derivative_segments", _I, [_P, _P, _I, _D, _P, _D, _P,
                                              _P]),
    ("tg_segment_ks_save", _I, [_P, _P, _P]),
    ("tg_segment_ks_restore", _I, [_P, _P, _P]),
    ("tg_ksm_solve_multi", _I, [_P, _I, _P, _P, _I, _P, _P, _P, _P]),
    ("tg_ksm_get_graph_info", _I, [_P, _IP, _IP, _IP]),
    ("tg_eval_functions_noalloc", _I, [_I, _I, _P, _P, _P, _D, _D, _D, _I,
                                       _P, _P, _D, _P, _P]),
]

_lib = None


class TacsGpuError(RuntimeError):
    pass


def lib():
    """Load libtacs_gb300.so; raise if it is missing (no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise TacsGpuError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, what=""):
    """Raise TacsGpuError for a negative status; return rc otherwise."""
    if rc < 0:
        msg = lib().tg_last_error().decode(errors="replace")
        raise TacsGpuError(f"{what}: {ERRORS.get(rc, rc)}: {msg}")
    return rc


def exported_symbols():
    return [s[0] for s in SIGNATURES]
