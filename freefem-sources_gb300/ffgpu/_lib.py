"""ctypes binding of libffgpu.so (the C ABI declared in include/ffgpu.h).

The library is built in-tree by ``ffgpu.build.build()``.  There is no fallback: if the
shared object is missing or no GPU is visible, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "lib", "libffgpu.so")

FFGPU_OK = 0
ERRORS = {-1: "EINVAL", -2: "ECUDA", -3: "ENOCONV", -4: "EMESH", -5: "ENOMEM"}
FE_P0, FE_P1, FE_P2, FE_P2VEC3 = 0, 1, 2, 3
FORM_DIFFUSION, FORM_ELASTICITY = 0, 1

# every symbol include/ffgpu.h declares
EXPORTS = [
    "ffgpu_ctx_create", "ffgpu_ctx_destroy", "ffgpu_last_error", "ffgpu_ctx_kernel_launches",
    "ffgpu_ctx_stream",
    "ffgpu_space_create", "ffgpu_space_destroy", "ffgpu_space_set_boundary", "ffgpu_space_bc_mask", "ffgpu_matrix_assemble", "ffgpu_matrix_reassemble",
    "ffgpu_rhs_assemble", "ffgpu_matrix_from_csr", "ffgpu_matrix_destroy", "ffgpu_matrix_info",
    "ffgpu_matrix_spmv_layout",
    "ffgpu_matrix_time_spmv",
    "ffgpu_matrix_text_read",
    "ffgpu_matrix_text_write",
    "ffgpu_mesh_sizes",
    "ffgpu_mesh_build",
    "ffgpu_number_p2", "ffgpu_number_p2_2d", "ffgpu_gibbs_renumber",
    "ffgpu_matrix_csr", "ffgpu_matrix_mult", "ffgpu_solve_cg", "ffgpu_solve_gmres",
    "ffgpu_matrix_to_f32", "ffgpu_solve_ir", "ffgpu_diffusion_sensitivity",
    "ffgpu_solve_cg_csr_noalloc", "ffgpu_direct_method", "ffgpu_direct_factor", "ffgpu_solve_direct",
    "ffgpu_solve_direct_trans",
    "ffgpu_batch_create", "ffgpu_batch_assemble", "ffgpu_batch_solve", "ffgpu_batch_rhs",
    "ffgpu_batch_matrix", "ffgpu_batch_info", "ffgpu_batch_destroy",
]


class BTerm(C.Structure):
    _fields_ = [("nlabels", C.c_int), ("labels", C.c_void_p), ("robin", C.c_void_p),
                ("robin_const", C.c_double), ("g", C.c_void_p), ("g_const", C.c_double * 3)]


class FEFuncC(C.Structure):
    _fields_ = [("kind", C.c_int), ("values", C.c_void_p), ("dof", C.c_void_p)]


class ExprC(C.Structure):
    _fields_ = [("nops", C.c_int), ("ops", C.c_void_p), ("consts", C.c_void_p), ("nfe", C.c_int),
                ("fe", C.c_void_p)]


class TermC(C.Structure):
    _fields_ = [("iop", C.c_int), ("jop", C.c_int), ("c", C.c_double), ("expr", C.c_void_p)]


class Varf(C.Structure):
    _fields_ = [("form", C.c_int), ("kappa", C.c_void_p), ("c_stiff", C.c_double),
                ("c_mass", C.c_double), ("E", C.c_double), ("nu", C.c_double),
                ("f", C.c_void_p), ("f_const", C.c_double * 3), ("nbterms", C.c_int),
                ("bterms", C.c_void_p), ("nqp", C.c_int), ("qp_lambda", C.c_void_p),
                ("qp_weight", C.c_void_p), ("f_qp", C.c_void_p), ("mass_qp", C.c_void_p),
                ("stiff_qp", C.c_void_p), ("lame", C.c_void_p), ("f_expr", C.c_void_p),
                ("nterms", C.c_int), ("terms", C.c_void_p)]


class BC(C.Structure):
    _fields_ = [("onbc", C.c_void_p), ("g", C.c_void_p), ("tgv", C.c_double), ("nlabels", C.c_int),
                ("labels", C.c_void_p), ("comp_mask", C.c_int)]


class SolverParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("itmax", C.c_int), ("dim_krylov", C.c_int),
                ("tgv", C.c_double), ("verb", C.c_int), ("unroll", C.c_int), ("spmv_mode", C.c_int),
                ("spmv_layout", C.c_int)]


class SolverStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("gcg", C.c_double),
                ("eps2", C.c_double), ("residual", C.c_double), ("outer_iterations", C.c_int),
                ("elapsed_ms", C.c_double)]


class IRParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("eps_inner", C.c_double), ("itmax_inner", C.c_int),
                ("max_outer", C.c_int), ("tgv", C.c_double), ("unroll", C.c_int),
                ("restart_inner", C.c_int)]


class FFGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ffgpu error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError(f"libffgpu.so not built ({LIBPATH}); run ffgpu.build.build()")
    L = C.CDLL(LIBPATH)
    vp, i32, i64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_double
    P = C.POINTER
    sig = {
        "ffgpu_ctx_create": (i32, [i32, P(vp)]),
        "ffgpu_ctx_destroy": (i32, [vp]),
        "ffgpu_last_error": (C.c_char_p, []),
        "ffgpu_ctx_kernel_launches": (i64, [vp]),
        "ffgpu_ctx_stream": (vp, [vp]),
        "ffgpu_space_create": (i32, [vp, i32, i32, vp, i32, vp, i32, i32, vp, i32, P(vp)]),
        "ffgpu_space_destroy": (i32, [vp]),
        "ffgpu_space_set_boundary": (i32, [vp, i32, vp, vp]),
        "ffgpu_space_bc_mask": (i32, [vp, i32, vp, i32, vp]),
        "ffgpu_matrix_assemble": (i32, [vp, P(Varf), P(BC), vp, P(vp)]),
        "ffgpu_matrix_reassemble": (i32, [vp, P(Varf), P(BC), vp]),
        "ffgpu_rhs_assemble": (i32, [vp, P(Varf), P(BC), vp]),
        "ffgpu_matrix_from_csr": (i32, [vp, i32, i64, vp, vp, vp, P(vp)]),
        "ffgpu_matrix_destroy": (i32, [vp]),
        "ffgpu_matrix_info": (i32, [vp, P(i32), P(i64), P(i32)]),
        "ffgpu_matrix_spmv_layout": (i32, [vp, i32]),
        "ffgpu_matrix_time_spmv": (i32, [vp, i32, i32, P(C.c_float)]),
        "ffgpu_matrix_text_read": (i32, [C.c_char_p, P(i32), P(i32), P(i64), P(i32), vp, vp, vp]),
        "ffgpu_matrix_text_write": (i32, [C.c_char_p, i32, i32, i32, i32, vp, vp, vp]),
        "ffgpu_mesh_sizes": (i32, [i32, i32, i32, i32, P(i32), P(i32), P(i32)]),
        "ffgpu_mesh_build": (i32, [vp, i32, i32, i32, i32, vp, vp, vp, vp]),
        "ffgpu_number_p2": (i32, [vp, i32, i32, vp, vp, P(i32)]),
        "ffgpu_number_p2_2d": (i32, [i32, i32, vp, vp, P(i32)]),
        "ffgpu_gibbs_renumber": (i32, [i64, vp, vp, vp, P(i64), P(i64)]),
        "ffgpu_matrix_csr": (i32, [vp, vp, vp, vp]),
        "ffgpu_matrix_mult": (i32, [vp, vp, vp, i32]),
        "ffgpu_solve_cg": (i32, [vp, vp, vp, i32, i32, P(SolverParams), P(SolverStats)]),
        "ffgpu_solve_gmres": (i32, [vp, vp, vp, i32, i32, P(SolverParams), P(SolverStats)]),
        "ffgpu_matrix_to_f32": (i32, [vp]),
        "ffgpu_direct_method": (i32, [vp, i32]),
        "ffgpu_direct_factor": (i32, [vp]),
        "ffgpu_solve_direct": (i32, [vp, vp, vp, i32, P(SolverStats)]),
        "ffgpu_solve_direct_trans": (i32, [vp, vp, vp, i32, i32, P(SolverStats)]),
        "ffgpu_solve_ir": (i32, [vp, vp, vp, P(IRParams), P(SolverStats)]),
        "ffgpu_diffusion_sensitivity": (i32, [vp, vp, vp, dbl, vp, vp]),
        "ffgpu_solve_cg_csr_noalloc": (i32, [i32, i64, vp, vp, vp, vp, vp, dbl, i32, dbl, vp,
                                              P(i32), vp]),
        "ffgpu_batch_create": (i32, [vp, i32, vp, vp, vp, vp, P(vp)]),
        "ffgpu_batch_assemble": (i32, [vp, vp, dbl, vp, dbl]),
        "ffgpu_batch_solve": (i32, [vp, vp, P(IRParams), vp, P(SolverStats)]),
        "ffgpu_batch_rhs": (i32, [vp, vp]),
        "ffgpu_batch_matrix": (vp, [vp]),
        "ffgpu_batch_info": (i32, [vp, P(i32), P(i32), P(C.c_float)]),
        "ffgpu_batch_destroy": (i32, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(code: int) -> int:
    if code != FFGPU_OK:
        msg = lib().ffgpu_last_error()
        raise FFGPUError(code, msg.decode() if msg else "")
    return code
