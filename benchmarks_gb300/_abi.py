"""ctypes declarations of the C ABI in include/mfgb.h (libmfgb.so)."""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

OK, ERR_INVALID_ARG, ERR_OUT_OF_MEMORY, ERR_NOT_CONVERGED = 0, 1, 2, 3
ERR_TIMEOUT, ERR_NONFINITE, ERR_CUDA, ERR_UNSUPPORTED = 4, 5, 6, 7
ERR_RANGE = 8
ARITH_FP64, ARITH_FP64_DF, ARITH_FP32, ARITH_FP64_TC = 0, 1, 2, 3
INVALID_DOF = 0xFFFFFFFF


class MfgbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"mfgb status {status}: {message}")
        self.status = status


class BoxDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("degree", ctypes.c_int), ("lo", ctypes.c_double * 3),
                ("hi", ctypes.c_double * 3), ("amplitude", ctypes.c_double),
                ("geometry_degree", ctypes.c_int)]


class CgControl(ctypes.Structure):
    _fields_ = [("max_steps", ctypes.c_int), ("tol", ctypes.c_double),
                ("reduce", ctypes.c_double), ("arith", ctypes.c_int)]


class MgParams(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("chebyshev_degree", ctypes.c_int),
                ("smoothing_range", ctypes.c_double), ("eig_iterations", ctypes.c_int),
                ("coarse_cells", ctypes.c_int), ("coarse_tol", ctypes.c_double)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("initial", ctypes.c_double),
                ("last", ctypes.c_double), ("converged", ctypes.c_int)]


def library_path() -> str:
    return os.path.join(HERE, "libmfgb.so")


def lib():
    """Load libmfgb.so; raises if it has not been built (there is no CPU
    fallback for any operator call)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    P, I64, I32, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
    PP = ctypes.POINTER(ctypes.c_void_p)
    sigs = {
        "mfgb_status_string": ([I32], ctypes.c_char_p),
        "mfgb_last_error": ([], ctypes.c_char_p),
        "mfgb_version": ([], I32),
        "mfgb_set_kernel_shape": ([I32, I32, I32], I32),
        "mfgb_get_kernel_shape": ([I32, I32, ctypes.POINTER(I32)], I32),
        "mfgb_check_device_errors": ([P], I32),
        "mfgb_operator_create_box": ([ctypes.POINTER(BoxDesc), PP], I32),
        "mfgb_operator_create": ([I32, I64, I64, P, P, I64, P, PP], I32),
        "mfgb_operator_create_box_gauss": ([ctypes.POINTER(BoxDesc), PP], I32),
        "mfgb_operator_create_box_helmholtz": ([ctypes.POINTER(BoxDesc), PP], I32),
        "mfgb_operator_create_box_bp3": ([ctypes.POINTER(BoxDesc), PP], I32),
        "mfgb_operator_destroy": ([P], I32),
        "mfgb_operator_info": ([P, P, P, P, P], I32),
        "mfgb_operator_export": ([P, P, P, P], I32),
        "mfgb_vmult": ([P, P, P, I32, P], I32),
        "mfgb_vmult_add": ([P, P, P, I32, P], I32),
        "mfgb_vmult_f32": ([P, P, P, P], I32),
        "mfgb_vmult_host": ([P, P, P, I32, P], I32),
        "mfgb_set_host_pipeline": ([I32], I32),
        "mfgb_vmult_vector": ([P, P, P, I32, I32, P], I32),
        "mfgb_copy_constrained": ([P, P, P, P], I32),
        "mfgb_bk5_lvector": ([I32, I64, P, P, P, P, P, I32, P], I32),
        "mfgb_bk5_evector": ([I32, I64, P, P, P, P, I32, P], I32),
        "mfgb_compute_diagonal": ([P, P, P], I32),
        "mfgb_invert_diagonal": ([I64, P, P], I32),
        "mfgb_rhs_uniform": ([P, ctypes.c_uint64, P, P], I32),
        "mfgb_cg_solve": ([P, P, P, P, ctypes.POINTER(CgControl), ctypes.POINTER(SolveInfo), P],
                          I32),
        "mfgb_cg_solve_noalloc": ([P, P, P, P, ctypes.POINTER(CgControl),
                                   ctypes.POINTER(SolveInfo), P], I32),
        "mfgb_dot": ([I64, P, P, ctypes.POINTER(D), P], I32),
        "mfgb_pipe_rate": ([I32, I32, I32, ctypes.POINTER(D)], I32),
        "mfgb_link_rate": ([I32, I64, I32, ctypes.POINTER(D)], I32),
        "mfgb_cell_error_reduction": ([P, P, I32, ctypes.c_uint64, P, P], I32),
        "mfgb_test_fail_allocation": ([I32], I32),
        "mfgb_test_expire_copy_wait": ([I32], I32),
        "mfgb_mg_set_smoother_weights": ([P, P], I32),
        "mfgb_mlp_n_params": ([], I32),
        "mfgb_cell_features": ([P, P, P], I32),
        "mfgb_cell_lambda": ([P, P, I32, P], I32),
        "mfgb_mlp_loss_grad": ([P, P, P, I32, P, P], I32),
        "mfgb_mlp_train": ([P, P, P, I64, I32, I32, ctypes.c_float, ctypes.c_uint64, P], I32),
        "mfgb_mlp_forward_f32": ([P, P, I32, P], I32),
        "mfgb_mlp_infer": ([P, P, I64, P, P], I32),
        "mfgb_mg_setup": ([ctypes.POINTER(BoxDesc), ctypes.POINTER(MgParams), PP], I32),
        "mfgb_mg_setup_shared": ([P, ctypes.POINTER(MgParams), PP], I32),
        "mfgb_mg_destroy": ([P], I32),
        "mfgb_mg_info": ([P, P, P, P, P], I32),
        "mfgb_mg_vmult": ([P, P, P, P], I32),
        "mfgb_mg_cg_solve": ([P, P, P, P, ctypes.POINTER(CgControl), ctypes.POINTER(SolveInfo), P],
                             I32),
        "mfgb_bk1_evector": ([I32, I64, P, P, P, P, I32, P], I32),
        "mfgb_bk3_evector": ([I32, I64, P, P, P, P, P, I32, P], I32),
        "mfgb_batch_create": ([ctypes.POINTER(BoxDesc), I32, ctypes.POINTER(MgParams), PP], I32),
        "mfgb_batch_destroy": ([P], I32),
        "mfgb_batch_info": ([P, P, P, P, P, P], I32),
        "mfgb_batch_rhs_uniform": ([P, P, P, P], I32),
        "mfgb_batch_vmult": ([P, P, P, P], I32),
        "mfgb_batch_precondition": ([P, P, P, P], I32),
        "mfgb_batch_cg_solve": ([P, P, P, ctypes.POINTER(CgControl), P, P], I32),
        "mfgb_batch_last_solve_stats": ([P, ctypes.POINTER(I32)], I32),
        "mfgb_batch_last_solve_launches": ([P, ctypes.POINTER(I32)], I32),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _LIB = L
    return L


def check(status: int) -> None:
    if status != OK:
        raise MfgbError(status, lib().mfgb_last_error().decode(errors="replace"))
