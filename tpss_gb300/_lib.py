"""ctypes binding of libtpss_gpu.so (the C ABI declared in include/tpss_gpu.h).

The library is built in-tree by tpss_gb300/build.py.  There is no fallback: when the
shared library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

TPSS_OK = 0
TPSS_ERR_INVALID_ARGUMENT = 1
TPSS_ERR_NOT_IMPLEMENTED = 2
TPSS_ERR_CUDA = 3
TPSS_ERR_OUT_OF_MEMORY = 4
TPSS_ERR_NOT_FINITE = 5
TPSS_ERR_NOT_CONVERGED = 6
TPSS_ERR_STATE = 7

TPSS_DOF_DGQ = 0
TPSS_PATCH_CELL = 0
TPSS_PATCH_VERTEX = 1
TPSS_ADDITIVE = 0
TPSS_MULTIPLICATIVE = 1
TPSS_FP64 = 0
TPSS_FP32 = 1
TPSS_KERNEL_AUTO = 0
TPSS_KERNEL_COLOR = 1
TPSS_KERNEL_STREAM = 2
TPSS_PENALTY_REFERENCE = 0
TPSS_PENALTY_2KP1SQ = 1


class TPSSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[tpss status {code}] {msg}")
        self.code = code


class TPSSNotImplemented(TPSSError, NotImplementedError):
    pass


class TPSSInvalidArgument(TPSSError, ValueError):
    pass


class TPSSNotConverged(TPSSError):
    pass


class LayoutDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("degree", C.c_int), ("dof_layout", C.c_int),
                ("patch_variant", C.c_int), ("smoother_variant", C.c_int),
                ("n_cells", C.c_int * 3), ("cell_h", C.POINTER(C.c_double) * 3),
                ("cell_dof_start", C.POINTER(C.c_int64)), ("patch_color", C.POINTER(C.c_int32)),
                ("vertex_coords", C.POINTER(C.c_double)), ("surrogate_n_q", C.c_int)]


class PrecondDesc(C.Structure):
    _fields_ = [("relaxation", C.c_double), ("reverse", C.c_int), ("symmetrized", C.c_int),
                ("use_ras_weights", C.c_int), ("use_ras_boolean_weights", C.c_int),
                ("precision", C.c_int), ("ip_factor", C.c_double), ("check_finite", C.c_int),
                ("kernel_variant", C.c_int), ("stream_variant", C.c_int),
                ("local_solver", C.c_int), ("model", C.c_void_p), ("penalty_mode", C.c_int)]


class C0ipDesc(C.Structure):
    _fields_ = [("degree", C.c_int), ("n_rep", C.c_int), ("n_cells_fine", C.c_int),
                ("ip_factor", C.c_double), ("local_solver", C.c_int), ("precision", C.c_int),
                ("relaxation", C.c_double), ("problem", C.c_int)]


class MlpDesc(C.Structure):
    _fields_ = [("n_in", C.c_int), ("n_hidden", C.c_int), ("n_hidden_layers", C.c_int),
                ("n_out", C.c_int), ("seed", C.c_uint64)]


class TimeInfo(C.Structure):
    _fields_ = [("time", C.c_double), ("n_calls", C.c_int64), ("description", C.c_char * 64)]


class MgDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("degree", C.c_int), ("n_rep", C.c_int),
                ("n_cells_fine", C.c_int), ("ip_factor", C.c_double),
                ("patch_variant", C.c_int), ("smoother_variant", C.c_int),
                ("relaxation", C.c_double), ("precision", C.c_int), ("coarse_tol", C.c_double),
                ("coarse_solver", C.c_int), ("use_graph", C.c_int),
                ("vertex_coords", C.POINTER(C.c_double)), ("surrogate_n_q", C.c_int),
                ("local_solver", C.c_int), ("model", C.c_void_p), ("auto_relaxation", C.c_int),
                ("vcycle_precision", C.c_int), ("penalty_mode", C.c_int), ("fp64_level_mask", C.c_int),
                ("autotune", C.c_int)]


_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)

# symbol -> (restype, argtypes); every symbol declared in include/tpss_gpu.h
SIGNATURES = {
    "tpss_layout_create": (C.c_int, [C.POINTER(LayoutDesc), C.POINTER(_vp)]),
    "tpss_layout_info": (C.c_int, [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    "tpss_layout_patches": (C.c_int, [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "tpss_layout_destroy": (None, [_vp]),
    "tpss_operator_create": (C.c_int, [_vp, C.c_double, C.POINTER(_vp)]),
    "tpss_operator_create_penalty": (C.c_int, [_vp, C.c_double, C.c_int, C.POINTER(_vp)]),
    "tpss_operator_vmult": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_operator_vmult_fp32": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_operator_destroy": (None, [_vp]),
    "tpss_precond_create": (C.c_int, [_vp, _vp, C.POINTER(PrecondDesc), C.POINTER(_vp)]),
    "tpss_precond_create_shallow": (C.c_int, [_vp, C.POINTER(PrecondDesc), C.POINTER(_vp)]),
    "tpss_precond_vmult": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_precond_vmult_add": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_precond_Tvmult": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_precond_vmult_static_scratch": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_precond_vmult_host": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_precond_autotune": (C.c_int, [_vp, _vp, _vp, C.c_int, C.POINTER(C.c_int), _dp,
                                        C.POINTER(C.c_int), _vp]),
    "tpss_precond_time_info": (C.c_int, [_vp, C.POINTER(TimeInfo), C.POINTER(C.c_int)]),
    "tpss_precond_destroy": (None, [_vp]),
    "tpss_smoother_create": (C.c_int, [_vp, _vp, C.c_int, C.c_double, C.POINTER(_vp)]),
    "tpss_smoother_step": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_smoother_vmult": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_smoother_destroy": (None, [_vp]),
    "tpss_mg_create": (C.c_int, [C.POINTER(MgDesc), C.POINTER(_vp)]),
    "tpss_mg_n_dofs": (C.c_int, [_vp, C.POINTER(C.c_int64)]),
    "tpss_mg_vmult": (C.c_int, [_vp, _vp, _vp, _vp]),
    "tpss_mg_cg_solve": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_double, C.c_int,
                                   C.POINTER(C.c_int), _dp, _vp]),
    "tpss_mg_level": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)]),
    "tpss_mg_n_levels": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "tpss_mg_destroy": (None, [_vp]),
    "tpss_transfer_prolongate_add": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int), _vp, _vp, _vp]),
    "tpss_transfer_restrict_add": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int), _vp, _vp, _vp]),
    "tpss_diag_fma_peak": (C.c_int, [C.c_int, C.c_int, _dp, _vp]),
    "tpss_mg_relaxation": (C.c_int, [_vp, C.c_int, _dp, _dp]),
    "tpss_c0ip_create": (C.c_int, [C.POINTER(C0ipDesc), C.POINTER(_vp)]),
    "tpss_c0ip_info": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    "tpss_c0ip_operator_vmult": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "tpss_c0ip_smoother_vmult": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "tpss_c0ip_cg_solve": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_double, C.c_int,
                                     C.POINTER(C.c_int), _dp, _vp]),
    "tpss_c0ip_destroy": (None, [_vp]),
    "tpss_batch_create": (C.c_int, [C.POINTER(MgDesc), C.c_int, C.c_int, C.POINTER(_vp)]),
    "tpss_batch_problem": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "tpss_batch_solve": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.c_double, C.c_double, C.c_int,
                                   C.POINTER(C.c_int), _vp]),
    "tpss_batch_destroy": (None, [_vp]),
    "tpss_mlp_create": (C.c_int, [C.POINTER(MlpDesc), C.POINTER(_vp)]),
    "tpss_mlp_sizes": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "tpss_mlp_n_params": (C.c_int, [_vp, C.POINTER(C.c_int64)]),
    "tpss_mlp_get_params": (C.c_int, [_vp, _fp]),
    "tpss_mlp_set_params": (C.c_int, [_vp, _fp]),
    "tpss_mlp_forward": (C.c_int, [_vp, _vp, C.c_int64, _vp, _vp]),
    "tpss_mlp_loss_grad": (C.c_int, [_vp, _vp, _vp, C.c_int64, _dp, _fp]),
    "tpss_mlp_eval_loss": (C.c_int, [_vp, _vp, _vp, C.c_int64, _dp]),
    "tpss_mlp_train": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int, C.c_int, C.c_double, C.c_uint64,
                                 _dp, _vp]),
    "tpss_mlp_destroy": (None, [_vp]),
    "tpss_learned_sizes": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "tpss_learned_features": (C.c_int, [_vp, _vp]),
    "tpss_learned_targets": (C.c_int, [_vp, _vp, C.c_double, _vp]),
    "tpss_local_matrices": (C.c_int, [_vp, _vp, C.c_int64, C.c_int64, _vp]),
    "tpss_precond_local_inverse": (C.c_int, [_vp, C.c_int64, C.c_int64, _vp]),
    "tpss_kronecker_approx": (C.c_int, [_vp, C.c_int64, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.c_int, C.c_int, _vp, _vp]),
    "tpss_local_inverse_error": (C.c_int, [_vp, _vp, C.c_int64, C.c_int64, _dp]),
    "tpss_last_error": (C.c_char_p, []),
    "tpss_version": (C.c_char_p, []),
}


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libtpss_gpu.so (building it with nvcc when it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise ImportError(f"{path} is missing; build it with tpss_gb300.build.build()")
            _build.build()
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return _lib


def check(code: int):
    if code == TPSS_OK:
        return
    msg = load().tpss_last_error()
    msg = msg.decode() if msg else ""
    if code == TPSS_ERR_NOT_IMPLEMENTED:
        raise TPSSNotImplemented(code, msg)
    if code == TPSS_ERR_INVALID_ARGUMENT:
        raise TPSSInvalidArgument(code, msg)
    if code == TPSS_ERR_NOT_CONVERGED:
        raise TPSSNotConverged(code, msg)
    raise TPSSError(code, msg)
