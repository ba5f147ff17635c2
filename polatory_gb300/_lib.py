"""ctypes binding of libpolatory_gpu.so (the C ABI in include/polatory_gpu.h).

The shared library must be built in-tree (python polatory_gb300/build.py); importing this module
raises when it is missing. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libpolatory_gpu.so"

PGPU_OK = 0
PGPU_INVALID_ARGUMENT = 1
PGPU_RUNTIME_ERROR = 2
PGPU_CUDA_ERROR = 3
PGPU_OUT_OF_MEMORY = 4
PGPU_NOT_IMPLEMENTED = 5
PGPU_MAX_ITER = 6
PGPU_TIMEOUT = 7
PGPU_REJECTED = 8

INJECT_ALLOC = 1
INJECT_M2L_STALL = 2

PRECISION_PLAIN = 0
PRECISION_MIXED = 1
REQUEST_FIT = 0
REQUEST_EVALUATE = 1

KERNEL_VALUE = 0
KERNEL_GRADIENT = 1
KERNEL_GRADIENT_TRANSPOSE = 2
KERNEL_HESSIAN = 3

RBF_KINDS = ["bh2", "bh3", "cub", "exp", "gau", "gc3", "gc5", "gc7", "gc9", "sph", "sp3", "sp5",
             "sp7", "sp9", "th2", "th3"]
MAX_RBFS = 4


class PgpuRbf(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("params", C.c_double * 2),
                ("aniso", C.c_double * 9)]


class PgpuModel(C.Structure):
    _fields_ = [("n_rbfs", C.c_int32), ("poly_degree", C.c_int32), ("nugget", C.c_double),
                ("rbfs", PgpuRbf * MAX_RBFS)]


class PgpuFitStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("levels", C.c_int32), ("residual", C.c_double),
                ("grad_residual", C.c_double), ("setup_seconds", C.c_double),
                ("solve_seconds", C.c_double), ("n_domains", C.c_int64),
                ("precision_used", C.c_int32), ("fell_back", C.c_int32)]


class PgpuFitProblem(C.Structure):
    _fields_ = [("points", C.c_void_p), ("n", C.c_int64), ("values", C.c_void_p),
                ("tolerance", C.c_double), ("max_iter", C.c_int32), ("iterations", C.c_int32),
                ("eval_points", C.c_void_p), ("m", C.c_int64), ("eval_out", C.c_void_p),
                ("weights_out", C.c_void_p), ("residual", C.c_double), ("status", C.c_int32),
                ("reserved", C.c_int32)]


class PgpuRequest(C.Structure):
    _fields_ = [("kind", C.c_int32), ("slot", C.c_int32), ("model", C.c_void_p),
                ("points", C.c_void_p), ("n", C.c_int64), ("values", C.c_void_p),
                ("tolerance", C.c_double), ("max_iter", C.c_int32), ("precision", C.c_int32),
                ("out", C.c_void_p)]


class PgpuServerStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "completed", "failed", "rejected",
                                         "in_flight", "queued", "bytes_in_use", "peak_bytes",
                                         "budget_bytes")]


class PolatoryError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def _load():
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with python polatory_gb300/build.py")
    lib = C.CDLL(str(LIB_PATH))
    P = C.c_void_p
    D = C.POINTER(C.c_double)
    I64 = C.c_int64
    sig = {
        "pgpu_last_error": ([], C.c_char_p),
        "pgpu_version": ([], C.c_int),
        "pgpu_set_device": ([C.c_int], C.c_int),
        "pgpu_release_cached_memory": ([], C.c_int),
        "pgpu_profile_enable": ([C.c_int], C.c_int),
        "pgpu_profile_reset": ([], C.c_int),
        "pgpu_profile_report": ([C.c_char_p, I64], C.c_int),
        "pgpu_launch_count": ([C.POINTER(I64)], C.c_int),
        "pgpu_synchronize": ([], C.c_int),
        "pgpu_debug_inject": ([C.c_int, I64], C.c_int),
        "pgpu_operator_cache_stats": ([C.POINTER(I64), C.POINTER(I64), C.POINTER(I64)], C.c_int),
        "pgpu_operator_cache_limit": ([I64], C.c_int),
        "pgpu_stream": ([C.POINTER(C.c_void_p)], C.c_int),
        "pgpu_rbf_evaluate": ([C.POINTER(PgpuRbf), P, I64, P, P, P], C.c_int),
        "pgpu_rbf_cpd_order": ([C.POINTER(PgpuRbf), C.POINTER(C.c_int)], C.c_int),
        "pgpu_rbf_support_radius_isotropic": ([C.POINTER(PgpuRbf), D], C.c_int),
        "pgpu_model_validate": ([C.POINTER(PgpuModel)], C.c_int),
        "pgpu_model_poly_basis_size": ([C.POINTER(PgpuModel), C.POINTER(I64)], C.c_int),
        "pgpu_evaluator_create": ([C.POINTER(PgpuRbf), C.c_int, C.c_int, P, C.c_int,
                                   C.POINTER(P)], C.c_int),
        "pgpu_evaluator_destroy": ([P], C.c_int),
        "pgpu_evaluator_set_accuracy": ([P, C.c_double], C.c_int),
        "pgpu_evaluator_set_source_points": ([P, P, I64], C.c_int),
        "pgpu_evaluator_set_target_points": ([P, P, I64], C.c_int),
        "pgpu_evaluator_set_points": ([P, P, I64], C.c_int),
        "pgpu_evaluator_set_weights": ([P, P, I64], C.c_int),
        "pgpu_evaluator_configure": ([P, C.c_int, C.c_int, C.c_int], C.c_int),
        "pgpu_evaluator_evaluate": ([P, P, I64], C.c_int),
        "pgpu_direct_evaluate_noalloc": ([C.POINTER(PgpuRbf), P, I64, P, P, I64, P, P], C.c_int),
        "pgpu_krylov_fgmres_dense": ([I64, P, P, P, P, C.c_int, P, P], C.c_int),
        "pgpu_ras_domain_solve": ([C.POINTER(PgpuModel), P, I64, P, P, C.c_int, C.c_int,
                                   C.c_int, P, P], C.c_int),
        "pgpu_interpolant_create": ([C.POINTER(PgpuModel), C.POINTER(P)], C.c_int),
        "pgpu_interpolant_destroy": ([P], C.c_int),
        "pgpu_interpolant_set_precision": ([P, C.c_int], C.c_int),
        "pgpu_interpolant_fit": ([P, P, I64, P, I64, P, C.c_double, C.c_double, C.c_int,
                                  C.c_double, C.c_double, P], C.c_int),
        "pgpu_interpolant_evaluate": ([P, P, I64, P, I64, C.c_double, C.c_double, P], C.c_int),
        "pgpu_interpolant_evaluate_impl": ([P, P, I64, P, I64, P], C.c_int),
        "pgpu_interpolant_evaluate_lattice": ([P, P, P, P, I64, C.c_double, P], C.c_int),
        "pgpu_interpolant_set_evaluation_bbox": ([P, P, C.c_double, C.c_double], C.c_int),
        "pgpu_interpolant_is_fitted": ([P, C.POINTER(C.c_int)], C.c_int),
        "pgpu_interpolant_num_weights": ([P, C.POINTER(I64)], C.c_int),
        "pgpu_interpolant_weights": ([P, P, I64], C.c_int),
        "pgpu_interpolant_num_centers": ([P, C.POINTER(I64), C.POINTER(I64)], C.c_int),
        "pgpu_interpolant_centers": ([P, P, P], C.c_int),
        "pgpu_interpolant_bbox": ([P, P], C.c_int),
        "pgpu_interpolant_fit_stats": ([P, C.POINTER(PgpuFitStats)], C.c_int),
        "pgpu_interpolant_fit_incrementally": ([P, P, I64, P, I64, P, C.c_double, C.c_double,
                                                C.c_int, C.c_double, C.c_double], C.c_int),
        "pgpu_interpolant_fit_inequality": ([P, P, I64, P, P, P, C.c_double, C.c_int,
                                             C.c_double], C.c_int),
        "pgpu_interpolant_save": ([P, C.c_char_p], C.c_int),
        "pgpu_interpolant_load": ([C.c_char_p, C.POINTER(P)], C.c_int),
        "pgpu_fit_batch": ([C.POINTER(PgpuModel), C.c_int, C.POINTER(PgpuFitProblem), I64,
                            C.c_int], C.c_int),
        "pgpu_server_create": ([C.c_int, I64, C.POINTER(P)], C.c_int),
        "pgpu_server_destroy": ([P], C.c_int),
        "pgpu_server_submit": ([P, C.POINTER(PgpuRequest), C.POINTER(I64)], C.c_int),
        "pgpu_server_poll": ([P, I64, C.POINTER(C.c_int), C.POINTER(C.c_int),
                              C.POINTER(C.c_double)], C.c_int),
        "pgpu_server_wait": ([P, I64, C.POINTER(C.c_int), C.POINTER(C.c_double)], C.c_int),
        "pgpu_server_stats_get": ([P, C.POINTER(PgpuServerStats)], C.c_int),
        "pgpu_server_estimate_bytes": ([C.POINTER(PgpuRequest)], I64),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


lib = _load()


def check(rc: int) -> None:
    if rc != PGPU_OK:
        msg = lib.pgpu_last_error().decode()
        raise PolatoryError(rc, msg)


def ptr(a) -> C.c_void_p:
    """Address of a C-contiguous float64 numpy array or a torch CUDA tensor (device pointer)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
        raise TypeError("expected a C-contiguous float64 array")
    return C.c_void_p(a.ctypes.data)


def as_points(a) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if a.ndim == 1 and a.size == 0:
        a = a.reshape(0, 3)
    if a.ndim != 2 or a.shape[1] != 3:
        raise ValueError("points must have shape (n, 3)")
    return a
