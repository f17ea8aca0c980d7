"""ctypes binding of libgb300solve.so (the C ABI declared in include/gb300solve.h).

The library is built in-tree by ``eigen_gb300.build``; loading fails loudly if
it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

c_i64 = C.c_int64
c_int = C.c_int
c_vp = C.c_void_p
c_dp = C.POINTER(C.c_double)
c_ip = C.POINTER(C.c_int)

GBS_SUCCESS = 0
GBS_NUMERICAL_ISSUE = 1
GBS_INVALID_ARGUMENT = 2
GBS_NO_CONVERGENCE = 3
GBS_CUDA_ERROR = 4
GBS_NO_DEVICE = 5
GBS_TIMEOUT = 6
GBS_NOT_INITIALIZED = 7
GBS_OUT_OF_MEMORY = 8
STATUS_NAMES = {0: "SUCCESS", 1: "NUMERICAL_ISSUE", 2: "INVALID_ARGUMENT", 3: "NO_CONVERGENCE", 4: "CUDA_ERROR",
                5: "NO_DEVICE", 6: "TIMEOUT", 7: "NOT_INITIALIZED", 8: "OUT_OF_MEMORY"}
GBS_F64, GBS_F32 = 0, 1
GBS_LOWER, GBS_UPPER = 0, 1

# name -> (restype, argtypes); the complete exported surface of include/gb300solve.h
PROTOTYPES: dict[str, tuple] = {
    "gbs_last_error": (C.c_char_p, []),
    "gbs_version": (C.c_char_p, []),
    "gbs_device_count": (c_int, []),
    # failure detection
    "gbs_set_wait_limit": (C.c_double, [C.c_double]),
    "gbs_selftest_solve_timeout": (c_int, [c_int]),
    "gbs_selftest_barrier_timeout": (c_int, []),
    # plug-in level
    "gbs_llt_blocked_d": (c_i64, [c_i64, c_vp, c_i64, c_int]),
    "gbs_llt_blocked_s": (c_i64, [c_i64, c_vp, c_i64, c_int]),
    "gbs_partial_lu_blocked_d": (c_i64, [c_i64, c_i64, c_vp, c_i64, c_vp, c_ip]),
    "gbs_partial_lu_blocked_s": (c_i64, [c_i64, c_i64, c_vp, c_i64, c_vp, c_ip]),
    # LAPACK level
    "gbs_dgetrf": (c_int, [c_ip, c_ip, c_vp, c_ip, c_vp, c_ip]),
    "gbs_sgetrf": (c_int, [c_ip, c_ip, c_vp, c_ip, c_vp, c_ip]),
    "gbs_dgetrs": (c_int, [C.c_char_p, c_ip, c_ip, c_vp, c_ip, c_vp, c_vp, c_ip, c_ip]),
    "gbs_sgetrs": (c_int, [C.c_char_p, c_ip, c_ip, c_vp, c_ip, c_vp, c_vp, c_ip, c_ip]),
    "gbs_dpotrf": (c_int, [C.c_char_p, c_ip, c_vp, c_ip, c_ip]),
    "gbs_spotrf": (c_int, [C.c_char_p, c_ip, c_vp, c_ip, c_ip]),
    "gbs_dpotrs": (c_int, [C.c_char_p, c_ip, c_ip, c_vp, c_ip, c_vp, c_ip, c_ip]),
    "gbs_spotrs": (c_int, [C.c_char_p, c_ip, c_ip, c_vp, c_ip, c_vp, c_ip, c_ip]),
    "gbs_dgetrf_noalloc": (c_int, [c_int, c_int, c_vp, c_int, c_vp, c_vp, c_vp]),
    # LLT object
    "gbs_llt_create": (c_int, [C.POINTER(c_vp), c_int, c_int]),
    "gbs_llt_destroy": (c_int, [c_vp]),
    "gbs_llt_compute": (c_int, [c_vp, c_i64, c_vp, c_i64]),
    "gbs_llt_compute_device": (c_int, [c_vp, c_i64, c_vp, c_i64]),
    "gbs_llt_info": (c_int, [c_vp]),
    "gbs_llt_failed_column": (c_i64, [c_vp]),
    "gbs_llt_solve": (c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_i64]),
    "gbs_llt_solve_device": (c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_i64]),
    "gbs_llt_rcond": (c_int, [c_vp, c_dp]),
    "gbs_llt_l1_norm": (c_int, [c_vp, c_dp]),
    "gbs_llt_matrix": (c_int, [c_vp, c_vp, c_i64]),
    "gbs_llt_device_matrix": (c_vp, [c_vp, C.POINTER(c_i64)]),
    "gbs_llt_synchronize": (c_int, [c_vp]),
    "gbs_llt_set_stream": (c_int, [c_vp, c_vp]),
    # LU object
    "gbs_lu_create": (c_int, [C.POINTER(c_vp), c_int]),
    "gbs_lu_destroy": (c_int, [c_vp]),
    "gbs_lu_compute": (c_int, [c_vp, c_i64, c_vp, c_i64]),
    "gbs_lu_compute_device": (c_int, [c_vp, c_i64, c_vp, c_i64]),
    "gbs_lu_first_zero_pivot": (c_i64, [c_vp]),
    "gbs_lu_nb_transpositions": (c_int, [c_vp]),
    "gbs_lu_solve": (c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_int]),
    "gbs_lu_solve_device": (c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_int]),
    "gbs_lu_rcond": (c_int, [c_vp, c_dp]),
    "gbs_lu_l1_norm": (c_int, [c_vp, c_dp]),
    "gbs_lu_determinant": (c_int, [c_vp, c_dp]),
    "gbs_lu_inverse": (c_int, [c_vp, c_vp, c_i64]),
    "gbs_lu_inverse_device": (c_int, [c_vp, c_vp, c_i64]),
    "gbs_lu_matrix": (c_int, [c_vp, c_vp, c_i64]),
    "gbs_lu_transpositions": (c_int, [c_vp, c_vp]),
    "gbs_lu_permutation": (c_int, [c_vp, c_vp]),
    "gbs_lu_device_matrix": (c_vp, [c_vp, C.POINTER(c_i64)]),
    "gbs_lu_synchronize": (c_int, [c_vp]),
    "gbs_lu_set_stream": (c_int, [c_vp, c_vp]),
    "gbs_llt_rank_update": (c_int, [c_vp, c_vp, C.c_double]),
    "gbs_llt_rank_update_device": (c_int, [c_vp, c_vp, C.c_double]),
    # BLAS level 3 (scalars and sizes by pointer, as in the reference's shim)
    **{f"gbs_{p}gemm{d}": (c_int, [C.c_char_p, C.c_char_p, c_ip, c_ip, c_ip, c_vp, c_vp, c_ip, c_vp, c_ip, c_vp, c_vp,
                                   c_ip] + ([c_vp] if d else []))
       for p in "ds" for d in ("", "_device")},
    **{f"gbs_{p}trsm{d}": (c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, c_ip, c_ip, c_vp, c_vp, c_ip, c_vp,
                                   c_ip] + ([c_vp] if d else []))
       for p in "ds" for d in ("", "_device")},
    **{f"gbs_{p}syrk{d}": (c_int, [C.c_char_p, C.c_char_p, c_ip, c_ip, c_vp, c_vp, c_ip, c_vp, c_vp, c_ip]
                           + ([c_vp] if d else []))
       for p in "ds" for d in ("", "_device")},
    # LDLT object
    "gbs_ldlt_create": (c_int, [C.POINTER(c_vp), c_int, c_int]),
    "gbs_ldlt_destroy": (c_int, [c_vp]),
    "gbs_ldlt_compute": (c_int, [c_vp, c_i64, c_vp, c_i64]),
    "gbs_ldlt_compute_device": (c_int, [c_vp, c_i64, c_vp, c_i64]),
    "gbs_ldlt_info": (c_int, [c_vp]),
    "gbs_ldlt_sign": (c_int, [c_vp]),
    "gbs_ldlt_is_positive": (c_int, [c_vp]),
    "gbs_ldlt_is_negative": (c_int, [c_vp]),
    "gbs_ldlt_solve": (c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_i64]),
    "gbs_ldlt_solve_device": (c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_i64]),
    "gbs_ldlt_rcond": (c_int, [c_vp, c_dp]),
    "gbs_ldlt_l1_norm": (c_int, [c_vp, c_dp]),
    "gbs_ldlt_matrix": (c_int, [c_vp, c_vp, c_i64]),
    "gbs_ldlt_vector_d": (c_int, [c_vp, c_vp]),
    "gbs_ldlt_transpositions": (c_int, [c_vp, c_vp]),
    "gbs_ldlt_device_matrix": (c_vp, [c_vp, C.POINTER(c_i64)]),
    "gbs_ldlt_synchronize": (c_int, [c_vp]),
    "gbs_ldlt_set_stream": (c_int, [c_vp, c_vp]),
    # tensor cores
    "gbs_tc_gemm_sub": (c_int, [c_int, c_int, c_int, c_int, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_int, c_vp]),
    # mixed precision
    "gbs_refine_options_default": (None, [c_vp]),
    "gbs_dgeresid_device": (c_int, [c_int, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_int, c_vp]),
    "gbs_dgesv_mixed_device": (c_int, [c_int, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_vp, c_vp]),
    "gbs_dgesv_mixed": (c_int, [c_int, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_vp]),
    "gbs_dposv_mixed_device": (c_int, [c_int, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_vp, c_vp]),
    "gbs_dposv_mixed": (c_int, [c_int, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_vp]),
    # batched
    "gbs_batched_create": (c_int, [C.POINTER(c_vp), c_int, c_i64, c_vp, c_vp, c_int]),
    "gbs_batched_destroy": (c_int, [c_vp]),
    "gbs_batched_matrix_elements": (c_i64, [c_vp]),
    "gbs_batched_rhs_elements": (c_i64, [c_vp]),
    "gbs_batched_offsets": (c_int, [c_vp, c_vp, c_vp]),
    "gbs_batched_solve": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "gbs_batched_solve_host": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "gbs_batched_autotune": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_int]),
    "gbs_batched_config": (c_int, [c_vp, c_ip, c_ip]),
    "gbs_batched_buckets": (c_int, [c_vp, c_int, c_ip, c_ip]),
    "gbs_batched_set_variant": (c_int, [c_vp, c_int, c_int, c_int]),
    # medium batches + router
    "gbs_mbatch_create": (c_int, [C.POINTER(c_vp), c_i64, c_vp]),
    "gbs_mbatch_destroy": (c_int, [c_vp]),
    "gbs_mbatch_matrix_elements": (c_i64, [c_vp]),
    "gbs_mbatch_vector_elements": (c_i64, [c_vp]),
    "gbs_mbatch_offsets": (c_int, [c_vp, c_vp, c_vp]),
    "gbs_mbatch_lu_rcond": (c_int, [c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "gbs_mbatch_ir": (c_int, [c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, C.c_double, c_int, c_int, c_vp,
                              c_vp]),
    "gbs_mbatch_gmres_ir": (c_int, [c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, C.c_double, c_int, c_int, c_int,
                                    c_vp, c_vp, c_vp]),
    "gbs_mbatch_features": (c_int, [c_vp, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "gbs_router_feature_count": (c_int, []),
    "gbs_mlp_create": (c_int, [C.POINTER(c_vp), c_int, c_int, C.c_uint64]),
    "gbs_mlp_destroy": (c_int, [c_vp]),
    "gbs_mlp_param_count": (c_int, [c_vp]),
    "gbs_mlp_get_params": (c_int, [c_vp, c_vp]),
    "gbs_mlp_set_params": (c_int, [c_vp, c_vp]),
    "gbs_mlp_gradients": (c_int, [c_vp, c_vp, c_vp, c_int, c_vp, c_dp]),
    "gbs_mlp_train_step": (c_int, [c_vp, c_vp, c_vp, c_int, C.c_float, c_dp]),
    "gbs_mlp_fit": (c_int, [c_vp, c_vp, c_vp, c_int, c_int, c_int, C.c_float, C.c_uint64, c_dp]),
    "gbs_mlp_predict": (c_int, [c_vp, c_vp, c_int, c_vp, c_vp]),
    "gbs_router_route": (c_int, [c_vp, c_int, C.c_float, C.c_float, c_vp, c_vp]),
    # tracing
    "gbs_kernel_launch_count": (C.c_uint64, []),
    "gbs_profile_enable": (c_int, [c_int]),
    "gbs_profile_reset": (c_int, []),
    "gbs_profile_collect": (c_int, [c_int, c_dp, C.POINTER(c_i64), c_dp, c_dp]),
    "gbs_profile_timeline": (c_int, [c_ip, c_ip, c_dp, c_dp, c_int]),
    "gbs_streamed_input_plan": (c_int, [c_int, c_int, c_ip, c_ip, c_ip]),
}

PHASES = {"panel": 0, "laswp": 1, "trsm_lu": 2, "gemm": 3, "potrf_diag": 4, "trsm_llt": 5, "syrk": 6,
          "tri_solve": 7, "norm": 8, "mixed": 9, "tc_gemm": 10, "residual": 11, "batched": 12, "router": 13,
          "copy": 14}


class GBSError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = ""
        try:
            msg = lib().gbs_last_error().decode()
        except Exception:
            pass
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} ({msg})")


def lib() -> C.CDLL:
    """Load (building first if needed) libgb300solve.so."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not path.exists():
                path = _build.build()
            L = C.CDLL(str(path))
            for name, (res, args) in PROTOTYPES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != GBS_SUCCESS:
        raise GBSError(status, where)
