"""Mixed-precision solve with FP64 iterative refinement (gbs_dgesv_mixed*).

``solve_mixed(A, B, tier)`` factors A in a low precision on the tensor cores,
refines in FP64 to a normwise backward error <= tol and falls back to the
plain FP64 factorization (the reference's pivots) when refinement stalls.
A and B are numpy arrays (host buffers) or column-major CUDA torch tensors
(device buffers, ordered on torch's current stream).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

TIERS = {"fp64": 0, "tf32x3": 1, "tf32": 2, "bf16": 3, "fp16": 4}
TIER_NAMES = {v: k for k, v in TIERS.items()}


class RefineInfo(C.Structure):
    _fields_ = [("tier_used", C.c_int), ("iterations", C.c_int), ("fell_back", C.c_int), ("singular", C.c_int),
                ("backward_error", C.c_double)]

    def as_dict(self):
        return {"tier_used": TIER_NAMES.get(self.tier_used, self.tier_used), "iterations": self.iterations,
                "fell_back": bool(self.fell_back), "singular": bool(self.singular),
                "backward_error": self.backward_error}


def _tier(t) -> int:
    return TIERS[t] if isinstance(t, str) else int(t)


def solve_mixed(A, B, tier="tf32x3", tol=1e-13, max_iter=30):
    """Returns (X, info dict)."""
    lib = L.lib()
    info = RefineInfo()
    if hasattr(A, "is_cuda") and A.is_cuda:
        import torch
        n = A.shape[0]
        vec = B.dim() == 1
        Bm = B.reshape(-1, 1) if vec else B
        nrhs = Bm.shape[1]
        X = torch.empty((nrhs, n), dtype=torch.float64, device=A.device).t()
        lda = max(A.stride(1), 1) if A.stride(0) == 1 else None
        ldb = max(Bm.stride(1), n, 1) if Bm.stride(0) == 1 else None
        if lda is None or ldb is None:
            raise ValueError("device matrices must be column-major")
        L.check(lib.gbs_dgesv_mixed_device(n, nrhs, C.c_void_p(A.data_ptr()), lda, C.c_void_p(Bm.data_ptr()), ldb,
                                           C.c_void_p(X.data_ptr()), max(n, 1), _tier(tier), tol, max_iter,
                                           C.byref(info), C.c_void_p(torch.cuda.current_stream().cuda_stream)),
                "gbs_dgesv_mixed_device")
        return (X.reshape(-1) if vec else X), info.as_dict()
    a = np.asfortranarray(A, dtype=np.float64)
    b = np.asarray(B, dtype=np.float64)
    vec = b.ndim == 1
    bm = np.asfortranarray(b.reshape(-1, 1) if vec else b)
    n, nrhs = a.shape[0], bm.shape[1]
    x = np.empty((n, nrhs), dtype=np.float64, order="F")
    L.check(lib.gbs_dgesv_mixed(n, nrhs, a.ctypes.data_as(C.c_void_p), max(n, 1), bm.ctypes.data_as(C.c_void_p),
                                max(n, 1), x.ctypes.data_as(C.c_void_p), max(n, 1), _tier(tier), tol, max_iter,
                                C.byref(info)), "gbs_dgesv_mixed")
    return (x.reshape(-1) if vec else x), info.as_dict()
