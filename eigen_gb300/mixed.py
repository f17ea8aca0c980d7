"""Mixed-precision solves with FP64 refinement (gbs_dgesv_mixed*, gbs_dposv_mixed*).

``solve_mixed(A, B, tier)`` (general A) and ``solve_spd_mixed(A, B, tier)``
(SPD A, lower triangle read) factor in a low precision on the tensor cores,
refine in FP64 (classic or GMRES-IR) to a normwise backward error <= tol and
fall back to the plain FP64 factorization when refinement stalls.  A and B are
numpy arrays (host buffers) or column-major CUDA torch tensors (device
buffers, ordered on torch's current stream).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

TIERS = {"fp64": 0, "tf32x3": 1, "tf32": 2, "bf16": 3, "fp16": 4}
TIER_NAMES = {v: k for k, v in TIERS.items()}
REFINE = {"auto": 0, "classic": 1, "gmres": 2}
REFINE_NAMES = {v: k for k, v in REFINE.items()}


class RefineOptions(C.Structure):
    _fields_ = [("tier", C.c_int), ("refine", C.c_int), ("tol", C.c_double), ("max_iter", C.c_int),
                ("gmres_restart", C.c_int), ("gmres_tol", C.c_double), ("shift_factor", C.c_double),
                ("residual", C.c_int), ("pivoting", C.c_int), ("lookahead", C.c_int)]


class RefineInfo(C.Structure):
    _fields_ = [("tier_used", C.c_int), ("solver", C.c_int), ("iterations", C.c_int), ("inner_iterations", C.c_int),
                ("fell_back", C.c_int), ("singular", C.c_int), ("backward_error", C.c_double),
                ("shift", C.c_double)]

    def as_dict(self):
        return {"tier_used": TIER_NAMES.get(self.tier_used, self.tier_used),
                "solver": REFINE_NAMES.get(self.solver, self.solver), "iterations": self.iterations,
                "inner_iterations": self.inner_iterations, "fell_back": bool(self.fell_back),
                "singular": bool(self.singular), "backward_error": self.backward_error, "shift": self.shift}


RESIDUAL = {"auto": 0, "fp64": 1, "ozaki": 2}
PIVOTING = {"auto": 0, "tournament": 1, "partial": 2}


def options(tier="tf32x3", tol=1e-13, max_iter=30, refine="auto", gmres_restart=40, gmres_tol=1e-10,
            shift_factor=4.0, lookahead=True, residual="auto", pivoting="auto") -> RefineOptions:
    o = RefineOptions()
    L.lib().gbs_refine_options_default(C.byref(o))
    o.tier = TIERS[tier] if isinstance(tier, str) else int(tier)
    o.refine = REFINE[refine] if isinstance(refine, str) else int(refine)
    o.tol, o.max_iter, o.gmres_restart, o.gmres_tol, o.shift_factor = tol, max_iter, gmres_restart, gmres_tol, \
        shift_factor
    o.lookahead = int(bool(lookahead))
    o.residual = RESIDUAL[residual] if isinstance(residual, str) else int(residual)
    o.pivoting = PIVOTING[pivoting] if isinstance(pivoting, str) else int(pivoting)
    return o


def _solve(kind, A, B, opt, allow_not_spd=False):
    lib = L.lib()
    info = RefineInfo()
    dev_fn = lib.gbs_dgesv_mixed_device if kind == "ge" else lib.gbs_dposv_mixed_device
    host_fn = lib.gbs_dgesv_mixed if kind == "ge" else lib.gbs_dposv_mixed
    if hasattr(A, "is_cuda") and A.is_cuda:
        import torch
        n = A.shape[0]
        vec = B.dim() == 1
        Bm = B.reshape(-1, 1) if vec else B
        nrhs = Bm.shape[1]
        X = torch.empty((nrhs, n), dtype=torch.float64, device=A.device).t()
        if A.stride(0) != 1 or Bm.stride(0) != 1:
            raise ValueError("device matrices must be column-major")
        rc = dev_fn(n, nrhs, C.c_void_p(A.data_ptr()), max(A.stride(1), n, 1), C.c_void_p(Bm.data_ptr()),
                    max(Bm.stride(1), n, 1), C.c_void_p(X.data_ptr()), max(n, 1), C.byref(opt), C.byref(info),
                    C.c_void_p(torch.cuda.current_stream().cuda_stream))
        out = X.reshape(-1) if vec else X
    else:
        a = np.asfortranarray(A, dtype=np.float64)
        b = np.asarray(B, dtype=np.float64)
        vec = b.ndim == 1
        bm = np.asfortranarray(b.reshape(-1, 1) if vec else b)
        n, nrhs = a.shape[0], bm.shape[1]
        x = np.empty((n, nrhs), dtype=np.float64, order="F")
        rc = host_fn(n, nrhs, a.ctypes.data_as(C.c_void_p), max(n, 1), bm.ctypes.data_as(C.c_void_p), max(n, 1),
                     x.ctypes.data_as(C.c_void_p), max(n, 1), C.byref(opt), C.byref(info))
        out = x.reshape(-1) if vec else x
    if not (allow_not_spd and rc == L.GBS_NUMERICAL_ISSUE):
        L.check(rc, f"gbs_d{kind}sv_mixed")
    return out, info.as_dict()


def solve_mixed(A, B, tier="tf32x3", tol=1e-13, max_iter=30, refine="auto", **kw):
    """General A: returns (X, info dict)."""
    return _solve("ge", A, B, options(tier, tol, max_iter, refine, **kw))


def solve_spd_mixed(A, B, tier="tf32x3", tol=1e-13, max_iter=30, refine="auto", allow_not_spd=False, **kw):
    """SPD A (lower triangle read): returns (X, info dict)."""
    return _solve("po", A, B, options(tier, tol, max_iter, refine, **kw), allow_not_spd)
