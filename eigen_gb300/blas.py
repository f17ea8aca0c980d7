"""BLAS level 3 on the GPU with the semantics of the reference's BLAS shim
(blas/level3_impl.h): gemm, trsm, syrk through gbs_?gemm / gbs_?trsm / gbs_?syrk
(host arrays) and their *_device variants (torch CUDA tensors, in place)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _prefix(dtype) -> str:
    return "d" if np.dtype(dtype) == np.float64 else "s"


def _scalar(x, dtype):
    return C.byref(C.c_double(x) if np.dtype(dtype) == np.float64 else C.c_float(x))


def _i(v):
    return C.byref(C.c_int(int(v)))


def _check(rc: int, what: str):
    if rc > 0:
        raise ValueError(f"{what}: argument {rc} is invalid ({L.lib().gbs_last_error().decode()})")
    if rc < 0:
        raise L.GBSError(f"{what}: status {-rc - 100} ({L.lib().gbs_last_error().decode()})")


def _is_torch(x) -> bool:
    return hasattr(x, "is_cuda") and x.is_cuda


def _torch_np_dtype(t):
    return np.float64 if str(t.dtype) == "torch.float64" else np.float32


def _ld(x):
    """Leading dimension of a column-major host array or torch tensor."""
    if _is_torch(x):
        assert x.stride(0) == 1, "column-major tensor expected"
        return max(x.stride(1), x.shape[0], 1)
    return max(x.shape[0], 1)


def _host(x, dtype):
    return np.asfortranarray(np.asarray(x, dtype=dtype))


def gemm(transa: str, transb: str, alpha, a, b, beta, c, stream=None):
    """C = alpha op(A) op(B) + beta C.  Host arrays: returns the new C; torch
    CUDA tensors (column-major): C is updated in place and returned."""
    if _is_torch(c):
        dt = _torch_np_dtype(c)
        m, n = c.shape
        k = a.shape[1] if transa in "Nn" else a.shape[0]
        s = stream if stream is not None else __import__("torch").cuda.current_stream().cuda_stream
        _check(getattr(L.lib(), f"gbs_{_prefix(dt)}gemm_device")(
            transa.encode(), transb.encode(), _i(m), _i(n), _i(k), _scalar(alpha, dt), C.c_void_p(a.data_ptr()),
            _i(_ld(a)), C.c_void_p(b.data_ptr()), _i(_ld(b)), _scalar(beta, dt), C.c_void_p(c.data_ptr()), _i(_ld(c)),
            C.c_void_p(s)), "gemm")
        return c
    dt = np.asarray(c).dtype
    a, b, c = _host(a, dt), _host(b, dt), np.array(c, dtype=dt, order="F", copy=True)
    m, n = c.shape
    k = a.shape[1] if transa in "Nn" else a.shape[0]
    _check(getattr(L.lib(), f"gbs_{_prefix(dt)}gemm")(
        transa.encode(), transb.encode(), _i(m), _i(n), _i(k), _scalar(alpha, dt), a.ctypes.data_as(C.c_void_p),
        _i(_ld(a)), b.ctypes.data_as(C.c_void_p), _i(_ld(b)), _scalar(beta, dt), c.ctypes.data_as(C.c_void_p),
        _i(_ld(c))), "gemm")
    return c


def trsm(side: str, uplo: str, transa: str, diag: str, alpha, a, b, stream=None):
    """X with op(A) X = alpha B (side 'L') or X op(A) = alpha B (side 'R')."""
    if _is_torch(b):
        dt = _torch_np_dtype(b)
        m, n = b.shape
        s = stream if stream is not None else __import__("torch").cuda.current_stream().cuda_stream
        _check(getattr(L.lib(), f"gbs_{_prefix(dt)}trsm_device")(
            side.encode(), uplo.encode(), transa.encode(), diag.encode(), _i(m), _i(n), _scalar(alpha, dt),
            C.c_void_p(a.data_ptr()), _i(_ld(a)), C.c_void_p(b.data_ptr()), _i(_ld(b)), C.c_void_p(s)), "trsm")
        return b
    dt = np.asarray(b).dtype
    a, b = _host(a, dt), np.array(b, dtype=dt, order="F", copy=True)
    m, n = b.shape
    _check(getattr(L.lib(), f"gbs_{_prefix(dt)}trsm")(
        side.encode(), uplo.encode(), transa.encode(), diag.encode(), _i(m), _i(n), _scalar(alpha, dt),
        a.ctypes.data_as(C.c_void_p), _i(_ld(a)), b.ctypes.data_as(C.c_void_p), _i(_ld(b))), "trsm")
    return b


def syrk(uplo: str, trans: str, alpha, a, beta, c, stream=None):
    """C = alpha op(A) op(A)^T + beta C on the uplo triangle of C."""
    if _is_torch(c):
        dt = _torch_np_dtype(c)
        n = c.shape[0]
        k = a.shape[1] if trans in "Nn" else a.shape[0]
        s = stream if stream is not None else __import__("torch").cuda.current_stream().cuda_stream
        _check(getattr(L.lib(), f"gbs_{_prefix(dt)}syrk_device")(
            uplo.encode(), trans.encode(), _i(n), _i(k), _scalar(alpha, dt), C.c_void_p(a.data_ptr()), _i(_ld(a)),
            _scalar(beta, dt), C.c_void_p(c.data_ptr()), _i(_ld(c)), C.c_void_p(s)), "syrk")
        return c
    dt = np.asarray(c).dtype
    a, c = _host(a, dt), np.array(c, dtype=dt, order="F", copy=True)
    n = c.shape[0]
    k = a.shape[1] if trans in "Nn" else a.shape[0]
    _check(getattr(L.lib(), f"gbs_{_prefix(dt)}syrk")(
        uplo.encode(), trans.encode(), _i(n), _i(k), _scalar(alpha, dt), a.ctypes.data_as(C.c_void_p), _i(_ld(a)),
        _scalar(beta, dt), c.ctypes.data_as(C.c_void_p), _i(_ld(c))), "syrk")
    return c
