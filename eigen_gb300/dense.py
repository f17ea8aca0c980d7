"""Python mirror of Eigen's LLT / PartialPivLU over libgb300solve.

Same method names and meaning as the reference classes
(Eigen/src/Cholesky/LLT.h, Eigen/src/LU/PartialPivLU.h); storage is
column-major.  Inputs may be numpy arrays (host; the library copies them to the
GPU) or CUDA torch tensors viewed column-major (device; ``compute`` reads them
in place without modifying them).  Every call goes through the C ABI.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

ComputationInfo = {L.GBS_SUCCESS: "Success", L.GBS_NUMERICAL_ISSUE: "NumericalIssue"}


def _dtype_code(dt) -> int:
    if dt in (np.float64, "float64", "f64"):
        return L.GBS_F64
    if dt in (np.float32, "float32", "f32"):
        return L.GBS_F32
    raise TypeError(f"unsupported scalar type {dt}")


def _np_dtype(code: int):
    return np.float64 if code == L.GBS_F64 else np.float32


def _is_torch_cuda(x) -> bool:
    return hasattr(x, "is_cuda") and x.is_cuda


def _colmajor_host(a: np.ndarray, dtype) -> np.ndarray:
    return np.asfortranarray(a, dtype=dtype)


def _torch_colmajor_ld(t) -> int:
    """Leading dimension of a column-major 2-D CUDA tensor (stride(0) == 1)."""
    if t.dim() == 1:
        return max(t.shape[0], 1)
    if t.stride(0) != 1:
        raise ValueError("device matrices must be column-major (use t.t().contiguous().t())")
    return max(t.stride(1), t.shape[0], 1)


class _Decomposition:
    _prefix = ""

    def __init__(self, dtype):
        self._code = _dtype_code(np.dtype(dtype).type if not isinstance(dtype, int) else dtype)
        self._h = C.c_void_p()
        self._n = 0

    def _fn(self, name):
        return getattr(L.lib(), f"gbs_{self._prefix}_{name}")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._fn("destroy")(h)
            except Exception:
                pass
            self._h = C.c_void_p()

    def rows(self):
        return self._n

    def cols(self):
        return self._n

    def _bind_torch_stream(self):
        """Order device-buffer calls after the torch work that produced the data."""
        import torch
        self._fn("set_stream")(self._h, C.c_void_p(torch.cuda.current_stream().cuda_stream))

    def _compute(self, a):
        if _is_torch_cuda(a):
            self._bind_torch_stream()
            n = a.shape[0]
            assert a.shape[0] == a.shape[1], "square matrix expected"
            ld = _torch_colmajor_ld(a)
            L.check(self._fn("compute_device")(self._h, n, C.c_void_p(a.data_ptr()), ld), f"{self._prefix}.compute")
        else:
            a = _colmajor_host(a, _np_dtype(self._code))
            n = a.shape[0]
            assert a.shape[0] == a.shape[1], "square matrix expected"
            L.check(self._fn("compute")(self._h, n, a.ctypes.data_as(C.c_void_p), max(n, 1)),
                    f"{self._prefix}.compute")
        self._n = n
        return self

    def _solve(self, b, *extra):
        if _is_torch_cuda(b):
            import torch
            self._bind_torch_stream()
            vec = b.dim() == 1
            bb = b.reshape(-1, 1) if vec else b
            x = torch.empty((bb.shape[1], bb.shape[0]), dtype=b.dtype, device=b.device).t()
            L.check(self._fn("solve_device")(self._h, bb.shape[1], C.c_void_p(bb.data_ptr()), _torch_colmajor_ld(bb),
                                             C.c_void_p(x.data_ptr()), max(x.stride(1), 1), *extra),
                    f"{self._prefix}.solve")
            self._fn("synchronize")(self._h)
            return x.reshape(-1) if vec else x
        b = np.asarray(b)
        vec = b.ndim == 1
        bb = _colmajor_host(b.reshape(-1, 1) if vec else b, _np_dtype(self._code))
        x = np.empty_like(bb, order="F")
        L.check(self._fn("solve")(self._h, bb.shape[1], bb.ctypes.data_as(C.c_void_p), max(bb.shape[0], 1),
                                  x.ctypes.data_as(C.c_void_p), max(x.shape[0], 1), *extra), f"{self._prefix}.solve")
        return x.reshape(-1) if vec else x

    def rcond(self) -> float:
        r = C.c_double()
        L.check(self._fn("rcond")(self._h, C.byref(r)), f"{self._prefix}.rcond")
        return r.value

    def l1_norm(self) -> float:
        r = C.c_double()
        L.check(self._fn("l1_norm")(self._h, C.byref(r)), f"{self._prefix}.l1_norm")
        return r.value

    def _matrix(self):
        out = np.empty((self._n, self._n), dtype=_np_dtype(self._code), order="F")
        L.check(self._fn("matrix")(self._h, out.ctypes.data_as(C.c_void_p), max(self._n, 1)),
                f"{self._prefix}.matrix")
        return out


class LLT(_Decomposition):
    """Eigen::LLT<Matrix<S,Dynamic,Dynamic>, UpLo> on the GPU."""
    _prefix = "llt"

    def __init__(self, a=None, dtype=np.float64, upper: bool = False):
        if a is not None and not isinstance(dtype, int):
            dtype = a.dtype if not _is_torch_cuda(a) else {"torch.float64": np.float64,
                                                           "torch.float32": np.float32}[str(a.dtype)]
        super().__init__(dtype)
        self.upper = upper
        L.check(L.lib().gbs_llt_create(C.byref(self._h), self._code, L.GBS_UPPER if upper else L.GBS_LOWER),
                "llt.create")
        if a is not None:
            self.compute(a)

    def compute(self, a):
        return self._compute(a)

    def info(self) -> int:
        return L.lib().gbs_llt_info(self._h)

    def failed_column(self) -> int:
        return int(L.lib().gbs_llt_failed_column(self._h))

    def solve(self, b):
        return self._solve(b)

    def matrixLLT(self):
        return self._matrix()

    def rankUpdate(self, v, sigma: float = 1.0):
        """LLT::rankUpdate (LLT.h:461-472): the factor of A + sigma v v^T."""
        if _is_torch_cuda(v):
            self._bind_torch_stream()
            L.check(L.lib().gbs_llt_rank_update_device(self._h, C.c_void_p(v.contiguous().data_ptr()), float(sigma)),
                    "llt.rank_update")
        else:
            vv = np.ascontiguousarray(np.asarray(v).reshape(-1), dtype=_np_dtype(self._code))
            L.check(L.lib().gbs_llt_rank_update(self._h, vv.ctypes.data_as(C.c_void_p), float(sigma)),
                    "llt.rank_update")
        return self

    def matrixL(self):
        m = self._matrix()
        return np.tril(m) if not self.upper else np.triu(m).T.copy(order="F")

    def matrixU(self):
        return np.asfortranarray(self.matrixL().T)

    def reconstructedMatrix(self):
        l = self.matrixL()
        return l @ l.T


class LDLT(_Decomposition):
    """Eigen::LDLT<Matrix<S,Dynamic,Dynamic>, UpLo> on the GPU (Cholesky with
    diagonal pivoting, A = P^T L D L^T P, LDLT.h)."""
    _prefix = "ldlt"
    SIGNS = ("PositiveSemiDef", "NegativeSemiDef", "ZeroSign", "Indefinite")   # LDLT.h:22

    def __init__(self, a=None, dtype=np.float64, upper: bool = False):
        if a is not None and not isinstance(dtype, int):
            dtype = a.dtype if not _is_torch_cuda(a) else {"torch.float64": np.float64,
                                                           "torch.float32": np.float32}[str(a.dtype)]
        super().__init__(dtype)
        self.upper = upper
        L.check(L.lib().gbs_ldlt_create(C.byref(self._h), self._code, L.GBS_UPPER if upper else L.GBS_LOWER),
                "ldlt.create")
        if a is not None:
            self.compute(a)

    def compute(self, a):
        return self._compute(a)

    def info(self) -> int:
        return L.lib().gbs_ldlt_info(self._h)

    def sign(self) -> int:
        return int(L.lib().gbs_ldlt_sign(self._h))

    def isPositive(self) -> bool:
        return bool(L.lib().gbs_ldlt_is_positive(self._h))

    def isNegative(self) -> bool:
        return bool(L.lib().gbs_ldlt_is_negative(self._h))

    def solve(self, b):
        return self._solve(b)

    def matrixLDLT(self):
        return self._matrix()

    def vectorD(self):
        out = np.empty(self._n, dtype=_np_dtype(self._code))
        L.check(L.lib().gbs_ldlt_vector_d(self._h, out.ctypes.data_as(C.c_void_p)), "ldlt.vector_d")
        return out

    def transpositionsP(self) -> np.ndarray:
        out = np.zeros(max(self._n, 1), dtype=np.int32)
        L.check(L.lib().gbs_ldlt_transpositions(self._h, out.ctypes.data_as(C.c_void_p)), "ldlt.transpositions")
        return out[: self._n]

    def matrixL(self):
        m = self._matrix()
        l = np.tril(m, -1) if not self.upper else np.triu(m, 1).T
        return np.asfortranarray(l + np.eye(self._n, dtype=m.dtype))

    def reconstructedMatrix(self):
        """P^T L D L^T P (LDLT.h:594-618)."""
        l = self.matrixL()
        r = l @ np.diag(self.vectorD()) @ l.T
        tr = self.transpositionsP()
        p = np.arange(self._n)
        for k in range(self._n):
            p[[k, tr[k]]] = p[[tr[k], k]]
        out = np.empty_like(r)
        out[np.ix_(p, p)] = r
        return out


class PartialPivLU(_Decomposition):
    """Eigen::PartialPivLU<Matrix<S,Dynamic,Dynamic>> on the GPU."""
    _prefix = "lu"

    def __init__(self, a=None, dtype=np.float64):
        if a is not None and not isinstance(dtype, int):
            dtype = a.dtype if not _is_torch_cuda(a) else {"torch.float64": np.float64,
                                                           "torch.float32": np.float32}[str(a.dtype)]
        super().__init__(dtype)
        L.check(L.lib().gbs_lu_create(C.byref(self._h), self._code), "lu.create")
        if a is not None:
            self.compute(a)

    def compute(self, a):
        return self._compute(a)

    def solve(self, b):
        return self._solve(b, 0)

    def solve_transposed(self, b):
        """_solve_impl_transposed<false>: x with A^T x = b."""
        return self._solve(b, 1)

    def matrixLU(self):
        return self._matrix()

    def transpositions(self) -> np.ndarray:
        t = np.empty(max(self._n, 1), dtype=np.int32)
        L.check(L.lib().gbs_lu_transpositions(self._h, t.ctypes.data_as(C.c_void_p)), "lu.transpositions")
        return t[: self._n]

    def permutationP(self) -> np.ndarray:
        """permutationP().indices()"""
        p = np.empty(max(self._n, 1), dtype=np.int32)
        L.check(L.lib().gbs_lu_permutation(self._h, p.ctypes.data_as(C.c_void_p)), "lu.permutation")
        return p[: self._n]

    def determinant(self) -> float:
        d = C.c_double()
        L.check(L.lib().gbs_lu_determinant(self._h, C.byref(d)), "lu.determinant")
        return d.value

    def inverse(self):
        """PartialPivLU::inverse(): A^-1 = solve(I), on the host (numpy)."""
        out = np.empty((self._n, self._n), dtype=_np_dtype(self._code), order="F")
        L.check(L.lib().gbs_lu_inverse(self._h, out.ctypes.data_as(C.c_void_p), max(self._n, 1)), "lu.inverse")
        return out

    def first_zero_pivot(self) -> int:
        return int(L.lib().gbs_lu_first_zero_pivot(self._h))

    def nb_transpositions(self) -> int:
        return int(L.lib().gbs_lu_nb_transpositions(self._h))

    def reconstructedMatrix(self):
        lu = self._matrix()
        l = np.tril(lu, -1) + np.eye(self._n, dtype=lu.dtype)
        u = np.triu(lu)
        res = l @ u
        p = self.permutationP()
        out = np.empty_like(res)
        out[np.arange(self._n)] = res[p]   # P^{-1} (L U): row i of result = row p[i]
        return out


# ------------------------------------------------------------------ plug-in level
def llt_blocked(a: np.ndarray, upper: bool = False) -> int:
    """In place on a (column-major); returns -1 or the failing column
    (llt_inplace<>::blocked)."""
    assert a.flags.f_contiguous
    fn = L.lib().gbs_llt_blocked_d if a.dtype == np.float64 else L.lib().gbs_llt_blocked_s
    n = a.shape[0]
    r = fn(n, a.ctypes.data_as(C.c_void_p), max(n, 1), int(upper))
    if r < -1:
        raise L.GBSError(int(-r - 100), "llt_blocked")
    return int(r)


def partial_lu_blocked(a: np.ndarray):
    """In place on a; returns (first_zero_pivot, transpositions, nb_transpositions)
    (partial_lu_impl<>::blocked_lu)."""
    assert a.flags.f_contiguous
    m, n = a.shape
    tr = np.zeros(max(min(m, n), 1), dtype=np.int32)
    nbt = C.c_int(0)
    fn = L.lib().gbs_partial_lu_blocked_d if a.dtype == np.float64 else L.lib().gbs_partial_lu_blocked_s
    r = fn(m, n, a.ctypes.data_as(C.c_void_p), max(m, 1), tr.ctypes.data_as(C.c_void_p), C.byref(nbt))
    if r < -1:
        raise L.GBSError(int(-r - 100), "partial_lu_blocked")
    return int(r), tr[: min(m, n)], int(nbt.value)


# ------------------------------------------------------------------ LAPACK level
def _ci(v):
    return C.byref(C.c_int(int(v)))


def getrf(a: np.ndarray):
    """?getrf_ in place: returns (ipiv 1-based, info)."""
    assert a.flags.f_contiguous
    m, n = a.shape
    ipiv = np.zeros(max(min(m, n), 1), dtype=np.int32)
    info = C.c_int(0)
    fn = L.lib().gbs_dgetrf if a.dtype == np.float64 else L.lib().gbs_sgetrf
    L.check(fn(_ci(m), _ci(n), a.ctypes.data_as(C.c_void_p), _ci(max(m, 1)), ipiv.ctypes.data_as(C.c_void_p),
               C.byref(info)), "getrf")
    return ipiv[: min(m, n)], info.value


def getrs(trans: str, lu: np.ndarray, ipiv: np.ndarray, b: np.ndarray) -> int:
    n = lu.shape[0]
    nrhs = b.shape[1]
    info = C.c_int(0)
    fn = L.lib().gbs_dgetrs if lu.dtype == np.float64 else L.lib().gbs_sgetrs
    ip = np.ascontiguousarray(ipiv, dtype=np.int32)
    L.check(fn(trans.encode(), _ci(n), _ci(nrhs), lu.ctypes.data_as(C.c_void_p), _ci(max(n, 1)),
               ip.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p), _ci(max(n, 1)), C.byref(info)), "getrs")
    return info.value


def potrf(uplo: str, a: np.ndarray) -> int:
    n = a.shape[0]
    info = C.c_int(0)
    fn = L.lib().gbs_dpotrf if a.dtype == np.float64 else L.lib().gbs_spotrf
    L.check(fn(uplo.encode(), _ci(n), a.ctypes.data_as(C.c_void_p), _ci(max(n, 1)), C.byref(info)), "potrf")
    return info.value


def potrs(uplo: str, a: np.ndarray, b: np.ndarray) -> int:
    n = a.shape[0]
    info = C.c_int(0)
    fn = L.lib().gbs_dpotrs if a.dtype == np.float64 else L.lib().gbs_spotrs
    L.check(fn(uplo.encode(), _ci(n), _ci(b.shape[1]), a.ctypes.data_as(C.c_void_p), _ci(max(n, 1)),
               b.ctypes.data_as(C.c_void_p), _ci(max(n, 1)), C.byref(info)), "potrs")
    return info.value
