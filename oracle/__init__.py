"""CPU oracle for the dense factor-and-solve path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only to check results or time the
CPU baseline: the product (``eigen_gb300`` / ``libgb300solve.so``) never calls
into it.

Two back ends with the same numpy-level API:

* ``port``  -- ``_build/liboracle.so``, the plain-C restatement of the
  reference algorithms (``dense_oracle_impl.h`` names the reference lines each
  routine follows).  Builds anywhere with gcc.
* ``ref``   -- ``_ref/libeigen_ref.so``, the reference (Eigen) itself plus its
  LAPACK shim, built from the reference tree where it is present.  Used to pin
  the port and to write the golden fixtures in ``tests/golden``.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

HERE = Path(__file__).resolve().parent

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="F_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_L = C.c_long

_port = None
_ref = None


def port() -> C.CDLL:
    global _port
    if _port is None:
        lib = C.CDLL(str(_build.build_oracle()))
        for sfx, p in (("d", _dp), ("s", _fp)):
            f = getattr(lib, f"oracle_llt_blocked_{sfx}"); f.restype = _L; f.argtypes = [_L, p, _L]
            f = getattr(lib, f"oracle_llt_blocked_upper_{sfx}"); f.restype = _L; f.argtypes = [_L, p, _L]
            f = getattr(lib, f"oracle_llt_unblocked_{sfx}"); f.restype = _L; f.argtypes = [_L, p, _L]
            f = getattr(lib, f"oracle_lu_blocked_{sfx}"); f.restype = _L
            f.argtypes = [_L, _L, p, _L, _ip, C.POINTER(C.c_int), _L]
            f = getattr(lib, f"oracle_llt_solve_{sfx}"); f.restype = None
            f.argtypes = [_L, p, _L, C.c_int, _L, p, _L]
            f = getattr(lib, f"oracle_lu_solve_{sfx}"); f.restype = None
            f.argtypes = [_L, p, _L, _ip, _L, p, _L]
            f = getattr(lib, f"oracle_lu_solve_transposed_{sfx}"); f.restype = None
            f.argtypes = [_L, p, _L, _ip, _L, p, _L]
            f = getattr(lib, f"oracle_rcond_{sfx}"); f.restype = C.c_double
            f.argtypes = [C.c_int, _L, p, _L, _ip, C.c_double]
            f = getattr(lib, f"oracle_l1_norm_{sfx}"); f.restype = C.c_double; f.argtypes = [_L, _L, p, _L]
            f = getattr(lib, f"oracle_sym_l1_norm_{sfx}"); f.restype = C.c_double
            f.argtypes = [_L, p, _L, C.c_int]
            f = getattr(lib, f"oracle_perm_from_transpositions_{sfx}"); f.restype = None
            f.argtypes = [_L, _ip, _ip]
            f = getattr(lib, f"oracle_ldlt_{sfx}"); f.restype = C.c_int
            f.argtypes = [_L, p, _L, _ip, C.POINTER(C.c_int)]
            f = getattr(lib, f"oracle_ldlt_solve_{sfx}"); f.restype = None
            f.argtypes = [_L, p, _L, _ip, _L, p, _L]
            f = getattr(lib, f"oracle_llt_rank_update_{sfx}"); f.restype = _L
            f.argtypes = [_L, p, _L, p, C.c_double]
            vp = C.c_void_p
            f = getattr(lib, f"oracle_batched_llt_solve_{sfx}"); f.restype = None
            f.argtypes = [_L, _ip, _lp, vp, _lp, vp, _ip]
            f = getattr(lib, f"oracle_batched_lu_solve_{sfx}"); f.restype = None
            f.argtypes = [_L, _ip, _lp, vp, _lp, vp, _ip, _ip]
        lib.oracle_fill_gauss.argtypes = [C.c_uint64, _L, _L, _dp, _L]
        lib.oracle_fill_uniform.argtypes = [C.c_uint64, _L, _L, _dp, _L]
        lib.oracle_make_spd.argtypes = [C.c_uint64, _L, C.c_double, C.c_double, _dp, _L]
        lib.oracle_backward_error.restype = C.c_double
        lib.oracle_backward_error.argtypes = [_L, _dp, _L, _L, _dp, _L, _dp, _L]
        lib.oracle_num_threads.restype = C.c_int
        _port = lib
    return _port


def ref_available() -> bool:
    return (HERE / "_ref" / "libeigen_ref.so").exists() or _build.reference_available()


def ref() -> C.CDLL:
    """The reference itself (Eigen), where it could be built."""
    global _ref
    if _ref is None:
        path = HERE / "_ref" / "libeigen_ref.so"
        if _build.reference_available():
            path = _build.build_reference()
        if not path.exists():
            raise FileNotFoundError("reference build oracle/_ref/libeigen_ref.so not present")
        lib = C.CDLL(str(path))
        for sfx, p in (("d", _dp), ("s", _fp)):
            f = getattr(lib, f"ref_llt_{sfx}"); f.restype = C.c_int
            f.argtypes = [_L, p, _L, C.c_int, _L, p, _L, p, p, C.POINTER(C.c_double)]
            f = getattr(lib, f"ref_lu_{sfx}"); f.restype = C.c_int
            f.argtypes = [_L, p, _L, _L, p, _L, p, _ip, p, p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
            f = getattr(lib, f"ref_lu_blocked_{sfx}"); f.restype = _L
            f.argtypes = [_L, _L, p, _L, _ip, C.POINTER(C.c_int)]
            f = getattr(lib, f"ref_ldlt_{sfx}"); f.restype = C.c_int
            f.argtypes = [_L, p, _L, C.c_int, _L, p, _L, p, _ip, p, C.POINTER(C.c_double), _ip]
            f = getattr(lib, f"ref_llt_rank_update_{sfx}"); f.restype = C.c_int
            f.argtypes = [_L, p, _L, C.c_int, p, C.c_double, p]
            sp = C.POINTER(C.c_double if sfx == "d" else C.c_float)
            ip_ = C.POINTER(C.c_int)
            f = getattr(lib, f"{sfx}gemm_"); f.restype = C.c_int
            f.argtypes = [C.c_char_p, C.c_char_p, ip_, ip_, ip_, sp, p, ip_, p, ip_, sp, p, ip_]
            f = getattr(lib, f"{sfx}trsm_"); f.restype = C.c_int
            f.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, ip_, ip_, sp, p, ip_, p, ip_]
            f = getattr(lib, f"{sfx}syrk_"); f.restype = C.c_int
            f.argtypes = [C.c_char_p, C.c_char_p, ip_, ip_, sp, p, ip_, sp, p, ip_]
        lib.ref_llt_blocked_d.restype = _L
        lib.ref_llt_blocked_d.argtypes = [_L, _dp, _L]
        ip = C.POINTER(C.c_int)
        for sfx, p in (("d", _dp), ("s", _fp)):
            f = getattr(lib, f"{sfx}getrf_"); f.restype = C.c_int; f.argtypes = [ip, ip, p, ip, _ip, ip]
            f = getattr(lib, f"{sfx}potrf_"); f.restype = C.c_int; f.argtypes = [C.c_char_p, ip, p, ip, ip]
            f = getattr(lib, f"{sfx}getrs_"); f.restype = C.c_int
            f.argtypes = [C.c_char_p, ip, ip, p, ip, _ip, p, ip, ip]
            f = getattr(lib, f"{sfx}potrs_"); f.restype = C.c_int
            f.argtypes = [C.c_char_p, ip, ip, p, ip, p, ip, ip]
        lib.ref_set_threads.argtypes = [C.c_int]
        _ref = lib
    return _ref


# ----------------------------------------------------------------- generators
def gauss(seed: int, m: int, n: int) -> np.ndarray:
    """Seeded, byte-stable m x n matrix (Irwin-Hall(12) approximation of
    N(0,1)); identical bytes on every host (integer arithmetic only)."""
    a = np.empty((m, n), dtype=np.float64, order="F")
    port().oracle_fill_gauss(seed, m, n, a, max(m, 1))
    return a


def uniform(seed: int, m: int, n: int) -> np.ndarray:
    a = np.empty((m, n), dtype=np.float64, order="F")
    port().oracle_fill_uniform(seed, m, n, a, max(m, 1))
    return a


def spd(seed: int, n: int, scale: float | None = None, shift: float = 1.0) -> np.ndarray:
    """A = G G^T / scale + shift I (scale defaults to n), exactly symmetric."""
    a = np.empty((n, n), dtype=np.float64, order="F")
    port().oracle_make_spd(seed, n, float(n if scale is None else scale), float(shift), a, max(n, 1))
    return a


# ----------------------------------------------------------------- port API
def _sfx(a: np.ndarray) -> str:
    return "d" if a.dtype == np.float64 else "s"


def llt(a: np.ndarray, upper: bool = False, blocked: bool = True):
    """Returns (factor, info) -- info is -1 on success or the failing column."""
    f = np.array(a, order="F", copy=True)
    n = f.shape[0]
    lib = port()
    if upper:
        ret = getattr(lib, f"oracle_llt_blocked_upper_{_sfx(f)}")(n, f, max(n, 1))
    elif blocked:
        ret = getattr(lib, f"oracle_llt_blocked_{_sfx(f)}")(n, f, max(n, 1))
    else:
        ret = getattr(lib, f"oracle_llt_unblocked_{_sfx(f)}")(n, f, max(n, 1))
    return f, int(ret)


def lu(a: np.ndarray, max_block: int = 256):
    """Returns (lu, transpositions(0-based), nb_transpositions, first_zero_pivot)."""
    f = np.array(a, order="F", copy=True)
    m, n = f.shape
    tr = np.zeros(max(min(m, n), 1), dtype=np.int32)
    nbt = C.c_int(0)
    ret = getattr(port(), f"oracle_lu_blocked_{_sfx(f)}")(m, n, f, max(m, 1), tr, C.byref(nbt), max_block)
    return f, tr[: min(m, n)], int(nbt.value), int(ret)


def llt_solve(fact: np.ndarray, b: np.ndarray, upper: bool = False) -> np.ndarray:
    x = np.array(b, order="F", copy=True, dtype=fact.dtype)
    if x.ndim == 1:
        x = x.reshape(-1, 1, order="F")
    n = fact.shape[0]
    getattr(port(), f"oracle_llt_solve_{_sfx(fact)}")(n, fact, max(n, 1), int(upper), x.shape[1], x, max(n, 1))
    return x.reshape(b.shape, order="F") if b.ndim == 1 else x


def lu_solve(fact: np.ndarray, tr: np.ndarray, b: np.ndarray, transpose: bool = False) -> np.ndarray:
    x = np.array(b, order="F", copy=True, dtype=fact.dtype)
    if x.ndim == 1:
        x = x.reshape(-1, 1, order="F")
    n = fact.shape[0]
    trc = np.ascontiguousarray(tr, dtype=np.int32)
    name = "oracle_lu_solve_transposed_" if transpose else "oracle_lu_solve_"
    getattr(port(), name + _sfx(fact))(n, fact, max(n, 1), trc, x.shape[1], x, max(n, 1))
    return x.reshape(b.shape, order="F") if b.ndim == 1 else x


def perm_from_transpositions(tr: np.ndarray) -> np.ndarray:
    n = len(tr)
    p = np.zeros(max(n, 1), dtype=np.int32)
    port().oracle_perm_from_transpositions_d(n, np.ascontiguousarray(tr, dtype=np.int32), p)
    return p[:n]


def l1_norm(a: np.ndarray) -> float:
    m, n = a.shape
    return getattr(port(), f"oracle_l1_norm_{_sfx(a)}")(m, n, np.asfortranarray(a), max(m, 1))


def sym_l1_norm(a: np.ndarray, upper: bool = False) -> float:
    n = a.shape[0]
    return getattr(port(), f"oracle_sym_l1_norm_{_sfx(a)}")(n, np.asfortranarray(a), max(n, 1), int(upper))


def lu_rcond(fact: np.ndarray, tr: np.ndarray, a_norm: float) -> float:
    n = fact.shape[0]
    return getattr(port(), f"oracle_rcond_{_sfx(fact)}")(0, n, fact, max(n, 1),
                                                          np.ascontiguousarray(tr, dtype=np.int32), a_norm)


def llt_rcond(fact: np.ndarray, a_norm: float, upper: bool = False) -> float:
    n = fact.shape[0]
    dummy = np.zeros(1, dtype=np.int32)
    return getattr(port(), f"oracle_rcond_{_sfx(fact)}")(2 if upper else 1, n, fact, max(n, 1), dummy, a_norm)


def llt_rank_update(fact: np.ndarray, v: np.ndarray, sigma: float, upper: bool = False):
    """LLT::rankUpdate on a factor (matrixLLT layout): (updated factor, failing
    column or -1).  Upper works on the transpose, as the reference does
    (LLT.h:386-390)."""
    f = np.array(fact, order="F", copy=True)
    n = f.shape[0]
    w = np.asfortranarray(f.T) if upper else f
    vv = np.asfortranarray(np.asarray(v, dtype=f.dtype).reshape(n, 1))
    ret = getattr(port(), f"oracle_llt_rank_update_{_sfx(f)}")(n, w, max(n, 1), vv, float(sigma))
    if upper:
        f = np.asfortranarray(w.T)
    return f, int(ret)


SIGN_NAMES = ("PositiveSemiDef", "NegativeSemiDef", "ZeroSign", "Indefinite")   # LDLT.h:22


def ldlt(a: np.ndarray, upper: bool = False):
    """LDLT of the lower (upper) triangle: (matrixLDLT, transpositions, ok, sign).
    Upper runs the lower algorithm on the transpose, as the reference does
    (LDLT.h:453-461); the other triangle keeps the input."""
    f = np.array(a, order="F", copy=True)
    n = f.shape[0]
    w = np.asfortranarray(f.T) if upper else f
    tr = np.zeros(max(n, 1), dtype=np.int32)
    sign = C.c_int(2)
    ok = getattr(port(), f"oracle_ldlt_{_sfx(f)}")(n, w, max(n, 1), tr, C.byref(sign))
    if upper:
        f = np.asfortranarray(w.T)
    return f, tr[:n], bool(ok), int(sign.value)


def ldlt_solve(fact: np.ndarray, tr: np.ndarray, b: np.ndarray, upper: bool = False) -> np.ndarray:
    x = np.array(b, order="F", copy=True, dtype=fact.dtype)
    if x.ndim == 1:
        x = x.reshape(-1, 1, order="F")
    n = fact.shape[0]
    w = np.asfortranarray(fact.T) if upper else fact
    getattr(port(), f"oracle_ldlt_solve_{_sfx(fact)}")(n, w, max(n, 1), np.ascontiguousarray(tr, dtype=np.int32),
                                                       x.shape[1], x, max(n, 1))
    return x.reshape(b.shape, order="F") if b.ndim == 1 else x


def ldlt_rcond(fact: np.ndarray, tr: np.ndarray, a_norm: float, upper: bool = False) -> float:
    n = fact.shape[0]
    w = np.asfortranarray(fact.T) if upper else fact
    return getattr(port(), f"oracle_rcond_{_sfx(fact)}")(3, n, w, max(n, 1), np.ascontiguousarray(tr, dtype=np.int32),
                                                          a_norm)


def backward_error(a: np.ndarray, x: np.ndarray, b: np.ndarray) -> float:
    """max over columns of ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf),
    residual accumulated in extended precision."""
    a = np.asfortranarray(a, dtype=np.float64)
    x2 = np.asfortranarray(x.reshape(x.shape[0], -1), dtype=np.float64)
    b2 = np.asfortranarray(b.reshape(b.shape[0], -1), dtype=np.float64)
    n = a.shape[0]
    return port().oracle_backward_error(n, a, max(n, 1), x2.shape[1], x2, max(n, 1), b2, max(n, 1))


def num_threads() -> int:
    return int(port().oracle_num_threads())


# ----------------------------------------------------------------- reference API
def ref_llt(a: np.ndarray, b: np.ndarray | None = None, upper: bool = False):
    """Eigen LLT<Matrix, Lower|Upper>: (matrixLLT, info(0 ok / 1 NumericalIssue), x, rcond)."""
    lib = ref()
    a = np.asfortranarray(a)
    n = a.shape[0]
    fact = np.zeros((n, n), dtype=a.dtype, order="F")
    nrhs = 0 if b is None else (1 if b.ndim == 1 else b.shape[1])
    bb = np.zeros((n, max(nrhs, 1)), dtype=a.dtype, order="F") if b is None else \
        np.asfortranarray(b.reshape(n, -1), dtype=a.dtype)
    x = np.zeros((n, max(nrhs, 1)), dtype=a.dtype, order="F")
    rc = C.c_double(np.nan)
    info = getattr(lib, f"ref_llt_{_sfx(a)}")(n, a, max(n, 1), int(upper), nrhs, bb, max(n, 1), fact, x,
                                              C.byref(rc))
    return fact, int(info), x[:, :nrhs], rc.value


def ref_lu(a: np.ndarray, b: np.ndarray | None = None):
    """Eigen PartialPivLU<Matrix>: (matrixLU, permutationP().indices(), x, x_transposed, rcond, det)."""
    lib = ref()
    a = np.asfortranarray(a)
    n = a.shape[0]
    fact = np.zeros((n, n), dtype=a.dtype, order="F")
    perm = np.zeros(max(n, 1), dtype=np.int32)
    nrhs = 0 if b is None else (1 if b.ndim == 1 else b.shape[1])
    bb = np.zeros((n, max(nrhs, 1)), dtype=a.dtype, order="F") if b is None else \
        np.asfortranarray(b.reshape(n, -1), dtype=a.dtype)
    x = np.zeros((n, max(nrhs, 1)), dtype=a.dtype, order="F")
    xt = np.zeros((n, max(nrhs, 1)), dtype=a.dtype, order="F")
    rc = C.c_double(np.nan)
    det = C.c_double(np.nan)
    getattr(lib, f"ref_lu_{_sfx(a)}")(n, a, max(n, 1), nrhs, bb, max(n, 1), fact, perm, x, xt, C.byref(rc),
                                      C.byref(det))
    return fact, perm[:n], x[:, :nrhs], xt[:, :nrhs], rc.value, det.value


def ref_lu_blocked(a: np.ndarray):
    """The reference's partial_lu_impl::blocked_lu on a copy: (lu, transpositions, nb_tr, first_zero)."""
    f = np.array(a, order="F", copy=True)
    m, n = f.shape
    tr = np.zeros(max(min(m, n), 1), dtype=np.int32)
    nbt = C.c_int(0)
    ret = getattr(ref(), f"ref_lu_blocked_{_sfx(f)}")(m, n, f, max(m, 1), tr, C.byref(nbt))
    return f, tr[: min(m, n)], int(nbt.value), int(ret)


def ref_ldlt(a: np.ndarray, b: np.ndarray | None = None, upper: bool = False):
    """Eigen LDLT<Matrix, Lower|Upper>: (matrixLDLT, transpositionsP().indices(),
    info (0 Success / 1 NumericalIssue), isPositive, isNegative, x, rcond)."""
    lib = ref()
    a = np.asfortranarray(a)
    n = a.shape[0]
    fact = np.zeros((n, n), dtype=a.dtype, order="F")
    tr = np.zeros(max(n, 1), dtype=np.int32)
    nrhs = 0 if b is None else (1 if b.ndim == 1 else b.shape[1])
    bb = np.zeros((n, max(nrhs, 1)), dtype=a.dtype, order="F") if b is None else \
        np.asfortranarray(b.reshape(n, -1), dtype=a.dtype)
    x = np.zeros((n, max(nrhs, 1)), dtype=a.dtype, order="F")
    rc = C.c_double(np.nan)
    flags = np.zeros(2, dtype=np.int32)
    info = getattr(lib, f"ref_ldlt_{_sfx(a)}")(n, a, max(n, 1), int(upper), nrhs, bb, max(n, 1), fact, tr, x,
                                               C.byref(rc), flags)
    return fact, tr[:n], int(info), bool(flags[0]), bool(flags[1]), x[:, :nrhs], rc.value


def ref_llt_rank_update(a: np.ndarray, v: np.ndarray, sigma: float, upper: bool = False):
    """Eigen LLT<Matrix, Lower|Upper>(A).rankUpdate(v, sigma): (matrixLLT, info
    (0 Success / 1 NumericalIssue))."""
    a = np.asfortranarray(a)
    n = a.shape[0]
    fact = np.zeros((n, n), dtype=a.dtype, order="F")
    vv = np.asfortranarray(v.reshape(n, 1), dtype=a.dtype)
    info = getattr(ref(), f"ref_llt_rank_update_{_sfx(a)}")(n, a, max(n, 1), int(upper), vv, float(sigma), fact)
    assert info != 2, "the input is not positive definite"
    return fact, int(info)


def _ci(v):
    return C.byref(C.c_int(int(v)))


def _cs(x, dtype):
    return C.byref(C.c_double(x) if dtype == np.float64 else C.c_float(x))


def ref_gemm(opa: str, opb: str, alpha, a, b, beta, c):
    """The reference's BLAS ?gemm_ (blas/level3_impl.h:12-75) on copies: returns C."""
    c = np.array(c, order="F", copy=True)
    m, n = c.shape
    k = a.shape[1] if opa in "Nn" else a.shape[0]
    getattr(ref(), f"{_sfx(c)}gemm_")(opa.encode(), opb.encode(), _ci(m), _ci(n), _ci(k), _cs(alpha, c.dtype),
                                      np.asfortranarray(a), _ci(max(a.shape[0], 1)), np.asfortranarray(b),
                                      _ci(max(b.shape[0], 1)), _cs(beta, c.dtype), c, _ci(max(m, 1)))
    return c


def ref_trsm(side: str, uplo: str, opa: str, diag: str, alpha, a, b):
    """The reference's BLAS ?trsm_ (blas/level3_impl.h:77-176) on copies: returns X."""
    b = np.array(b, order="F", copy=True)
    m, n = b.shape
    getattr(ref(), f"{_sfx(b)}trsm_")(side.encode(), uplo.encode(), opa.encode(), diag.encode(), _ci(m), _ci(n),
                                      _cs(alpha, b.dtype), np.asfortranarray(a), _ci(max(a.shape[0], 1)), b,
                                      _ci(max(m, 1)))
    return b


def ref_syrk(uplo: str, op: str, alpha, a, beta, c):
    """The reference's BLAS ?syrk_ (blas/level3_impl.h:357-433) on copies: returns C."""
    c = np.array(c, order="F", copy=True)
    n = c.shape[0]
    k = a.shape[1] if op in "Nn" else a.shape[0]
    getattr(ref(), f"{_sfx(c)}syrk_")(uplo.encode(), op.encode(), _ci(n), _ci(k), _cs(alpha, c.dtype),
                                      np.asfortranarray(a), _ci(max(a.shape[0], 1)), _cs(beta, c.dtype), c,
                                      _ci(max(n, 1)))
    return c


def ref_llt_blocked(a: np.ndarray):
    f = np.array(a, order="F", copy=True, dtype=np.float64)
    n = f.shape[0]
    ret = ref().ref_llt_blocked_d(n, f, max(n, 1))
    return f, int(ret)
