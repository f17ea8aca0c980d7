"""Parity of the GPU BLAS level-3 entry points (gbs_?gemm, gbs_?trsm,
gbs_?syrk and their *_device variants) with the reference's BLAS shim
(blas/level3_impl.h), and of LLT::rankUpdate (gbs_llt_rank_update) with the
reference's LLT<Matrix>::rankUpdate (LLT.h:231-299, 461-472).

Checked against the golden fixtures (the reference's outputs on seeded
operands, every op / side / uplo / diag combination):
  * results within 1e-12 relative Frobenius (FP32 1e-5); the seeded operands
    are multiples of 2^-17, so most products are exact and agree bit for bit;
  * beta = 0 ignores a C that holds NaN; diag 'U' never reads a diagonal that
    holds NaN, nor the other triangle; syrk leaves the other triangle as given;
  * argument errors return the reference's xerbla position;
  * rank updates and downdates: the factor within 1e-12 (or 10x the
    reference's noise floor), info identical (a downdate that loses
    definiteness fails), the other triangle as given.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from eigen_gb300 import LLT, _lib
from eigen_gb300 import blas
from tests.conftest import Golden, record_parity
from tests.golden.make_golden import blas_inputs, sketch_matrix

pytestmark = pytest.mark.gpu
G = Golden()
BLAS = G.cases("blas")
RANK = G.cases("rank_update")


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def blas_id(c):
    keys = ("op", "side", "uplo", "opa", "opb", "diag")
    return "-".join(str(c[k]) for k in keys if k in c) + f"-{c.get('m', c['n'])}x{c['n']}" + \
        ("-f32" if c.get("dtype") == "f32" else "")


def run_blas(case, x, y, z):
    op = case["op"]
    if op == "gemm":
        return blas.gemm(case["opa"], case["opb"], case["alpha"], x, y, case["beta"], z)
    if op == "trsm":
        return blas.trsm(case["side"], case["uplo"], case["opa"], case["diag"], case["alpha"], x, y)
    return blas.syrk(case["uplo"], case["opa"], case["alpha"], x, case["beta"], y)


@pytest.mark.parametrize("case", BLAS, ids=[blas_id(c) for c in BLAS])
def test_blas_matches_reference(case):
    x, y, z = blas_inputs(case)
    out = run_blas(case, x, y, z)
    f64 = out.dtype == np.float64
    bound = max(1e-12 if f64 else 1e-5, 10 * case["floor"])
    ref = G.arr(case, "out")
    tag = f"{case['op']} vs reference"
    if case["op"] == "syrk":
        keep = np.tril if case["uplo"] in "Ll" else np.triu
        other = ~keep(np.ones(out.shape, dtype=bool))
        assert np.array_equal(out[other], y[other], equal_nan=True), "syrk wrote the other triangle"
    if ref is not None:
        if case["op"] == "syrk":
            d = rel(keep(out), keep(ref))
        else:
            d = rel(out, ref)
    else:
        s = sketch_matrix(out.shape[1])
        d = rel(out.astype(np.float64) @ s, G.arr(case, "out_sketch"))
    record_parity(blas_id(case), tag, d, bound)
    assert np.all(np.isfinite(out if case["op"] != "syrk" else keep(out))), "a NaN the routine must not read leaked"
    assert d <= bound, f"{tag}: {d:.3e} > {bound:.1e}"


@pytest.mark.parametrize("op", ["gemm", "trsm", "syrk"])
def test_blas_device_variants_equal_host(op):
    """The *_device entry points on torch tensors give the host entry points'
    results, for the widest case of each routine."""
    torch = pytest.importorskip("torch")
    case = max((c for c in BLAS if c["op"] == op and c.get("dtype") != "f32"), key=lambda c: c["n"] * c.get("m", 1))
    x, y, z = blas_inputs(case)
    host = run_blas(case, x, y, z)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    if op == "gemm":
        out = blas.gemm(case["opa"], case["opb"], case["alpha"], dev(x), dev(y), case["beta"], dev(z))
    elif op == "trsm":
        out = blas.trsm(case["side"], case["uplo"], case["opa"], case["diag"], case["alpha"], dev(x), dev(y))
    else:
        out = blas.syrk(case["uplo"], case["opa"], case["alpha"], dev(x), case["beta"], dev(y))
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), host, equal_nan=True)


def test_blas_argument_errors_follow_the_reference():
    """blas/level3_impl.h:46-54, 146-154, 386-394: the position of the first
    invalid argument."""
    L = _lib.lib()
    ci = lambda v: C.byref(C.c_int(v))
    one = C.byref(C.c_double(1.0))
    a = np.zeros((4, 4), order="F")
    p = a.ctypes.data_as(C.c_void_p)
    g = lambda oa, ob, m, n, k, lda, ldb, ldc: L.gbs_dgemm(oa, ob, ci(m), ci(n), ci(k), one, p, ci(lda), p, ci(ldb),
                                                           one, p, ci(ldc))
    assert g(b"X", b"N", 2, 2, 2, 2, 2, 2) == 1
    assert g(b"N", b"Q", 2, 2, 2, 2, 2, 2) == 2
    assert g(b"N", b"N", -1, 2, 2, 2, 2, 2) == 3
    assert g(b"N", b"N", 2, -1, 2, 2, 2, 2) == 4
    assert g(b"N", b"N", 2, 2, -1, 2, 2, 2) == 5
    assert g(b"N", b"N", 3, 2, 2, 2, 2, 3) == 8
    assert g(b"N", b"N", 2, 2, 3, 2, 2, 2) == 10
    assert g(b"N", b"N", 3, 2, 2, 3, 2, 2) == 13
    t = lambda sd, ul, oa, dg, m, n, lda, ldb: L.gbs_dtrsm(sd, ul, oa, dg, ci(m), ci(n), one, p, ci(lda), p, ci(ldb))
    assert t(b"X", b"L", b"N", b"N", 2, 2, 2, 2) == 1
    assert t(b"L", b"X", b"N", b"N", 2, 2, 2, 2) == 2
    assert t(b"L", b"L", b"X", b"N", 2, 2, 2, 2) == 3
    assert t(b"L", b"L", b"N", b"X", 2, 2, 2, 2) == 4
    assert t(b"L", b"L", b"N", b"N", -1, 2, 2, 2) == 5
    assert t(b"L", b"L", b"N", b"N", 2, -1, 2, 2) == 6
    assert t(b"R", b"L", b"N", b"N", 2, 3, 2, 2) == 9
    assert t(b"L", b"L", b"N", b"N", 3, 2, 3, 2) == 11
    s = lambda ul, op, n, k, lda, ldc: L.gbs_dsyrk(ul, op, ci(n), ci(k), one, p, ci(lda), one, p, ci(ldc))
    assert s(b"X", b"N", 2, 2, 2, 2) == 1
    assert s(b"L", b"X", 2, 2, 2, 2) == 2
    assert s(b"L", b"N", -1, 2, 2, 2) == 3
    assert s(b"L", b"N", 2, -1, 2, 2) == 4
    assert s(b"L", b"T", 2, 3, 2, 2) == 7
    assert s(b"L", b"N", 3, 2, 3, 2) == 10
    assert b"argument 10" in L.gbs_last_error()


@pytest.mark.parametrize("case", RANK, ids=[f"n{c['n']}-s{c['sigma']}-{'U' if c['upper'] else 'L'}" for c in RANK])
def test_llt_rank_update_matches_reference(case):
    a = O.spd(case["seed"], case["n"])
    v = O.gauss(case["seed"] + 1, case["n"], 1)[:, 0]
    upper = case["upper"]
    llt = LLT(a, upper=upper)
    llt.rankUpdate(v, case["sigma"])
    assert (0 if llt.info() == _lib.GBS_SUCCESS else 1) == case["info"]
    f = llt.matrixLLT()
    tri = np.triu if upper else np.tril
    assert np.array_equal(f - tri(f), a - tri(a)), "the other triangle must stay as given"
    bound = max(1e-12, 10 * case["floor"])
    full = G.arr(case, "fact")
    if full is not None:
        d = rel(tri(f), tri(full))
    else:
        d = rel(tri(f) @ sketch_matrix(case["n"]), G.arr(case, "fact_sketch"))
    record_parity(f"rank_update n={case['n']} sigma={case['sigma']}", "LLT rank update factor vs reference", d, bound)
    assert d <= bound


def test_llt_rank_update_then_solve():
    """After an update the object solves A + sigma v v^T (host and device v)."""
    torch = pytest.importorskip("torch")
    n = 700
    a = O.spd(91, n)
    v = O.gauss(92, n, 1)[:, 0]
    b = O.gauss(93, n, 2)
    llt = LLT(a)
    llt.rankUpdate(torch.from_numpy(v).cuda(), 0.3)
    x = llt.solve(b)
    assert O.backward_error(np.asfortranarray(a + 0.3 * np.outer(v, v)), x, b) < 1e-14
    llt.rankUpdate(v, -0.3)
    x = llt.solve(b)
    assert O.backward_error(a, x, b) < 1e-14
