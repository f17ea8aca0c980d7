"""Parity of the plain GPU path (FP64 / FP32) with the reference.

Every call goes through the C ABI (libgb300solve.so).  Checked against
  * the golden fixtures (the reference's own outputs, tests/golden), and
  * the CPU oracle (oracle/, pinned to those fixtures by test_oracle_golden.py).

Parity criteria (pivots are integer work, so bit-exact):
  * transpositions / permutation identical to the reference's, including
    exact and 1e-10 pivot ties decided after hundreds of blocked updates;
  * LLT factor, LLT solution and LU factors within 1e-12 relative Frobenius
    of the reference at every size (FP32: 2e-5), unscaled.  Above 129 the
    whole factor is checked three ways: against a sketch F R of the
    reference's whole factor (R a seeded Gaussian n x 4 or n x 8), against
    2048 sampled entries and the diagonal, and against the C restatement's
    whole factor computed here;
  * the whole-factor difference also stays within 3x the reference's own
    noise floor (its distance to the C restatement: same blocking, another
    rounding order), so the different blocking adds nothing beyond rounding;
  * LU solutions: backward error at the FP64 floor (<= 1e-14) and a forward
    difference within 10x the noise floor of the reference's solution (the
    forward difference is bounded by the conditioning, not by 1e-12);
  * rcond equal to the reference's to 1e-6 relative (same algorithm, same
    decisions), and within 10x of the exact value;
  * info() / first failing column / first zero pivot identical.
The achieved errors are printed in pytest's terminal summary.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from eigen_gb300 import LLT, PartialPivLU, getrf, getrs, llt_blocked, partial_lu_blocked, potrf, potrs
from eigen_gb300 import _lib
from tests.conftest import Golden, case_id, record_parity
from tests.golden.make_golden import sketch_matrix

pytestmark = pytest.mark.gpu
G = Golden()


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def ftol(case):
    return 2e-5 if case.get("dtype") == "f32" else 1e-12


def check(case, what, value, bound):
    record_parity(case_id(case), what, value, bound)
    assert value <= bound, f"{what}: {value:.3e} > {bound:.1e}"


def check_factor(case, f, oracle_f, full_key, idx_key, val_key, diag_key, sketch_key):
    """f against the reference's factor (whole, or sampled + diagonal + sketch)
    and against the C restatement's whole factor."""
    tol = ftol(case)
    f64 = case.get("dtype") != "f32"
    full = G.arr(case, full_key)
    if full is not None:
        check(case, "factor vs reference (whole)", rel(f, full), tol)
    else:
        idx = G.arr(case, idx_key)
        check(case, "factor vs reference (2048 entries)", rel(f.reshape(-1, order="F")[idx], G.arr(case, val_key)),
              tol)
        if G.arr(case, diag_key) is not None:
            check(case, "factor diagonal vs reference", rel(np.diag(f), G.arr(case, diag_key)), tol)
        sk = G.arr(case, sketch_key)
        d = rel(f.astype(np.float64) @ sketch_matrix(case["n"]), sk)
        check(case, "factor vs reference (whole, sketch)", d, tol)
        if f64:
            check(case, "factor sketch / reference noise floor", d, max(3 * case["factor_floor"], 1e-15))
    check(case, "factor vs C restatement (whole)", rel(f, oracle_f), tol)


LU = G.cases("lu")
LLT_CASES = G.cases("llt")


@pytest.mark.parametrize("case", LU, ids=[case_id(c) for c in LU])
def test_lu_matches_reference(case):
    a = G.input(case)
    n = case["n"]
    lu = PartialPivLU(a)
    tr = lu.transpositions()
    assert np.array_equal(tr, G.arr(case, "tr")), "pivot sequence differs from the reference"
    assert np.array_equal(lu.permutationP(), G.arr(case, "perm"))
    assert lu.nb_transpositions() == case["nb_transpositions"]
    assert lu.first_zero_pivot() == case["first_zero_pivot"]
    f = lu.matrixLU()
    f_o, tr_o, _, _ = O.lu(a)
    assert np.array_equal(tr_o, G.arr(case, "tr"))
    check_factor(case, f, f_o, "lu", "lu_idx", "lu_val", "lu_diag", "lu_sketch")
    assert lu.l1_norm() == pytest.approx(case["l1_norm"], rel=1e-6)
    if case["first_zero_pivot"] >= 0:
        return
    nrhs = G.arr(case, "x").shape[1]
    b = G.rhs(case, nrhs)
    x = lu.solve(b)
    xt = lu.solve_transposed(b)
    if a.dtype == np.float64:
        check(case, "LU solve backward error", O.backward_error(a, x, b), 1e-14)
        check(case, "LU transposed solve backward error", O.backward_error(np.asfortranarray(a.T), xt, b), 1e-14)
        # the forward difference is bounded by the conditioning: measured
        # against the reference's own spread (its distance to the C
        # restatement of the same algorithm)
        check(case, "LU solution forward diff (10x noise floor)", rel(x, G.arr(case, "x")),
              max(10 * case["x_floor"], 1e-13))
        check(case, "LU transposed solution forward diff", rel(xt, G.arr(case, "xt")),
              max(10 * case["xt_floor"], 1e-13))
    else:
        assert rel(x, G.arr(case, "x")) < 1e-3
    if n <= 2048:
        rc = lu.rcond()
        assert rc == pytest.approx(case["rcond"], rel=1e-6 if a.dtype == np.float64 else 1e-3)
        det = lu.determinant()
        assert det == pytest.approx(case["det"], rel=1e-9 if a.dtype == np.float64 else 1e-3, abs=1e-300)


@pytest.mark.parametrize("case", LLT_CASES, ids=[case_id(c) for c in LLT_CASES])
def test_llt_matches_reference(case):
    a = G.input(case)
    upper = case.get("upper", False)
    llt = LLT(a, upper=upper)
    ok = case["info"] == 0
    assert (llt.info() == _lib.GBS_SUCCESS) == ok
    assert (llt.failed_column() + 1 if llt.failed_column() >= 0 else 0) == case["potrf_info"]
    m = llt.matrixLLT()
    # the triangle not used keeps the caller's bytes
    other = np.tril(m, -1) if upper else np.triu(m, 1)
    assert np.array_equal(other, np.tril(a, -1) if upper else np.triu(a, 1))
    if not ok:
        # matrix state after an early failure equals the reference blocking's
        f_or, _ = O.llt(a, upper=upper)
        assert rel(m, f_or) < 1e-12
        with pytest.raises(_lib.GBSError):
            llt.solve(G.rhs(case, 1))
        return
    tri = np.triu(m) if upper else np.tril(m)
    f_o, info_o = O.llt(a, upper=upper)
    assert info_o == -1
    check_factor(case, tri, np.triu(f_o) if upper else np.tril(f_o), "fact", "fact_idx", "fact_val", "fact_diag",
                 "fact_sketch")
    nrhs = G.arr(case, "x").shape[1]
    b = G.rhs(case, nrhs)
    x = llt.solve(b)
    check(case, "LLT solution vs reference", rel(x, G.arr(case, "x")), ftol(case) if a.dtype == np.float64 else 2e-4)
    assert llt.rcond() == pytest.approx(case["rcond"], rel=1e-6 if a.dtype == np.float64 else 1e-3)
    assert llt.l1_norm() == pytest.approx(case["l1_norm"], rel=1e-6)


def test_lu_8192_headline_pivots_and_backward_error():
    """Headline size: n = 8192 iid N(0,1), 16 right-hand sides.  Pivots are the
    reference's, backward error is at the FP64 floor."""
    case = next(c for c in LU if c["n"] == 8192)
    a = G.input(case)
    lu = PartialPivLU(a)
    assert np.array_equal(lu.transpositions(), G.arr(case, "tr"))
    b = O.gauss(4242, 8192, 16)
    x = lu.solve(b)
    be = max(O.backward_error(a, x[:, j:j + 1], b[:, j:j + 1]) for j in (0, 7, 15))
    assert be < 1e-15 * 8


# ------------------------------------------------------------------ plug-in level
@pytest.mark.parametrize("m,n", [(64, 64), (300, 129), (1000, 70), (17, 17), (5, 3)])
def test_partial_lu_blocked_tall_matches_oracle(m, n):
    a = O.gauss(1000 + m + n, m, n)
    f = np.array(a, order="F", copy=True)
    ret, tr, nbt = partial_lu_blocked(f)
    f_o, tr_o, nbt_o, ret_o = O.lu(a)
    assert ret == ret_o and nbt == nbt_o
    assert np.array_equal(tr, tr_o)
    assert rel(f, f_o) < 1e-12


def test_llt_blocked_returns_failing_column():
    a = O.spd(3, 300)
    a[130, 130] = -1.0
    f = np.array(a, order="F", copy=True)
    assert llt_blocked(f) == 130
    f_o, r_o = O.llt(a)
    assert r_o == 130
    assert rel(f, f_o) < 1e-12
    g = np.asfortranarray(O.spd(4, 200))
    assert llt_blocked(g) == -1
    assert rel(np.tril(g), np.tril(O.llt(O.spd(4, 200))[0])) < 1e-12


# ------------------------------------------------------------------ LAPACK level
@pytest.mark.parametrize("case", G.cases("getrf"), ids=[case_id(c) for c in G.cases("getrf")])
def test_getrf_rectangular(case):
    a = np.array(G.input(case), order="F", copy=True)
    ipiv, info = getrf(a)
    assert np.array_equal(ipiv, G.arr(case, "ipiv"))
    assert info == case["getrf_info"]
    assert rel(a, G.arr(case, "lu")) < 1e-12


def test_getrf_info_on_singular():
    case = next(c for c in LU if c["gen"] == "zero_col" and c["n"] == 100)
    a = np.array(G.input(case), order="F", copy=True)
    ipiv, info = getrf(a)
    assert info == case["getrf_info"] == 58
    assert np.array_equal(ipiv, G.arr(case, "ipiv"))


def test_getrs_and_potrs():
    n = 257
    a = O.gauss(77, n, n)
    b = O.gauss(78, n, 5)
    f = np.array(a, order="F", copy=True)
    ipiv, info = getrf(f)
    assert info == 0
    for trans, mat in (("N", a), ("T", np.asfortranarray(a.T)), ("C", np.asfortranarray(a.T))):
        x = np.array(b, order="F", copy=True)
        assert getrs(trans, f, ipiv, x) == 0
        assert O.backward_error(mat, x, b) < 1e-14
    s = O.spd(79, n)
    for uplo in ("L", "U"):
        fs = np.array(s, order="F", copy=True)
        assert potrf(uplo, fs) == 0
        x = np.array(b, order="F", copy=True)
        assert potrs(uplo, fs, x) == 0
        assert O.backward_error(s, x, b) < 1e-14


def test_lapack_argument_errors_follow_the_reference():
    """info codes of lapack/lu.cpp:17-20, :50-55 and lapack/cholesky.cpp:17-20, :45-50."""
    L = _lib.lib()
    a = np.asfortranarray(np.eye(4))
    ipiv = np.zeros(4, dtype=np.int32)
    info = C.c_int(0)
    ci = lambda v: C.byref(C.c_int(v))
    p = a.ctypes.data_as(C.c_void_p)
    ip = ipiv.ctypes.data_as(C.c_void_p)
    L.gbs_dgetrf(ci(-1), ci(4), p, ci(4), ip, C.byref(info)); assert info.value == -1
    L.gbs_dgetrf(ci(4), ci(-1), p, ci(4), ip, C.byref(info)); assert info.value == -2
    L.gbs_dgetrf(ci(4), ci(4), p, ci(3), ip, C.byref(info)); assert info.value == -4
    L.gbs_dgetrs(b"X", ci(4), ci(1), p, ci(4), ip, p, ci(4), C.byref(info)); assert info.value == -1
    L.gbs_dgetrs(b"N", ci(4), ci(-1), p, ci(4), ip, p, ci(4), C.byref(info)); assert info.value == -3
    L.gbs_dgetrs(b"N", ci(4), ci(1), p, ci(4), ip, p, ci(2), C.byref(info)); assert info.value == -8
    L.gbs_dpotrf(b"Q", ci(4), p, ci(4), C.byref(info)); assert info.value == -1
    L.gbs_dpotrf(b"L", ci(4), p, ci(2), C.byref(info)); assert info.value == -4
    L.gbs_dpotrs(b"L", ci(4), ci(1), p, ci(4), p, ci(1), C.byref(info)); assert info.value == -7
    # sizes 0 are a no-op with info 0
    L.gbs_dgetrf(ci(0), ci(4), p, ci(1), ip, C.byref(info)); assert info.value == 0


# ------------------------------------------------------------------ reference test ports
@pytest.mark.parametrize("n", [1, 2, 3, 4, 17, 100, 320])
def test_lu_partial_piv_properties(n):
    """test/lu.cpp:179-218: reconstruction, solve, inverse, rcond within 10x,
    transposed solve."""
    m1 = O.uniform(5000 + n, n, n)
    plu = PartialPivLU(m1)
    assert rel(plu.reconstructedMatrix(), m1) < 1e-12
    m3 = O.uniform(6000 + n, n, n)
    m2 = plu.solve(m3)
    assert rel(m1 @ m2, m3) < 1e-10
    inv = plu.solve(np.asfortranarray(np.eye(n)))
    assert rel(inv @ m3, m2) < 1e-8
    truth = 1.0 / (O.l1_norm(m1) * O.l1_norm(inv))
    est = plu.rcond()
    assert truth / 10 < est < truth * 10
    m2t = plu.solve_transposed(m3)
    assert rel(m1.T @ m2t, m3) < 1e-10


@pytest.mark.parametrize("n", [1, 5, 31, 64, 200, 320])
def test_cholesky_properties(n):
    """test/cholesky.cpp:58-142: reconstruction, vector/matrix solves, rcond
    within 10x, upper mode, NumericalIssue on -A, L/U adjoint consistency."""
    a0 = O.uniform(7000 + n, n, n)
    symm = a0 @ a0.T
    for k in range(3):
        a1 = O.uniform(7100 + 10 * n + k, n, n)
        symm += a1 @ a1.T
    symm = np.asfortranarray(symm)
    vec_b = O.uniform(7200 + n, n, 1)[:, 0]
    mat_b = O.uniform(7300 + n, n, n)
    for upper in (False, True):
        stored = np.triu(symm) if upper else np.tril(symm)
        chol = LLT(np.asfortranarray(stored), upper=upper)
        assert chol.info() == _lib.GBS_SUCCESS
        assert rel(chol.reconstructedMatrix(), symm) < 1e-12
        x = chol.solve(vec_b)
        assert rel(symm @ x, vec_b) < 1e-9
        X = chol.solve(mat_b)
        assert rel(symm @ X, mat_b) < 1e-9
        inv = chol.solve(np.asfortranarray(np.eye(n)))
        truth = 1.0 / (O.sym_l1_norm(stored, upper) * O.l1_norm(inv))
        assert truth / 10 < chol.rcond() < truth * 10
        assert np.array_equal(chol.matrixU(), chol.matrixL().T)
    neg = LLT(np.asfortranarray(-np.tril(symm)))
    assert neg.info() == _lib.GBS_NUMERICAL_ISSUE


@pytest.mark.parametrize("n", [2, 50, 160])
def test_inplace_semantics_device_buffers(n):
    """test/inplace_decomposition.cpp:17-110 analogue for the device path:
    compute() on a device buffer does not modify it, solve() is correct, and a
    later change of the buffer does not affect the decomposition."""
    torch = pytest.importorskip("torch")
    a = O.gauss(8000 + n, n, n)
    b = O.gauss(8100 + n, n, 1)
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()   # column-major view
    A0 = A.clone()
    lu = PartialPivLU(A)
    assert torch.equal(A, A0)
    B = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    x = lu.solve(B).cpu().numpy()
    assert O.backward_error(a, x, b) < 1e-14
    A.normal_()
    x2 = lu.solve(B).cpu().numpy()
    assert np.array_equal(x, x2)
    s = O.spd(8200 + n, n)
    S = torch.from_numpy(np.ascontiguousarray(s.T)).cuda().t()
    llt = LLT(S)
    xs = llt.solve(B).cpu().numpy()
    assert O.backward_error(s, xs, b) < 1e-14


def test_device_input_freshly_produced_on_a_torch_stream():
    """compute() on a tensor whose producing kernel may still be running must
    see the finished data (the object is bound to the producer's stream)."""
    torch = pytest.importorskip("torch")
    n = 3000
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        for seed in range(3):
            g = torch.Generator(device="cuda").manual_seed(seed)
            a = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g).t()
            lu = PartialPivLU(a)               # queued right behind randn on `side`
            assert lu.first_zero_pivot() == -1
            host = np.asfortranarray(a.cpu().numpy())
            assert np.array_equal(lu.transpositions(), O.lu(host)[1])


def test_nonfinite_input_returns_without_hang():
    """NaN / Inf entries must neither trap nor hang: the factorization finishes
    and NaN propagates as in the reference (a NaN pivot is not an exact zero)."""
    a = O.gauss(9, 64, 64)
    a[3, 5] = np.nan
    a[10, 0] = np.inf
    lu = PartialPivLU(a)
    tr_o = O.lu(a)[1]
    assert np.array_equal(lu.transpositions(), tr_o)
    s = O.spd(10, 64)
    s[20, 20] = np.nan
    llt = LLT(s)
    assert llt.failed_column() == O.llt(s)[1]


@pytest.mark.parametrize("n", [1, 7, 200, 1031])
def test_lu_inverse_matches_oracle_solve_of_identity(n):
    """PartialPivLU::inverse() is solve(I) (PartialPivLU.h:197-201)."""
    a = O.gauss(500 + n, n, n)
    lu = PartialPivLU(a)
    inv = lu.inverse()
    f, tr, _, _ = O.lu(a)
    ref = O.lu_solve(f, tr, np.eye(n))
    assert np.linalg.norm(inv - ref) <= 1e-12 * max(1.0, np.linalg.norm(ref))
    assert np.linalg.norm(a @ inv - np.eye(n)) <= 1e-9 * n
