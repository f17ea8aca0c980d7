"""Pin the CPU oracle (the plain-C restatement in oracle/) to the reference's
own outputs stored in tests/golden (made by running Eigen itself).

These run on CPU only.  The GPU parity tests then compare the CUDA path with
both the fixtures and this pinned oracle.
"""
import numpy as np
import pytest

import oracle as O
from tests.conftest import Golden, case_id
from tests.golden.make_golden import sketch_matrix

G = Golden()
MAX_N_CPU = 2048   # the 8192 case is exercised by the GPU tests


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def tol(case):
    return 2e-5 if case.get("dtype") == "f32" else 1e-12


LU = [c for c in G.cases("lu") if c["n"] <= MAX_N_CPU]
LLT = [c for c in G.cases("llt") if c["n"] <= MAX_N_CPU]


@pytest.mark.parametrize("case", LU, ids=[case_id(c) for c in LU])
def test_oracle_lu_matches_reference(case):
    a = G.input(case)
    f, tr, nbt, fz = O.lu(a)
    assert np.array_equal(tr, G.arr(case, "tr")), "pivot sequence differs from the reference"
    assert np.array_equal(O.perm_from_transpositions(tr), G.arr(case, "perm"))
    assert np.array_equal(tr + 1, G.arr(case, "ipiv"))
    assert nbt == case["nb_transpositions"]
    assert fz == case["first_zero_pivot"]
    assert (fz + 1 if fz >= 0 else 0) == case["getrf_info"]
    full = G.arr(case, "lu")
    if full is not None:
        assert rel(f, full) <= tol(case)
    else:
        idx = G.arr(case, "lu_idx")
        assert rel(f.reshape(-1, order="F")[idx], G.arr(case, "lu_val")) <= tol(case)
        assert rel(np.diag(f), G.arr(case, "lu_diag")) <= tol(case)
        # whole factor: the sketch F R sees every entry; its distance equals
        # the recorded noise floor up to the projection's spread
        d = rel(f.astype(np.float64) @ sketch_matrix(case["n"]), G.arr(case, "lu_sketch"))
        assert d <= tol(case)
        assert d <= 3 * case["factor_floor"] + 1e-16
    if case["gen"] in ("tie_rows", "near_tie_rows"):
        assert case["tie_decisions"] >= case["pairs"] - 1, "the tie construction no longer creates ties"
    if case["first_zero_pivot"] < 0:
        nrhs = G.arr(case, "x").shape[1]
        b = G.rhs(case, nrhs)
        x = O.lu_solve(f, tr, b)
        xt = O.lu_solve(f, tr, b, transpose=True)
        # LU solutions carry the conditioning of A; compare by backward error
        # and, loosely, by forward difference to the reference's solution
        if a.dtype == np.float64:
            assert O.backward_error(a, x, b) < 1e-14
            assert O.backward_error(np.asfortranarray(a.T), xt, b) < 1e-14
        assert rel(x, G.arr(case, "x")) < (1e-3 if a.dtype == np.float32 else 1e-9)
        rc = O.lu_rcond(f, tr, O.l1_norm(a))
        assert abs(rc - case["rcond"]) <= 1e-6 * abs(case["rcond"]) + (1e-3 * case["rcond"] if a.dtype == np.float32 else 0)
        assert O.l1_norm(a) == pytest.approx(case["l1_norm"], rel=1e-6)


@pytest.mark.parametrize("case", G.cases("getrf"), ids=[case_id(c) for c in G.cases("getrf")])
def test_oracle_rectangular_getrf(case):
    a = G.input(case)
    f, tr, nbt, fz = O.lu(a)
    assert np.array_equal(tr + 1, G.arr(case, "ipiv"))
    assert rel(f, G.arr(case, "lu")) < 1e-12
    assert case["getrf_info"] == (fz + 1 if fz >= 0 else 0)


@pytest.mark.parametrize("case", LLT, ids=[case_id(c) for c in LLT])
def test_oracle_llt_matches_reference(case):
    a = G.input(case)
    upper = case.get("upper", False)
    f, info = O.llt(a, upper=upper)
    # LLT::info(): Success/NumericalIssue; ?potrf_: first failing column + 1
    assert (info >= 0) == (case["info"] != 0)
    assert (info + 1 if info >= 0 else 0) == case["potrf_info"]
    if case.get("gen") == "late_fail":
        assert info == case["col"]
    # the untouched triangle keeps the input bytes (LLT.h: "upper part not used")
    if upper:
        assert np.array_equal(np.tril(f, -1), np.tril(a, -1))
    else:
        assert np.array_equal(np.triu(f, 1), np.triu(a, 1))
    if info >= 0:
        return
    tri = np.triu(f) if upper else np.tril(f)
    full = G.arr(case, "fact")
    if full is not None:
        assert rel(tri, full) <= tol(case)
    else:
        idx = G.arr(case, "fact_idx")
        assert rel(tri.reshape(-1, order="F")[idx], G.arr(case, "fact_val")) <= tol(case)
        d = rel(tri.astype(np.float64) @ sketch_matrix(case["n"]), G.arr(case, "fact_sketch"))
        assert d <= tol(case)
        assert d <= 3 * case["factor_floor"] + 1e-16
    nrhs = G.arr(case, "x").shape[1]
    b = G.rhs(case, nrhs)
    x = O.llt_solve(f, b, upper=upper)
    assert rel(x, G.arr(case, "x")) <= (tol(case) if a.dtype == np.float64 else 2e-4)
    rc = O.llt_rcond(f, O.sym_l1_norm(a, upper), upper=upper)
    assert rc == pytest.approx(case["rcond"], rel=1e-9 if a.dtype == np.float64 else 1e-4)
    assert O.sym_l1_norm(a, upper) == pytest.approx(case["l1_norm"], rel=1e-12)


def test_generators_are_byte_stable():
    """The fixtures store generator specs, not inputs: pin a few bytes."""
    g = O.gauss(123, 4, 3)
    u = O.uniform(123, 4, 3)
    assert g.dtype == np.float64 and g.flags.f_contiguous
    # Irwin-Hall(12): values are multiples of 2^-17 in (-6, 6)
    assert np.all(np.abs(g) < 6) and np.all((g * 131072) == np.rint(g * 131072))
    assert np.all(np.abs(u) <= 1) and np.all((u * 2**31) == np.rint(u * 2**31))
    big = O.gauss(5, 300, 300)
    assert abs(big.mean()) < 0.02 and abs(big.std() - 1) < 0.02
    s = O.spd(9, 50)
    assert np.array_equal(s, s.T)
    assert np.linalg.eigvalsh(s).min() > 0.9


def test_rcond_within_10x_of_truth():
    """test/cholesky.cpp:94-116 and test/lu.cpp:200-203: the estimate is within a
    factor 10 of 1/(||A||_1 ||A^-1||_1)."""
    for n in [5, 40, 200]:
        a = O.gauss(31 + n, n, n)
        f, tr, _, _ = O.lu(a)
        inv = O.lu_solve(f, tr, np.asfortranarray(np.eye(n)))
        truth = 1.0 / (O.l1_norm(a) * O.l1_norm(inv))
        est = O.lu_rcond(f, tr, O.l1_norm(a))
        assert truth / 10 < est < truth * 10
        s = O.spd(77 + n, n)
        fl, info = O.llt(s)
        inv = O.llt_solve(fl, np.asfortranarray(np.eye(n)))
        truth = 1.0 / (O.sym_l1_norm(s) * O.l1_norm(inv))
        est = O.llt_rcond(fl, O.sym_l1_norm(s))
        assert truth / 10 < est < truth * 10


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_batched_oracle_equals_the_pinned_per_item_oracle(dtype):
    """The batched CPU baseline (the oracle leg of bench.py --config batched) factors and
    solves each item with the per-item oracle pinned above: identical bytes,
    including failing and singular items."""
    import ctypes as C
    rng = np.random.default_rng(7)
    sizes = [int(rng.integers(1, 65)) for _ in range(40)]
    kinds = [i % 2 for i in range(40)]
    mats, rhs = [], []
    for i, (n, k) in enumerate(zip(sizes, kinds)):
        if k == 0:
            m = O.spd(500 + i, n)
            if i % 7 == 3:
                m[n // 2, n // 2] = -1.0                # not SPD
        else:
            m = O.gauss(600 + i, n, n)
            if i % 9 == 5:
                m[:, n // 3] = 0.0                      # exactly singular
        mats.append(np.asfortranarray(m.astype(dtype)))
        rhs.append(O.gauss(700 + i, n, 1)[:, 0].astype(dtype))
    lib = O.port()
    sfx = "d" if dtype == np.float64 else "s"
    for kind in (0, 1):
        idx = [i for i in range(40) if kinds[i] == kind]
        ns = np.array([sizes[i] for i in idx], dtype=np.int32)
        off = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
        roff = np.concatenate([[0], np.cumsum(ns.astype(np.int64))[:-1]]).astype(np.int64)
        a = np.concatenate([mats[i].reshape(-1, order="F") for i in idx]).astype(dtype)
        b = np.concatenate([rhs[i] for i in idx]).astype(dtype)
        info = np.zeros(len(idx), dtype=np.int32)
        if kind == 0:
            getattr(lib, f"oracle_batched_llt_solve_{sfx}")(len(idx), ns, off, a.ctypes.data_as(C.c_void_p), roff,
                                                              b.ctypes.data_as(C.c_void_p), info)
        else:
            tr = np.zeros(int(ns.sum()), dtype=np.int32)
            getattr(lib, f"oracle_batched_lu_solve_{sfx}")(len(idx), ns, off, a.ctypes.data_as(C.c_void_p), roff,
                                                             b.ctypes.data_as(C.c_void_p), tr, info)
        for q, i in enumerate(idx):
            n = sizes[i]
            f = a[off[q]:off[q] + n * n].reshape((n, n), order="F")
            x = b[roff[q]:roff[q] + n]
            if kind == 0:
                fo, io = O.llt(mats[i])
                assert info[q] == io and np.array_equal(np.tril(f), np.tril(fo))
                if io < 0:
                    assert np.array_equal(x, O.llt_solve(fo, rhs[i].reshape(-1, 1))[:, 0], equal_nan=True)
            else:
                fo, tro, _, fz = O.lu(mats[i])
                assert info[q] == fz and np.array_equal(f, fo)
                assert np.array_equal(tr[roff[q]:roff[q] + n], tro)
                assert np.array_equal(x, O.lu_solve(fo, tro, rhs[i].reshape(-1, 1))[:, 0], equal_nan=True)


RANK = G.cases("rank_update")


@pytest.mark.parametrize("case", RANK, ids=[f"n{c['n']}-s{c['sigma']}-{'U' if c['upper'] else 'L'}" for c in RANK])
def test_oracle_llt_rank_update_matches_reference(case):
    """LLT::rankUpdate (LLT.h:231-299) restated in C against the reference:
    the same info (a downdate that loses definiteness fails), the factor within
    1e-12 (the failing downdates: within the recorded floor)."""
    from tests.golden.make_golden import rel as grel
    a = O.spd(case["seed"], case["n"])
    v = O.gauss(case["seed"] + 1, case["n"], 1)[:, 0]
    upper = case["upper"]
    f0, _ = O.llt(a, upper=upper)
    f, r = O.llt_rank_update(f0, v, case["sigma"], upper=upper)
    assert (1 if r >= 0 else 0) == case["info"]
    tri = np.triu if upper else np.tril
    full = G.arr(case, "fact")
    if full is not None:
        assert grel(tri(f), tri(full)) <= max(1e-12, 1.001 * case["floor"])
        assert np.array_equal(f - tri(f), full - tri(full))
    else:
        d = grel(tri(f) @ sketch_matrix(case["n"]), G.arr(case, "fact_sketch"))
        assert d <= max(1e-12, 3 * case["floor"])


BLAS = G.cases("blas")


def blas_id(c):
    keys = ("op", "side", "uplo", "opa", "opb", "diag")
    return "-".join(str(c[k]) for k in keys if k in c) + f"-{c.get('m', c['n'])}x{c['n']}" + \
        ("-f32" if c.get("dtype") == "f32" else "")


@pytest.mark.parametrize("case", BLAS, ids=[blas_id(c) for c in BLAS])
def test_blas_fixtures_follow_the_blas_formulas(case):
    """The reference's BLAS outputs stored in the fixtures satisfy the BLAS
    definitions, checked with plain numpy (a sanity check of the fixtures and of
    the operand rebuild the GPU tests use): gemm C = alpha op(A) op(B) + beta C
    with beta = 0 ignoring C; trsm op(A) X = alpha B (X op(A) = alpha B)
    without reading the diagonal for 'U' or the other triangle; syrk on one
    triangle, the other untouched."""
    from tests.golden.make_golden import blas_inputs
    x, y, z = blas_inputs(case)
    f64 = case.get("dtype") != "f32"
    op = case["op"]
    if op == "gemm":
        oa = (x if case["opa"] in "Nn" else x.T).astype(np.float64)
        ob = (y if case["opb"] in "Nn" else y.T).astype(np.float64)
        zz = np.zeros(z.shape) if case["beta"] == 0 else case["beta"] * z.astype(np.float64)
        want = case["alpha"] * (oa @ ob) + zz
    elif op == "trsm":
        t = (np.tril(x) if case["uplo"] in "Ll" else np.triu(x)).astype(np.float64)
        if case["diag"] in "Uu":
            t[np.diag_indices(t.shape[0])] = 1.0
        t = t if case["opa"] in "Nn" else t.T
        yy = y.astype(np.float64)
        want = case["alpha"] * (np.linalg.solve(t, yy) if case["side"] in "Ll" else np.linalg.solve(t.T, yy.T).T)
    else:
        oa = (x if case["opa"] in "Nn" else x.T).astype(np.float64)
        keep = np.tril if case["uplo"] in "Ll" else np.triu
        zz = np.zeros(y.shape) if case["beta"] == 0 else case["beta"] * y.astype(np.float64)
        want = keep(case["alpha"] * (oa @ oa.T) + zz)
    out = G.arr(case, "out")
    bound = 1e-5 if not f64 else 1e-12
    if out is not None:
        if op == "syrk":
            keep = np.tril if case["uplo"] in "Ll" else np.triu
            other = ~keep(np.ones(out.shape, dtype=bool))
            assert np.array_equal(out[other], y[other], equal_nan=True), "syrk wrote the other triangle"
            assert rel(keep(out), want) <= bound
        else:
            assert rel(out, want) <= bound
    else:
        if op == "syrk":
            keep = np.tril if case["uplo"] in "Ll" else np.triu
            want = want + np.where(~keep(np.ones(want.shape, dtype=bool)), y, 0.0)
        s = sketch_matrix(want.shape[1])
        assert rel(G.arr(case, "out_sketch"), want @ s) <= bound


LDLT = [c for c in G.cases("ldlt") if c["n"] <= MAX_N_CPU]


@pytest.mark.parametrize("case", LDLT, ids=[case_id(c) + ("-" + c["pattern"] if "pattern" in c else "") for c in LDLT])
def test_oracle_ldlt_matches_reference(case):
    """The C restatement of LDLT.h against the reference's own outputs:
    identical transpositions, info and sign; factor and solution within the
    tolerance, or within the recorded noise floor where diagonal pivoting
    grows the rounding (indefinite matrices)."""
    a = G.input(case)
    upper = case.get("upper", False)
    f, tr, ok, sign = O.ldlt(a, upper=upper)
    assert np.array_equal(tr, G.arr(case, "tr")), "transpositions differ from the reference"
    assert (0 if ok else 1) == case["info"]
    assert (sign in (0, 2)) == case["is_positive"] and (sign in (1, 2)) == case["is_negative"]
    full = G.arr(case, "fact")
    tri = (lambda m: np.triu(m) if upper else np.tril(m))
    if full is not None:
        assert np.array_equal(f - tri(f), full - tri(full), equal_nan=True), "the other triangle must stay as given"
        if case["factor_floor"] is None:
            assert np.array_equal(f, full, equal_nan=True)
        else:
            assert rel(tri(f), tri(full)) <= max(tol(case), 1.001 * case["factor_floor"])
    else:
        d = rel(tri(f).astype(np.float64) @ sketch_matrix(case["n"]), G.arr(case, "fact_sketch"))
        assert d <= max(tol(case), 3 * case["factor_floor"])
    b = G.rhs(case, G.arr(case, "x").shape[1])
    x = O.ldlt_solve(f, tr, b, upper=upper)
    if case["x_floor"] is not None:
        assert rel(x, G.arr(case, "x")) <= max(tol(case), 1.001 * case["x_floor"])
    if case["rcond"] is not None and case["info"] == 0 and case["gen"] == "spd":
        rc = O.ldlt_rcond(f, tr, O.sym_l1_norm(a, upper), upper=upper)
        assert rc == pytest.approx(case["rcond"], rel=1e-9 if a.dtype == np.float64 else 1e-4)
