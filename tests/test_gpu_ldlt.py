"""Parity of the GPU LDLT (gbs_ldlt_*, Cholesky with diagonal pivoting) with the
reference's LDLT<Matrix, Lower|Upper> (Eigen/src/Cholesky/LDLT.h).

Every call goes through the C ABI.  Checked against the golden fixtures (the
reference's own outputs) and the CPU oracle (pinned to them by
test_oracle_golden.py):
  * transpositionsP() identical to the reference's, bit for bit;
  * info(), isPositive(), isNegative() identical, including the zero-pivot
    rules (a zero pivot whose column is not zero below the diagonal, a nonzero
    pivot after a zero one, the whole diagonal zero, a NaN first pivot);
  * matrixLDLT() within 1e-12 relative Frobenius of the reference (FP32 2e-5),
    or, for indefinite matrices, whose diagonal pivoting lets rounding grow,
    within 10x the reference's own noise floor (its distance to the C
    restatement of the same algorithm); the other triangle as given;
  * solve() within 1e-12 of the reference (or 10x its noise floor), backward
    error at the FP64 floor (1e-14), or within 10x the reference's own where
    growth raises it (indefinite matrices);
  * rcond() equal to the reference's to 1e-6 for SPD matrices.
"""
import numpy as np
import pytest

import oracle as O
from eigen_gb300 import LDLT, _lib
from tests.conftest import Golden, case_id, record_parity
from tests.golden.make_golden import sketch_matrix

pytestmark = pytest.mark.gpu
G = Golden()
CASES = G.cases("ldlt")


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def check(case, what, value, bound):
    record_parity(case_id(case), what, value, bound)
    assert value <= bound, f"{what}: {value:.3e} > {bound:.1e}"


@pytest.mark.parametrize("case", CASES, ids=[case_id(c) + ("-" + c["pattern"] if "pattern" in c else "") for c in CASES])
def test_ldlt_matches_reference(case):
    a = G.input(case)
    upper = case.get("upper", False)
    f64 = a.dtype == np.float64
    ldlt = LDLT(a, upper=upper)
    assert np.array_equal(ldlt.transpositionsP(), G.arr(case, "tr")), "transpositions differ from the reference"
    assert (ldlt.info() == _lib.GBS_SUCCESS) == (case["info"] == 0)
    assert ldlt.isPositive() == case["is_positive"] and ldlt.isNegative() == case["is_negative"]
    if np.isfinite(case["l1_norm"]):
        assert ldlt.l1_norm() == pytest.approx(case["l1_norm"], rel=1e-12 if f64 else 1e-5)
    m = ldlt.matrixLDLT()
    tri = (lambda x: np.triu(x) if upper else np.tril(x))
    assert np.array_equal(m - tri(m), a - tri(a), equal_nan=True), "the other triangle must stay as given"
    tol = 1e-12 if f64 else 2e-5
    floor = case["factor_floor"]
    bound = tol if floor is None else max(tol, 10 * floor)
    full = G.arr(case, "fact")
    if full is not None:
        if floor is None:
            assert np.array_equal(m, full, equal_nan=True)
        else:
            check(case, "LDLT factor vs reference (whole)", rel(tri(m), tri(full)), bound)
            f_o, _, _, _ = O.ldlt(a, upper=upper)
            check(case, "LDLT factor vs C restatement (whole)", rel(tri(m), tri(f_o)), bound)
    else:
        idx = G.arr(case, "fact_idx")
        check(case, "LDLT factor vs reference (2048 entries)",
              rel(tri(m).reshape(-1, order="F")[idx], G.arr(case, "fact_val")), bound)
        check(case, "LDLT factor vs reference (whole, sketch)",
              rel(tri(m).astype(np.float64) @ sketch_matrix(case["n"]), G.arr(case, "fact_sketch")), bound)
        f_o, _, _, _ = O.ldlt(a, upper=upper)
        check(case, "LDLT factor vs C restatement (whole)", rel(tri(m), tri(f_o)), bound)
    assert np.array_equal(ldlt.vectorD(), np.diag(m), equal_nan=True)
    b = G.rhs(case, G.arr(case, "x").shape[1])
    x = ldlt.solve(b)
    if case["x_floor"] is not None:
        xb = max(1e-12 if f64 else 1e-5, 10 * case["x_floor"])
        check(case, "LDLT solution vs reference", rel(x, G.arr(case, "x")), xb)
    if f64 and case["info"] == 0 and case["gen"] in ("spd", "sym_gauss"):
        # diagonal pivoting does not bound the growth on indefinite matrices:
        # the bar is the reference's own backward error on the same system
        sym = np.asfortranarray(np.triu(a) + np.triu(a, 1).T if upper else np.tril(a) + np.tril(a, -1).T)
        be_ref = O.backward_error(sym, G.arr(case, "x"), b)
        check(case, "LDLT solve backward error", O.backward_error(sym, x, b), max(1e-14, 10 * be_ref))
    if case["gen"] == "spd" and case["rcond"] is not None:
        assert ldlt.rcond() == pytest.approx(case["rcond"], rel=1e-6 if f64 else 1e-3)


def test_ldlt_reconstructs_the_matrix_and_solves_on_device_buffers():
    """P^T L D L^T P equals A; the device-buffer entry points give the host
    entry points' results (torch tensors, column-major)."""
    torch = pytest.importorskip("torch")
    n = 300
    g = O.gauss(77, n, n)
    a = np.asfortranarray((g + g.T) / 2 + 0.1 * np.eye(n))
    ldlt = LDLT(a)
    assert rel(ldlt.reconstructedMatrix(), a) < 1e-10
    b = O.gauss(78, n, 3)
    x = ldlt.solve(b)
    da = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    db = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    ld = LDLT(da)
    xd = ld.solve(db).cpu().numpy()
    assert np.array_equal(ld.transpositionsP(), ldlt.transpositionsP())
    assert rel(xd, x) < 1e-12
    # an indefinite matrix: the bar is the reference algorithm's own backward error
    f_o, tr_o, _, _ = O.ldlt(a)
    be_o = O.backward_error(a, O.ldlt_solve(f_o, tr_o, b), b)
    assert O.backward_error(a, xd, b) < max(1e-14, 10 * be_o)


def test_ldlt_large_spd_matches_oracle():
    """n = 3000 SPD, beyond the fixtures' sizes: transpositions equal the C
    restatement's, the whole factor within 1e-12, backward error at the FP64
    floor."""
    n = 3000
    a = O.spd(4321, n)
    ldlt = LDLT(a)
    f_o, tr_o, ok_o, sign_o = O.ldlt(a)
    assert np.array_equal(ldlt.transpositionsP(), tr_o)
    assert ldlt.info() == _lib.GBS_SUCCESS and ok_o
    d = rel(np.tril(ldlt.matrixLDLT()), np.tril(f_o))
    record_parity("ldlt-spd-3000", "LDLT factor vs C restatement (whole)", d, 1e-12)
    assert d < 1e-12
    b = O.gauss(4322, n, 2)
    assert O.backward_error(a, ldlt.solve(b), b) < 1e-14
