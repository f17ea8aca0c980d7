"""FP64-accurate residuals R = B - A X (gbs_dgeresid_device): the FP64 FMA
kernels and the Ozaki-scheme tensor-core kernels against an extended-precision
reference (numpy longdouble on sampled rows).

Bar: |R - R_ref| <= 2^-48 (|A| |X|)(r, c) elementwise on the sampled rows --
a few units of FP64 rounding of the row's absolute product, what an FP64 GEMV
achieves on such data -- under cancellation (B = fl(A X) + small
perturbations), ragged sizes, rows and columns scaled over 10^+-150, zero rows
and columns; non-finite entries give NaN in their row / column and nowhere
else.  The refinement reaches the same backward error with either residual.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from eigen_gb300 import _lib, solve_mixed

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
from tests.conftest import record_parity  # noqa: E402

METHODS = {"fp64": 1, "ozaki": 2}
BAR = 2.0 ** -48


def col_major(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).cuda().t()


def resid(a, x, b, method):
    n, nrhs = x.shape
    da, dx = col_major(a), col_major(x)
    db = col_major(b) if b is not None else None
    dr = col_major(np.zeros((n, nrhs)))
    rc = _lib.lib().gbs_dgeresid_device(n, nrhs, C.c_void_p(da.data_ptr()), n, C.c_void_p(dx.data_ptr()), n,
                                        C.c_void_p(db.data_ptr()) if db is not None else None, n,
                                        C.c_void_p(dr.data_ptr()), n, METHODS[method], None)
    _lib.check(rc, "gbs_dgeresid_device")
    return dr.cpu().numpy()


def reference(a, x, b, rows):
    al = a[rows].astype(np.longdouble)
    xl = x.astype(np.longdouble)
    ax = al @ xl
    r = (b[rows].astype(np.longdouble) - ax) if b is not None else ax
    scale = np.abs(a[rows]).astype(np.longdouble) @ np.abs(xl)
    return r, scale


def check(a, x, b, tag, rows=None):
    n = a.shape[0]
    rng = np.random.default_rng(7)
    rows = rows if rows is not None else np.sort(rng.choice(n, size=min(n, 48), replace=False))
    ref, scale = reference(a, x, b, rows)
    for m in METHODS:
        r = resid(a, x, b, m)[rows]
        fin = np.isfinite(scale)
        err = np.abs(r.astype(np.longdouble) - ref)
        worst = float(np.max(np.where(fin & (scale > 0), err / np.where(scale > 0, scale, 1), 0)))
        record_parity(tag, f"residual {m} / (|A||X|)", worst, BAR)
        assert worst <= BAR, (m, worst)
        assert np.all(r[scale == 0] == (b[rows][scale == 0] if b is not None else 0)), m


@pytest.mark.parametrize("n,nrhs", [(100, 1), (1000, 5), (2048, 16), (4100, 16), (1025, 3)])
def test_residual_under_cancellation(n, nrhs):
    a = O.gauss(10 + n, n, n)
    x = O.gauss(20 + n, n, nrhs) * 1e3
    b = a @ x                                                     # FP64 product: R is pure rounding
    b += np.random.default_rng(n).standard_normal(b.shape) * 1e-9
    check(a, x, b, f"cancellation n={n} nrhs={nrhs}")


def test_residual_scaled_rows_and_columns():
    n, nrhs = 1536, 7
    rng = np.random.default_rng(3)
    a = O.gauss(5, n, n) * (10.0 ** rng.integers(-150, 150, n))[:, None]
    a[11, :] = 0.0                                               # a zero row
    a[:, 17] *= 1e-40                                            # a column far below the rest of its rows
    x = O.gauss(6, n, nrhs) * (10.0 ** rng.integers(-150, 150, nrhs))[None, :]
    x[:, 2] = 0.0                                                 # a zero column
    b = a @ x
    check(a, x, b, "scaled rows / columns", rows=np.r_[0:8, 11, 17, 500:520, n - 8:n])
    check(a, x, None, "A X only", rows=np.r_[0:8, 11, n - 8:n])


def test_residual_nonfinite_entries_stay_local():
    n, nrhs = 1100, 4
    a = O.gauss(8, n, n)
    x = O.gauss(9, n, nrhs)
    b = O.gauss(10, n, nrhs)
    a[5, 40] = np.nan
    a[9, 3] = np.inf
    x[77, 2] = np.nan
    for m in METHODS:
        r = resid(a, x, b, m)
        assert np.all(np.isnan(r[5])) and not np.isfinite(r[9]).any()
        assert np.all(np.isnan(r[:, 2]))
        keep = np.ones(n, bool)
        keep[[5, 9]] = False
        assert np.all(np.isfinite(r[keep][:, [0, 1, 3]])), m


@pytest.mark.parametrize("tier", ["tf32x3", "bf16"])
def test_refinement_same_with_either_residual(tier):
    n = 3000
    a = O.gauss(31, n, n)
    b = O.gauss(32, n, 4)
    x_o, i_o = solve_mixed(a, b, tier=tier, residual="ozaki")
    x_f, i_f = solve_mixed(a, b, tier=tier, residual="fp64")
    assert O.backward_error(a, x_o, b) <= 1e-13 and O.backward_error(a, x_f, b) <= 1e-13
    assert abs(i_o["iterations"] - i_f["iterations"]) <= 1, (i_o, i_f)
    assert np.linalg.norm(x_o - x_f) / np.linalg.norm(x_f) <= 1e-9      # both within kappa * 1e-13
    # the library's own backward error (from its residual) agrees with the oracle's
    assert i_o["backward_error"] == pytest.approx(O.backward_error(a, x_o, b), rel=1e-2, abs=1e-17)
