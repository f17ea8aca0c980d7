"""Mixed-precision factor + FP64 refinement (gbs_dgesv_mixed*) through the C ABI.

Bar: normwise backward error <= 1e-13 for every tier (recomputed here with the
CPU oracle in extended precision, not taken from the library's report), with
the FP64 fallback taking over whenever refinement stalls.  The 3xTF32 tier
(FP32-accurate factors) must converge without fallback on well-conditioned
systems; the solution is also compared with the plain FP64 path.
"""
import numpy as np
import pytest

import oracle as O
from eigen_gb300 import PartialPivLU, solve_mixed, solve_spd_mixed

pytestmark = pytest.mark.gpu
BAR = 1e-13


@pytest.mark.parametrize("tier", ["tf32x3", "tf32", "bf16", "fp16", "fp64"])
@pytest.mark.parametrize("n", [100, 517, 2048])
def test_mixed_reaches_the_backward_error_bar(tier, n):
    a = O.gauss(100 + n, n, n)
    b = O.gauss(200 + n, n, 3)
    x, info = solve_mixed(a, b, tier=tier)
    be = O.backward_error(a, x, b)
    assert be <= BAR, (be, info)
    assert info["backward_error"] <= BAR
    if tier == "tf32x3":
        assert not info["fell_back"] and info["iterations"] <= 10, info
    x64 = PartialPivLU(a).solve(b)
    assert np.linalg.norm(x - x64) / np.linalg.norm(x64) < 1e-9


def test_mixed_many_rhs_groups():
    n = 700
    a = O.gauss(7, n, n)
    b = O.gauss(8, n, 37)            # three refinement groups of <= 16 columns
    x, info = solve_mixed(a, b, tier="tf32x3")
    assert O.backward_error(a, x, b) <= BAR


def test_ill_conditioned_falls_back_and_still_meets_the_bar():
    n = 300
    u, _ = np.linalg.qr(O.gauss(1, n, n))
    v, _ = np.linalg.qr(O.gauss(2, n, n))
    s = np.logspace(0, -13, n)
    a = np.asfortranarray((u * s) @ v.T)
    b = O.gauss(3, n, 2)
    x, info = solve_mixed(a, b, tier="bf16")
    assert info["fell_back"] and info["tier_used"] == "fp64"
    assert O.backward_error(a, x, b) <= BAR


def test_unreachable_tolerance_falls_back():
    n = 256
    a = O.gauss(11, n, n)
    b = O.gauss(12, n, 1)
    x, info = solve_mixed(a, b, tier="tf32x3", tol=0.0, max_iter=4)
    assert info["fell_back"]
    assert O.backward_error(a, x, b) <= BAR


def test_singular_reports_it():
    n = 64
    a = O.gauss(13, n, n)
    a[:, 10] = 0.0
    b = O.gauss(14, n, 1)
    _, info = solve_mixed(a, b, tier="tf32x3")
    assert info["fell_back"] and info["singular"]


def spd_with_condition(n, kappa, seed):
    """A = Q diag(sigma) Q^T, Q Haar-orthogonal (QR of a seeded Gaussian with
    the signs of diag(R) fixed), sigma log-spaced from 1 to kappa."""
    q, r = np.linalg.qr(O.gauss(seed, n, n))
    q = q * np.sign(np.diag(r))
    s = np.logspace(0, np.log10(kappa), n)
    a = (q * s) @ q.T
    return np.asfortranarray((a + a.T) / 2)


@pytest.mark.parametrize("kappa", [1e2, 1e6, 1e10])
@pytest.mark.parametrize("tier", ["tf32x3", "tf32", "bf16", "fp16"])
def test_spd_mixed_tiers_meet_the_bar(tier, kappa):
    from eigen_gb300 import solve_spd_mixed
    n = 640
    a = spd_with_condition(n, kappa, seed=int(np.log10(kappa)) + 17)
    b = O.gauss(23, n, 4)
    x, info = solve_spd_mixed(np.tril(a), b, tier=tier)
    be = O.backward_error(a, x, b)
    assert be <= BAR, (be, info)
    if kappa <= 1e6:
        # the refinement itself converges (no FP64 fallback) for moderate kappa
        assert not info["fell_back"], info


def test_spd_not_positive_definite_is_reported():
    from eigen_gb300 import solve_spd_mixed
    n = 200
    a = -O.spd(3, n)
    b = O.gauss(4, n, 1)
    _, info = solve_spd_mixed(a, b, tier="bf16", allow_not_spd=True)
    assert info["singular"] and info["fell_back"]


@pytest.mark.parametrize("tier", ["tf32", "bf16", "fp16"])
def test_gmres_ir_lets_low_tiers_converge_on_general_matrices(tier):
    n = 1024
    a = O.gauss(31, n, n)
    b = O.gauss(32, n, 2)
    x, info = solve_mixed(a, b, tier=tier, refine="gmres")
    assert info["solver"] == "gmres"
    assert O.backward_error(a, x, b) <= BAR
    assert not info["fell_back"], info


def test_mixed_device_buffers():
    torch = pytest.importorskip("torch")
    n = 1500
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g).t()
    B = torch.randn(4, n, dtype=torch.float64, device="cuda", generator=g).t()
    X, info = solve_mixed(A, B, tier="tf32x3")
    a = np.asfortranarray(A.cpu().numpy())
    assert O.backward_error(a, X.cpu().numpy(), B.cpu().numpy()) <= BAR
    assert not info["fell_back"]


@pytest.mark.parametrize("spd", [False, True])
def test_mixed_device_orders_after_pending_default_stream_work(spd):
    """A NULL stream is the legacy default stream: a solve queued right after
    an unfinished producer of A on that stream must read the finished A."""
    torch = pytest.importorskip("torch")
    from eigen_gb300 import solve_spd_mixed
    n = 3072
    g = torch.Generator(device="cuda").manual_seed(9)
    G = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(2, n, dtype=torch.float64, device="cuda", generator=g).t()
    torch.cuda.synchronize()
    assert torch.cuda.current_stream().cuda_stream == 0
    fn = solve_spd_mixed if spd else solve_mixed
    for _ in range(2):
        A = (G @ G.t() + n * torch.eye(n, dtype=torch.float64, device="cuda")).t()   # ~50 ms of FP64 GEMM, async
        X, info = fn(A, B, tier="fp64")
        X2, _ = fn(A, B, tier="fp64")
        assert torch.equal(X, X2)
        a = np.asfortranarray(A.cpu().numpy())
        assert O.backward_error(a, X.cpu().numpy(), B.cpu().numpy()) <= BAR


@pytest.mark.parametrize("tier", ["tf32x3", "bf16"])
@pytest.mark.parametrize("n", [300, 2048, 4100])
def test_lookahead_gives_identical_results(tier, n):
    """The look-ahead schedule (block k+1's panels on a second stream during
    block k's wide update) performs every element's operations in the same
    order as the single-stream schedule: identical solutions and iterations."""
    a = O.gauss(500 + n, n, n)
    b = O.gauss(600 + n, n, 2)
    x1, i1 = solve_mixed(a, b, tier=tier, lookahead=True)
    x1b, _ = solve_mixed(a, b, tier=tier, lookahead=True)
    assert np.array_equal(x1, x1b), "the look-ahead solve is not deterministic"
    x0, i0 = solve_mixed(a, b, tier=tier, lookahead=False)
    assert np.array_equal(x1, x0)
    assert i1["iterations"] == i0["iterations"] and i1["fell_back"] == i0["fell_back"]
    assert O.backward_error(a, x1, b) <= BAR


@pytest.mark.parametrize("tier", ["tf32x3", "bf16"])
@pytest.mark.parametrize("n", [2048, 3000, 8192])
def test_streamed_host_input_matches_device_buffers(tier, n):
    """From host buffers the LU solve copies A in column chunks that join the
    look-ahead factorization as they land: each late chunk is gathered through
    the interchanges so far, then the earlier blocks' updates are replayed on
    it.  The solution must be bit-identical to the device-buffer solve."""
    torch = pytest.importorskip("torch")
    a = O.gauss(700 + n, n, n)
    b = O.gauss(800 + n, n, 3)
    xh, ih = solve_mixed(a, b, tier=tier)
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    B = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    xd, idv = solve_mixed(A, B, tier=tier)
    assert np.array_equal(xh, xd.cpu().numpy())
    assert (ih["iterations"], ih["fell_back"]) == (idv["iterations"], idv["fell_back"])
    assert O.backward_error(a, xh, b) <= BAR


def test_streamed_host_input_with_padded_leading_dimension():
    """A host matrix with lda > n: every chunk's copy strides over the padding."""
    import ctypes as C
    from eigen_gb300 import _lib
    from eigen_gb300.mixed import RefineInfo, options
    n, pad, nrhs = 3000, 7, 2
    a = O.gauss(901, n, n)
    b = O.gauss(902, n, nrhs)
    ah = np.full((n, n + pad), np.nan)                 # row-major (n, lda): column-major A with lda = n + pad
    ah[:, :n] = a.T
    bh = np.asfortranarray(b)
    x = np.empty((n, nrhs), order="F")
    info = RefineInfo()
    opt = options("tf32x3")
    _lib.check(_lib.lib().gbs_dgesv_mixed(n, nrhs, ah.ctypes.data_as(C.c_void_p), n + pad,
                                          bh.ctypes.data_as(C.c_void_p), n, x.ctypes.data_as(C.c_void_p), n,
                                          C.byref(opt), C.byref(info)), "gbs_dgesv_mixed")
    x0, _ = solve_mixed(a, b, tier="tf32x3")
    assert np.array_equal(x, x0)
    assert O.backward_error(a, x, b) <= BAR


@pytest.mark.parametrize("n", [700, 2500])
def test_spd_host_solve_reads_the_lower_triangle_only(n):
    """Like Eigen's LLT (only the lower triangle of A is considered), the SPD
    host solve copies just the lower trapezoid of each column block: NaN in the
    strict upper triangle must not change the solution."""
    a = spd_with_condition(n, 1e3, 77)
    b = O.gauss(78, n, 2)
    x0, i0 = solve_spd_mixed(a, b, tier="tf32x3")
    au = a.copy()
    au[np.triu_indices(n, 1)] = np.nan
    x1, i1 = solve_spd_mixed(au, b, tier="tf32x3")
    assert np.array_equal(x0, x1)
    assert i0["iterations"] == i1["iterations"]
    assert O.backward_error(a, x1, b) <= BAR
    torch = pytest.importorskip("torch")            # and from device buffers holding the NaNs
    A = torch.from_numpy(np.ascontiguousarray(au.T)).cuda().t()
    B = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    x2, _ = solve_spd_mixed(A, B, tier="tf32x3")
    assert np.array_equal(x0, x2.cpu().numpy())


@pytest.mark.parametrize("tier", ["tf32x3", "bf16"])
@pytest.mark.parametrize("n", [600, 2048, 5000])
def test_tournament_and_partial_pivoting_both_converge(tier, n):
    """Tournament pivoting (an option of the mixed LU's panels) against the
    reference's partial pivoting: both reach the bound and agree to the
    conditioning.  Classic refinement needs the same number of steps
    (within one); GMRES on 16-bit factors may need more inner iterations with
    tournament pivoting (its growth factor is larger), but at most 1.6x."""
    a = O.gauss(700 + n, n, n)
    b = O.gauss(800 + n, n, 3)
    x_t, i_t = solve_mixed(a, b, tier=tier, pivoting="tournament")
    x_p, i_p = solve_mixed(a, b, tier=tier, pivoting="partial")
    for x, info in ((x_t, i_t), (x_p, i_p)):
        assert O.backward_error(a, x, b) <= BAR, info
        if tier == "tf32x3":
            assert not info["fell_back"], info
    if tier == "tf32x3":
        assert abs(i_t["iterations"] - i_p["iterations"]) <= 1, (i_t, i_p)
    elif not i_t["fell_back"] and not i_p["fell_back"]:
        assert i_t["inner_iterations"] <= 1.6 * i_p["inner_iterations"] + 5, (i_t, i_p)
    assert np.linalg.norm(x_t - x_p) / np.linalg.norm(x_p) <= 1e-9


def test_tournament_pivoting_on_hard_panels():
    """Panels that defeat a careless candidate choice: rows whose magnitudes
    span 30 orders, a block of exactly dependent rows (rank-deficient
    candidates in one CTA), and a lower-triangular matrix (every pivot sits
    on the diagonal).  Each solve meets the bound, by refinement or by the
    FP64 fallback."""
    n = 3000
    rng = np.random.default_rng(4)
    a1 = O.gauss(41, n, n) * (10.0 ** rng.uniform(-15, 15, n))[:, None]
    a2 = O.gauss(42, n, n)
    a2[100:900] = a2[100] * rng.uniform(0.5, 2.0, 800)[:, None] + 1e-3 * a2[100:900]
    a3 = np.tril(O.gauss(43, n, n)) + 50.0 * np.eye(n)
    for a in (a1, a2, a3):
        b = O.gauss(44, n, 2)
        x, info = solve_mixed(a, b, tier="tf32x3", pivoting="tournament")
        assert O.backward_error(a, x, b) <= BAR, info


@pytest.mark.parametrize("tier", ["tf32x3", "fp16"])
@pytest.mark.parametrize("n", [1500, 3000])
def test_spd_lookahead_gives_identical_results(tier, n):
    """The Cholesky's look-ahead schedule (block k+1's diagonal factor and
    TRSM beside block k's wide SYRK) gives the single-stream results exactly."""
    a = O.spd(900 + n, n)
    b = O.gauss(901 + n, n, 2)
    x1, i1 = solve_spd_mixed(a, b, tier=tier, lookahead=True)
    x0, i0 = solve_spd_mixed(a, b, tier=tier, lookahead=False)
    assert np.array_equal(x1, x0)
    assert i1["iterations"] == i0["iterations"] and i1["fell_back"] == i0["fell_back"]
    assert O.backward_error(a, x1, b) <= BAR
