"""Failure detection and concurrent use on the GPU.

Every wait of one CTA on another gives up after a wall-time limit
(gbs_set_wait_limit), the call reports GBS_TIMEOUT and the CUDA context stays
usable.  The waits are made to run out without any GPU fault: a ready flag that
no CTA ever publishes (the persistent triangular solve with block 0's ticket
skipped) and a grid barrier that counts one CTA more than the launch has.

The reference's CPU code has no inter-thread waits; its counterpart of the
concurrency check is that independent decompositions can be used from several
threads at once (each object owns its state), which the threaded test below
exercises through the C ABI: four host threads factoring and solving different
systems at the same time, each result checked against the oracle.
"""
import ctypes as C
import threading
import time

import numpy as np
import pytest

import oracle as O
from eigen_gb300 import _lib, solve_mixed

pytestmark = pytest.mark.gpu


@pytest.fixture
def short_waits():
    L = _lib.lib()
    prev = L.gbs_set_wait_limit(0.005)
    yield L
    L.gbs_set_wait_limit(prev)


def normal_solve_works():
    n = 384
    a = O.gauss(5, n, n)
    b = O.gauss(6, n, 2)
    x, info = solve_mixed(a, b, tier="fp64")
    return O.backward_error(a, x, b) <= 1e-13


@pytest.mark.parametrize("n", [64, 4096])
def test_unpublished_ready_flag_times_out(short_waits, n):
    L = short_waits
    t0 = time.perf_counter()
    rc = L.gbs_selftest_solve_timeout(n)
    dt = time.perf_counter() - t0
    assert rc == _lib.GBS_TIMEOUT, (rc, L.gbs_last_error())
    assert b"timed out" in L.gbs_last_error()
    assert dt < 1.0, f"the 5 ms limit was not honoured: {dt:.3f} s"
    assert normal_solve_works(), "the context is unusable after the timeout"


def test_grid_barrier_times_out(short_waits):
    L = short_waits
    t0 = time.perf_counter()
    rc = L.gbs_selftest_barrier_timeout()
    assert rc == _lib.GBS_TIMEOUT, (rc, L.gbs_last_error())
    assert time.perf_counter() - t0 < 1.0
    assert normal_solve_works()


def test_default_limit_is_restored_after_a_timeout():
    L = _lib.lib()
    prev = L.gbs_set_wait_limit(0.002)
    try:
        assert L.gbs_selftest_barrier_timeout() == _lib.GBS_TIMEOUT
    finally:
        L.gbs_set_wait_limit(0.0)
    # a full-size factorization with the default limit: no spurious timeout
    n = 4096
    a = O.gauss(9, n, n)
    b = O.gauss(10, n, 1)
    x, _ = solve_mixed(a, b, tier="fp64")
    assert O.backward_error(a, x, b) <= 1e-13
    L.gbs_set_wait_limit(prev)


def _getrf(a):
    L = _lib.lib()
    f = np.array(a, order="F", copy=True)
    n = f.shape[0]
    ipiv = np.zeros(n, dtype=np.int32)
    info = C.c_int(-7)
    ci = lambda v: C.byref(C.c_int(v))
    rc = L.gbs_dgetrf(ci(n), ci(n), f.ctypes.data_as(C.c_void_p), ci(n), ipiv.ctypes.data_as(C.c_void_p),
                      C.byref(info))
    return rc, f, ipiv, info.value


def test_four_threads_factor_and_solve_concurrently():
    """gbs_dgetrf and gbs_dgesv_mixed from four host threads at once on
    different matrices: factors, pivots and solutions as when run alone."""
    cases = []
    for t in range(4):
        n = 700 + 123 * t
        a = O.gauss(300 + t, n, n)
        f, tr, _, _ = O.lu(a)
        b = O.gauss(400 + t, n, 2)
        cases.append((a, f, tr + 1, b))
    errors = []
    start = threading.Barrier(4)

    def worker(t):
        a, f_ref, ipiv_ref, b = cases[t]
        try:
            start.wait()
            for _ in range(3):
                rc, f, ipiv, info = _getrf(a)
                assert rc == 0 and info == 0, (rc, info)
                assert np.array_equal(ipiv, ipiv_ref), "pivots differ from the oracle"
                d = np.linalg.norm(f - f_ref) / np.linalg.norm(f_ref)
                assert d <= 1e-12, d
                x, rinfo = solve_mixed(a, b, tier="tf32x3")
                be = O.backward_error(a, x, b)
                assert be <= 1e-13, (be, rinfo)
        except BaseException as e:       # reported by the main thread
            errors.append((t, repr(e)))

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join(timeout=300)
    assert not any(th.is_alive() for th in threads), "a worker did not finish"
    assert not errors, errors
