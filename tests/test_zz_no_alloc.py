"""The allocation-free LU entry point, gbs_dgetrf_noalloc.

It serves callers that cannot let a library call cudaMalloc: real-time loops
that run under a no-allocation rule, and applications that give all device
memory to their own pool.  Through the C ABI, these tests check that it
returns the same factors, pivots and info as the existing entry point
gbs_dgetrf on two calls in a row (the shared scratch keeps the previous
call's contents), that a call leaves the device's free memory unchanged, and
that sizes beyond its fixed scratch are refused.

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from eigen_gb300 import _lib

pytestmark = pytest.mark.gpu

FACTOR_TOL = 1e-12   # the factor tolerance of the other FP64 parity tests


def _existing_getrf(a):
    """gbs_dgetrf (host buffers): factors, 1-based ipiv, info."""
    L = _lib.lib()
    f = np.array(a, order="F", copy=True, dtype=np.float64)
    m, n = f.shape
    ipiv = np.zeros(max(min(m, n), 1), dtype=np.int32)
    info = C.c_int(0)
    ci = lambda v: C.byref(C.c_int(v))
    _lib.check(L.gbs_dgetrf(ci(m), ci(n), f.ctypes.data_as(C.c_void_p), ci(max(m, 1)),
                            ipiv.ctypes.data_as(C.c_void_p), C.byref(info)), "gbs_dgetrf")
    return f, ipiv[: min(m, n)], info.value


def _noalloc_getrf(torch, a):
    """gbs_dgetrf_noalloc on device buffers: factors, 1-based ipiv, info."""
    L = _lib.lib()
    m, n = a.shape
    d_a = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()     # column-major, lda = m
    d_ipiv = torch.zeros(max(min(m, n), 1), dtype=torch.int32, device="cuda")
    d_info = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = L.gbs_dgetrf_noalloc(m, n, C.c_void_p(d_a.data_ptr()), max(m, 1), C.c_void_p(d_ipiv.data_ptr()),
                              C.c_void_p(d_info.data_ptr()), C.c_void_p(stream.cuda_stream))
    _lib.check(rc, "gbs_dgetrf_noalloc")
    stream.synchronize()
    return (np.asfortranarray(d_a.cpu().numpy()), d_ipiv.cpu().numpy()[: min(m, n)], int(d_info.cpu().item()))


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _same(torch, a):
    f0, p0, i0 = _existing_getrf(a)
    f1, p1, i1 = _noalloc_getrf(torch, a)
    assert i1 == i0
    assert np.array_equal(p1, p0)
    assert _rel(f1, f0) <= FACTOR_TOL


def test_noalloc_matches_existing_entry_point_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    a1 = O.gauss(31337, 700, 700)
    a2 = O.gauss(31338, 1000, 600)          # second call: different shape, tall
    _same(torch, a1)
    _same(torch, a2)
    singular = O.gauss(31339, 300, 300)
    singular[:, 123] = 0.0                  # info = 124 from both entry points
    _same(torch, singular)
    _same(torch, a1)                        # the scratch's old contents do not leak into a new call


@pytest.mark.parametrize("m,n", [(12000, 64), (40000, 32)])
def test_noalloc_tall_panels_match_existing_entry_point(m, n):
    """Panels taller than one thread-block cluster holds (m > 8192) run on the
    grid-cooperative panel kernel, whose candidate-exchange buffers and grid
    barrier counters live in the fixed array; 40000 rows need two rows per
    thread.  Two calls in a row, each equal to gbs_dgetrf."""
    torch = pytest.importorskip("torch")
    a = O.gauss(52000 + m, m, n)
    _same(torch, a)
    _same(torch, a)


def test_noalloc_leaves_device_free_memory_unchanged():
    """After one small call (the per-device set-up), calls of other shapes --
    a square matrix on the cluster panel and a tall one on the cooperative
    panel, with other GEMM tile sizes -- leave free device memory unchanged."""
    torch = pytest.importorskip("torch")
    _noalloc_getrf(torch, O.gauss(4710, 40, 40))     # first call on this device: set-up
    L = _lib.lib()
    shapes = [(900, 900), (20000, 48)]
    bufs = []
    for i, (m, n) in enumerate(shapes):
        a = O.gauss(4711 + i, m, n)
        bufs.append((m, n, torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t(),
                     torch.zeros(min(m, n), dtype=torch.int32, device="cuda"),
                     torch.full((1,), -7, dtype=torch.int32, device="cuda")))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        for m, n, d_a, d_ipiv, d_info in bufs:
            _lib.check(L.gbs_dgetrf_noalloc(m, n, C.c_void_p(d_a.data_ptr()), m, C.c_void_p(d_ipiv.data_ptr()),
                                            C.c_void_p(d_info.data_ptr()),
                                            C.c_void_p(torch.cuda.current_stream().cuda_stream)), "noalloc")
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert all(int(b[4].item()) == 0 for b in bufs)


def test_noalloc_refuses_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = _lib.lib()
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    ip = torch.zeros(4, dtype=torch.int32, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.gbs_dgetrf_noalloc(65537, 1, C.c_void_p(dummy.data_ptr()), 65537, C.c_void_p(ip.data_ptr()),
                              C.c_void_p(info.data_ptr()), None)
    assert rc == _lib.GBS_INVALID_ARGUMENT
    assert b"65536" in L.gbs_last_error()
    rc = L.gbs_dgetrf_noalloc(4, 4, C.c_void_p(dummy.data_ptr()), 3, C.c_void_p(ip.data_ptr()),
                              C.c_void_p(info.data_ptr()), None)
    assert rc == _lib.GBS_INVALID_ARGUMENT
