"""The tcgen05 trailing-update kernel (gbs_tc_gemm_sub) against an FP64
reference of the same operation with the operands rounded to the tier's
precision (FP32 accumulation is the only remaining error).

Tolerances (relative Frobenius of C_gpu - C_ref over the update's scale
||A|| ||B||): 2e-6 for BF16/FP16/TF32 against rounded operands, and 4e-6 for
3xTF32 against the unrounded FP32 operands (FP32-level accuracy).
"""
import ctypes as C

import numpy as np
import pytest

from eigen_gb300 import _lib

pytestmark = pytest.mark.gpu


def round_tf32(x):
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((b + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)   # round half away from zero
    return r.reshape(x.shape)


def rounded(x, kind):
    torch = pytest.importorskip("torch")
    if kind == 0:
        return torch.from_numpy(x).bfloat16().float().numpy()
    if kind == 1:
        return torch.from_numpy(x).half().float().numpy()
    if kind == 2:
        return round_tf32(x)
    return x


def run(kind, m, n, k, lower=False, seed=0):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = a.T.copy() if lower else rng.standard_normal((k, n)).astype(np.float32)
    c = rng.standard_normal((m, n)).astype(np.float32)
    dA = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    dB = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    dC = torch.from_numpy(np.ascontiguousarray(c.T)).cuda().t()
    torch.cuda.synchronize()
    rc = _lib.lib().gbs_tc_gemm_sub(kind, m, n, k, C.c_void_p(dA.data_ptr()), m, C.c_void_p(dB.data_ptr()), k,
                                    C.c_void_p(dC.data_ptr()), m, int(lower), None)
    _lib.check(rc, "gbs_tc_gemm_sub")
    torch.cuda.synchronize()
    out = dC.cpu().numpy()
    ar, br = rounded(a, kind).astype(np.float64), rounded(b, kind).astype(np.float64)
    ref = c.astype(np.float64) - ar @ br
    if lower:
        mask = np.tril(np.ones((m, n), dtype=bool))
        assert np.array_equal(out[~mask], c[~mask]), "strict upper triangle must stay untouched"
        ref = np.where(mask, ref, c)
    scale = np.linalg.norm(ar) * np.linalg.norm(br) / np.sqrt(k)
    return np.linalg.norm(out - ref) / scale


@pytest.mark.parametrize("kind", [0, 1, 2, 3], ids=["bf16", "fp16", "tf32", "tf32x3"])
@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (300, 200, 32), (1000, 777, 128), (129, 257, 31), (2048, 1536, 96)])
def test_tc_gemm_matches_reference(kind, m, n, k):
    err = run(kind, m, n, k, seed=m + n + k)
    assert err < (4e-6 if kind == 3 else 2e-6), err


@pytest.mark.parametrize("kind", [0, 3], ids=["bf16", "tf32x3"])
def test_tc_syrk_lower_only(kind):
    err = run(kind, 700, 700, 64, lower=True, seed=5)
    assert err < 4e-6


def test_tc_gemm_large_many_tiles():
    err = run(0, 4096, 4096, 128, seed=9)
    assert err < 2e-6
