"""The C-ABI library builds, loads without a GPU, and exports every function
include/*.h declares (no compute calls here)."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(gbs_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_functions():
    names = declared_functions()
    assert "gbs_dgetrf" in names and "gbs_llt_blocked_d" in names and "gbs_lu_rcond" in names
    assert len(names) > 40


def test_library_exports_every_declared_symbol():
    from eigen_gb300 import _lib
    L = _lib.lib()   # builds on first use; loads without a GPU
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib._build.LIB)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bgbs_\w+", out))
    assert set(declared_functions()) <= exported
    # the Python binding covers the whole surface
    assert set(declared_functions()) <= set(_lib.PROTOTYPES)


def test_no_device_is_reported_not_faked():
    """Without a usable sm_103 GPU every entry point reports GBS_NO_DEVICE
    (there is no CPU fallback)."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    import ctypes as C
    import numpy as np
    from eigen_gb300 import _lib
    L = _lib.lib()
    assert L.gbs_device_count() == 0
    h = C.c_void_p()
    assert L.gbs_lu_create(C.byref(h), 0) == _lib.GBS_NO_DEVICE
    a = np.asfortranarray(np.eye(3))
    tr = np.zeros(3, dtype=np.int32)
    nbt = C.c_int(0)
    r = L.gbs_partial_lu_blocked_d(3, 3, a.ctypes.data_as(C.c_void_p), 3, tr.ctypes.data_as(C.c_void_p), C.byref(nbt))
    assert r == -(100 + _lib.GBS_NO_DEVICE)
    assert b"device" in L.gbs_last_error()


def test_wait_limit_setter_round_trips():
    """gbs_set_wait_limit is host state only: it returns the previous limit and
    restores the 2 s default for values <= 0."""
    from eigen_gb300 import _lib
    L = _lib.lib()
    first = L.gbs_set_wait_limit(0.25)
    try:
        assert L.gbs_set_wait_limit(0.001) == pytest.approx(0.25)
        assert L.gbs_set_wait_limit(0.0) == pytest.approx(0.001)
        assert L.gbs_set_wait_limit(-1.0) == pytest.approx(2.0)
    finally:
        L.gbs_set_wait_limit(first)
    assert L.gbs_selftest_barrier_timeout() in (_lib.GBS_NO_DEVICE, _lib.GBS_TIMEOUT)
