"""The Eigen plug-in header (include/eigen_gb300/GB300Support) against the
reference's own headers, on CPU: the same program is built twice -- stock
Eigen, and Eigen + the plug-in linked to a test double of the plug-in level
of the C ABI (tests/plugin/mock_gbs.c, which forwards to the C oracle) -- and
both must print the same results, with every factorization routed through
the plug-in.  Needs the reference tree (Eigen headers) and g++; skipped where
they are absent.  The GPU side of these four functions is covered by
tests/test_gpu_dense.py.
"""
import subprocess
from pathlib import Path

import pytest

from oracle import build as obuild

ROOT = Path(__file__).resolve().parents[1]
PLUG = ROOT / "tests" / "plugin"


def _build(tmp_path, with_plugin):
    out = tmp_path / ("with" if with_plugin else "stock")
    cmd = ["g++", "-O2", "-std=c++14", "-w", f"-I{obuild.REF_ROOT}", f"-I{ROOT / 'include'}",
           str(PLUG / "plugin_test.cpp"), "-o", str(out)]
    if with_plugin:
        objs = []
        for src in (PLUG / "mock_gbs.c", ROOT / "oracle" / "dense_oracle.c"):
            o = tmp_path / (src.stem + ".o")
            r = subprocess.run(["gcc", "-O2", "-std=gnu11", "-c", str(src), "-o", str(o)], capture_output=True,
                               text=True)
            assert r.returncode == 0, r.stderr[-2000:]
            objs.append(str(o))
        cmd[1:1] = ["-DUSE_GB300"]
        cmd += objs + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    run = subprocess.run([str(out)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stderr
    return dict(line.split(" ", 1) for line in run.stdout.strip().splitlines())


def _fields(s):
    out = {}
    for tok in s.split():
        if "=" in tok:
            k, v = tok.split("=")
            out[k] = float(v)
    return out


@pytest.mark.skipif(not obuild.reference_available(), reason="reference headers not present")
def test_plugin_routes_eigen_api_and_matches_stock_eigen(tmp_path):
    stock = _build(tmp_path, False)
    plug = _build(tmp_path, True)
    assert plug["plugin_calls"].strip() == "8", "every LLT / PartialPivLU compute must go through the plug-in"
    for key in ("llt_lower", "llt_upper", "llt_rowmajor", "llt_negative", "llt_inplace", "lu", "lu_float",
                "lu_inplace"):
        a, b = _fields(stock[key]), _fields(plug[key])
        assert a.keys() == b.keys(), key
        for k in a:
            if k in ("info", "p0", "p1", "p5", "plast", "modified"):
                assert a[k] == b[k], (key, k, a[k], b[k])     # integer results: identical
            else:
                tol = 1e-4 if key == "lu_float" else 1e-10
                assert abs(a[k] - b[k]) <= tol * max(1.0, abs(a[k])), (key, k, a[k], b[k])
