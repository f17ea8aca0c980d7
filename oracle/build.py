"""Build recipe for the CPU oracle (test infrastructure, not the product).

* ``oracle/_build/liboracle.so`` -- the plain-C restatement (dense_oracle.c),
  compiled on whatever host runs the tests (x86 here, Arm on the GPU host).
  ``-ffp-contract=off`` keeps its results identical on both.
* ``oracle/_ref/libeigen_ref.so`` -- the reference itself: a small C++ wrapper
  (eigen_ref.cpp) over Eigen's own LLT / PartialPivLU / rcond plus Eigen's own
  LAPACK shim (lapack/lu.cpp, lapack/cholesky.cpp, blas/xerbla.cpp) and BLAS
  level-3 shim (blas/level3_impl.h), compiled
  directly from the read-only reference tree.  Built only where that tree is
  present; the fixtures it produces are committed under tests/golden/.

The reference's AVX-512 code path crashes in large products, so the x86 build
uses ``-mavx2 -mfma``; elsewhere the default target is used.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_ROOT = Path(os.environ.get("EIGEN_REFERENCE_ROOT", "/root/reference"))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"oracle build failed: {cmd[0]} exited {r.returncode}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_oracle(force: bool = False) -> Path:
    out_dir = HERE / "_build"
    out_dir.mkdir(exist_ok=True)
    out = out_dir / "liboracle.so"
    deps = [HERE / "dense_oracle.c", HERE / "dense_oracle_impl.h"]
    if force or _stale(out, deps):
        tmp = out.with_suffix(f".so.tmp{os.getpid()}")
        _run(["gcc", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=gnu11",
              "-o", str(tmp), str(HERE / "dense_oracle.c"), "-lm"])
        os.replace(tmp, out)
    return out


def reference_available() -> bool:
    return (REF_ROOT / "Eigen" / "Cholesky").exists()


def build_reference(force: bool = False) -> Path | None:
    """Compile Eigen (from the reference tree) into oracle/_ref/libeigen_ref.so."""
    if not reference_available():
        return None
    out_dir = HERE / "_ref"
    out_dir.mkdir(exist_ok=True)
    out = out_dir / "libeigen_ref.so"
    deps = [HERE / "eigen_ref.cpp", HERE / "eigen_lapack_ref.cpp", HERE / "eigen_blas_ref.cpp"]
    if not (force or _stale(out, deps)):
        return out
    arch = ["-mavx2", "-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    inc = [f"-I{REF_ROOT}", f"-I{REF_ROOT / 'lapack'}", f"-I{REF_ROOT / 'blas'}"]
    common = ["g++", "-O3", "-DNDEBUG", "-fopenmp", "-fPIC", "-std=c++14", "-w"] + arch + inc
    objs = []
    for src, defs in (("eigen_ref.cpp", []),
                      ("eigen_lapack_ref.cpp", ["-DGB_REF_DOUBLE"]),
                      ("eigen_lapack_ref.cpp", ["-DGB_REF_SINGLE"]),
                      ("eigen_blas_ref.cpp", ["-DGB_REF_DOUBLE"]),
                      ("eigen_blas_ref.cpp", ["-DGB_REF_SINGLE"])):
        o = out_dir / (Path(src).stem + ("".join(d[2:].lower() for d in defs) or "") + ".o")
        _run(common + defs + ["-c", str(HERE / src), "-o", str(o)])
        objs.append(str(o))
    xo = out_dir / "xerbla.o"
    _run(common + ["-c", str(REF_ROOT / "blas" / "xerbla.cpp"), "-o", str(xo)])
    objs.append(str(xo))
    tmp = out.with_suffix(f".so.tmp{os.getpid()}")
    _run(["g++", "-shared", "-fopenmp", "-o", str(tmp)] + objs)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
