"""Builds libgb300solve.so in-tree (eigen_gb300/_build/) for sm_103a only.

Every .cu file under csrc/ is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into
one shared library exposing the C ABI of include/gb300solve.h.  Rebuilds only
what changed (object newer than its source and the shared headers).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libgb300solve.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-Wno-unused-function", "-I", str(INCLUDE), "-I", str(CSRC)]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _compile(src: Path, extra: list[str]) -> Path:
    obj = OUT_DIR / (src.stem + ".o")
    deps = [src] + _headers()
    if obj.exists() and all(d.stat().st_mtime <= obj.stat().st_mtime for d in deps):
        return obj
    tmp = obj.with_suffix(f".o.tmp{os.getpid()}")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", str(src), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{' '.join(cmd)}\n{r.stdout}{r.stderr}")
    os.replace(tmp, obj)
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


def ptxas_report(src: str) -> str:
    """Registers / spills / shared memory per kernel of one source file."""
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-Xptxas", "-v", "-c", str(CSRC / src), "-o", os.devnull]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.stdout + r.stderr


if __name__ == "__main__":
    if "--ptxas" in sys.argv:
        print(ptxas_report(sys.argv[sys.argv.index("--ptxas") + 1]))
    else:
        build(verbose=True)
