import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: large sizes (seconds of CPU oracle work)")


_PARITY: list[tuple[str, str, float, float]] = []
_NOTES: list[tuple[str, str]] = []


def record_note(what: str, text: str) -> None:
    """A measurement a test made (times, counts), printed in the terminal summary."""
    _NOTES.append((what, text))


def record_parity(case: str, what: str, value: float, bound: float) -> None:
    """Keeps an achieved error next to the bound it was asserted against; the
    session's worst ratio per quantity is printed in the terminal summary."""
    _PARITY.append((case, what, float(value), float(bound)))


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    if _NOTES:
        terminalreporter.section("measurements")
        for what, text in _NOTES:
            terminalreporter.write_line(f"{what}: {text}")
    if not _PARITY:
        return
    worst: dict[str, tuple[str, float, float]] = {}
    for case, what, v, b in _PARITY:
        r = v / b if b > 0 else 0.0
        if what not in worst or r > worst[what][1] / max(worst[what][2], 1e-300):
            worst[what] = (case, v, b)
    terminalreporter.section("achieved parity (worst case per quantity)")
    for what in sorted(worst):
        case, v, b = worst[what]
        terminalreporter.write_line(f"{what:44s} {v:9.2e}  bound {b:8.1e}  ({case})")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


class Golden:
    """The reference's outputs on seeded inputs (tests/golden/make_golden.py)."""

    def __init__(self):
        with open(GOLDEN / "eigen_dense.json") as f:
            self.meta = json.load(f)
        self.arrays = np.load(GOLDEN / "eigen_dense.npz")

    def cases(self, kind):
        return [c for c in self.meta["cases"] if c["kind"] == kind]

    def arr(self, case, key):
        k = case["name"] + key
        return self.arrays[k] if k in self.arrays.files else None

    @staticmethod
    def input(case):
        from tests.golden.make_golden import gen
        return gen(case)

    @staticmethod
    def rhs(case, nrhs):
        from tests.golden.make_golden import rhs
        return rhs(case, nrhs)


@pytest.fixture(scope="session")
def golden():
    return Golden()


def case_id(c):
    s = f"{c['kind']}-{c['gen']}-{c['m']}x{c['n']}"
    if c.get("dtype") == "f32":
        s += "-f32"
    if c.get("upper"):
        s += "-upper"
    return s
