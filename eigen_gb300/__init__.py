"""GB300-native (sm_103a) dense factor-and-solve: Eigen's LLT / PartialPivLU
path on one GPU, behind the C ABI of include/gb300solve.h."""
from . import _lib
from .dense import LDLT, LLT, PartialPivLU, getrf, getrs, llt_blocked, partial_lu_blocked, potrf, potrs
from .mixed import TIERS, solve_mixed, solve_spd_mixed

__all__ = ["LLT", "LDLT", "PartialPivLU", "solve_mixed", "solve_spd_mixed", "TIERS", "getrf", "getrs", "potrf", "potrs", "llt_blocked", "partial_lu_blocked", "lib"]


def lib():
    return _lib.lib()
