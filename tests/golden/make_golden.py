"""Generate the golden fixtures for the dense factor-and-solve path by running
the reference itself (Eigen, built from the reference tree into
oracle/_ref/libeigen_ref.so) on seeded, byte-stable inputs.

    python tests/golden/make_golden.py

Writes tests/golden/eigen_dense.json (case list + scalars) and
tests/golden/eigen_dense.npz (arrays).  Inputs are not stored: every case
records the generator (oracle.gauss / oracle.uniform / oracle.spd with its
seed), whose bytes are identical on every host.  Small cases store the full
factors; large cases store pivots, solutions, a fixed sample of factor entries
and a sketch F R of the whole factor (R a seeded n x 4 or n x 8 Gaussian
matrix).  Every case also records the noise floor of the reference's
algorithm: the distance between the reference's factor and solution and those
of the C restatement (same blocking, another rounding order).

What each case pins (reference API used):
  lu    PartialPivLU<MatrixX?>(A): matrixLU(), permutationP().indices(),
        solve(B), transpose().solve(B), rcond(), determinant();
        partial_lu_impl::blocked_lu transpositions + count + first zero pivot;
        ?getrf_ ipiv (1-based) and info from the reference's LAPACK shim.
  llt   LLT<MatrixX?, Lower|Upper>(A): matrixLLT(), info(), solve(B), rcond();
        llt_inplace::blocked failing column; ?potrf_ info.
  ldlt  LDLT<MatrixX?, Lower|Upper>(A): matrixLDLT(), transpositionsP(), info(),
        isPositive(), isNegative(), solve(B), rcond().
  blas  the reference's BLAS level-3 shim (blas/level3_impl.h): ?gemm_, ?trsm_,
        ?syrk_ on seeded operands, every op / side / uplo / diag combination.
  rank_update  LLT<MatrixXd, Lower|Upper>(A).rankUpdate(v, sigma): factor, info.
"""
from __future__ import annotations

import ctypes as C
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
FULL_MAX = 129          # store whole factors up to this size
SAMPLE = 2048           # otherwise this many factor entries at fixed positions


def sample_idx(n: int) -> np.ndarray:
    rng = np.random.default_rng(1000 + n)  # positions only; stored in the fixture
    return np.sort(rng.choice(n * n, size=min(SAMPLE, n * n), replace=False)).astype(np.int64)


# LDLT cases whose arithmetic is exact, so info and the sign do not depend on
# rounding (LDLT.h:345-369)
NAN = float("nan")
LDLT_EXACT = {
    "zero": [[0.0] * 5 for _ in range(5)],                                   # ZeroSign, Success
    "zero_diag": [[0, 1, 0], [1, 0, 2], [0, 2, 0]],                          # whole diagonal zero: NumericalIssue
    "diag_mixed": [[3, 0, 0, 0, 0], [0, 0, 0, 0, 0], [0, 0, -2, 0, 0],
                   [0, 0, 0, 0, 0], [0, 0, 0, 0, 5]],                        # Indefinite, zero pivots last
    "semidef": [[4, 2, 0], [2, 1, 0], [0, 0, 0]],                            # PositiveSemiDef, Success
    "zero_then_nonzero": [[1, 1, 0], [1, 1, 0], [0, 0, 0.5]],                # NumericalIssue
    "nan_first": [[NAN, 1, 0], [1, 2, 0], [0, 0, 3]],                        # NaN first: the zero-diagonal branch
    "ties": [[2, 1, 0, 0, 1], [1, -2, 1, 0, 0], [0, 1, 2, 1, 0],
             [0, 0, 1, -2, 1], [1, 0, 0, 1, 2]],                             # equal |diagonal|: first one wins
    "negdef": [[-4, 1, 0], [1, -3, 1], [0, 1, -5]],                          # NegativeSemiDef
}


def sketch_cols(n: int) -> int:
    return 4 if n > 4096 else 8


def sketch_matrix(n: int) -> np.ndarray:
    """R (n x k, seeded generator) of the factor sketch F R.  Every entry of
    the factor enters the sketch, so ||(F - F_ref) R|| / ||F_ref R|| tracks the
    relative Frobenius difference of the whole factor (a Gaussian random
    projection), where the sampled entries see only 2048 of them."""
    return O.gauss(77000 + n, n, sketch_cols(n))


def rel(a: np.ndarray, b: np.ndarray) -> float:
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def gen(spec: dict) -> np.ndarray:
    k = spec["gen"]
    if k == "gauss":
        a = O.gauss(spec["seed"], spec["m"], spec["n"])
    elif k == "uniform":
        a = O.uniform(spec["seed"], spec["m"], spec["n"])
    elif k == "spd":
        a = O.spd(spec["seed"], spec["n"], spec.get("scale"), spec.get("shift", 1.0))
    elif k == "int":   # small integers in [-2, 2]: exact arithmetic, many exact pivot ties
        a = np.asfortranarray(np.rint(O.uniform(spec["seed"], spec["m"], spec["n"]) * 2.49))
    elif k == "neg_spd":
        a = -O.spd(spec["seed"], spec["n"])
    elif k == "late_fail":  # SPD except one diagonal entry made too small: fails at column `col`
        a = O.spd(spec["seed"], spec["n"])
        a[spec["col"], spec["col"]] = -1.0
    elif k == "zero_col":  # exactly singular: column `col` is zero
        a = O.gauss(spec["seed"], spec["m"], spec["n"])
        a[:, spec["col"]] = 0.0
    elif k == "ones":
        a = np.ones((spec["m"], spec["n"]), order="F")
    elif k in ("tie_rows", "near_tie_rows"):
        # `pairs` twin rows r, r+1 with row r+1 = -(row r) over the columns
        # [0, c0 + pairs): both twins see the same operations, so their
        # magnitudes stay equal through the first c0 elimination steps (many
        # blocked updates).  The twins are small (x 1/8) before column c0 and
        # dominant (x 64) in [c0, c0 + pairs), so at those steps the column
        # maximum is a tie between twins, broken by the first-maximum rule.
        # near_tie_rows scales the copy by (1 + 1e-10 g): the decision then
        # rests on a margin of ~1e-10, far above the rounding noise, and must
        # not depend on the operation order.  Beyond c0 + pairs the twins are
        # independent, so the matrix is nonsingular.
        a = O.gauss(spec["seed"], spec["m"], spec["n"])
        p, c0 = spec["pairs"], spec["c0"]
        rows = np.arange(p) * (spec["m"] // p)
        a[rows, :c0] *= 0.125
        a[rows, c0:c0 + p] *= 64.0
        scale = np.ones(p)
        if k == "near_tie_rows":
            scale = 1.0 + 1e-10 * O.gauss(spec["seed"] + 1, p, 1)[:, 0]
        a[rows + 1, :c0 + p] = -a[rows, :c0 + p] * scale[:, None]
    elif k == "sym_gauss":  # symmetric indefinite: (G + G^T) / 2
        g = O.gauss(spec["seed"], spec["n"], spec["n"])
        a = np.asfortranarray((g + g.T) / 2)
    elif k == "ldlt_exact":  # small patterns in exact arithmetic (zero / NaN pivots, diagonal ties)
        a = np.asfortranarray(np.array(LDLT_EXACT[spec["pattern"]], dtype=np.float64))
    else:
        raise ValueError(k)
    if spec.get("dtype", "f64") == "f32":
        a = np.asfortranarray(a.astype(np.float32))
    return a


def rhs(spec: dict, nrhs: int) -> np.ndarray:
    b = O.gauss(spec["seed"] + 7919, spec["n"], nrhs)
    return np.asfortranarray(b.astype(np.float32)) if spec.get("dtype", "f64") == "f32" else b


def tie_decisions(spec: dict, tr: np.ndarray) -> int:
    """Steps at which the reference's pivot was one twin while the other twin
    was still a candidate (an exact or 1e-10 tie decided by the rule)."""
    p = spec["pairs"]
    rows = np.arange(p) * (spec["m"] // p)
    twin = {int(r): int(r) + 1 for r in rows}
    twin.update({int(r) + 1: int(r) for r in rows})
    order = list(range(spec["m"]))
    ties = 0
    for k, t in enumerate(tr):
        order[k], order[t] = order[t], order[k]
        if order[k] in twin and twin[order[k]] in order[k + 1:]:
            ties += 1
    return ties


def lu_case(spec: dict, arrays: dict, name: str) -> dict:
    a = gen(spec)
    n = spec["n"]
    nrhs = spec.get("nrhs", 3)
    b = rhs(spec, nrhs)
    fact, perm, x, xt, rc, det = O.ref_lu(a, b)
    _, tr, nbt, fz = O.ref_lu_blocked(a)
    # the reference's LAPACK shim (1-based ipiv, info = first zero pivot + 1)
    lib = O.ref()
    pre = "d" if a.dtype == np.float64 else "s"
    ag = np.array(a, order="F", copy=True)
    ipiv = np.zeros(max(n, 1), dtype=np.int32)
    m_ = C.c_int(n); n_ = C.c_int(n); lda = C.c_int(max(n, 1)); info = C.c_int(0)
    getattr(lib, pre + "getrf_")(C.byref(m_), C.byref(n_), ag, C.byref(lda), ipiv, C.byref(info))
    out = dict(spec, kind="lu", rcond=rc, det=det, nb_transpositions=nbt, first_zero_pivot=fz,
               getrf_info=int(info.value), l1_norm=O.l1_norm(a))
    if spec["gen"] in ("tie_rows", "near_tie_rows"):
        out["tie_decisions"] = tie_decisions(spec, tr)
    arrays[name + "perm"] = perm.astype(np.int32)
    arrays[name + "tr"] = tr.astype(np.int32)
    arrays[name + "ipiv"] = ipiv[:n].astype(np.int32)
    arrays[name + "x"] = x
    arrays[name + "xt"] = xt
    if n <= FULL_MAX:
        arrays[name + "lu"] = fact
    else:
        idx = sample_idx(n)
        arrays[name + "lu_idx"] = idx
        arrays[name + "lu_val"] = fact.reshape(-1, order="F")[idx]
        arrays[name + "lu_diag"] = np.diag(fact).copy()
        arrays[name + "lu_sketch"] = fact.astype(np.float64) @ sketch_matrix(n)
    # the noise floor: the C restatement of the same algorithm (same blocking,
    # other rounding order) against the reference, whole factor and solution
    f_o, tr_o, _, _ = O.lu(a)
    out["pivots_oracle_equal"] = bool(np.array_equal(tr_o, tr))
    out["factor_floor"] = rel(f_o, fact)
    if fz < 0:
        out["x_floor"] = rel(O.lu_solve(f_o, tr_o, b), x)
        out["xt_floor"] = rel(O.lu_solve(f_o, tr_o, b, transpose=True), xt)
    return out


def lu_rect_case(spec: dict, arrays: dict, name: str) -> dict:
    """?getrf_ on an m x n (m > n) matrix: factors, 1-based ipiv, info."""
    a = gen(spec)
    m, n = a.shape
    lib = O.ref()
    pre = "d" if a.dtype == np.float64 else "s"
    ag = np.array(a, order="F", copy=True)
    ipiv = np.zeros(max(min(m, n), 1), dtype=np.int32)
    m_ = C.c_int(m); n_ = C.c_int(n); lda = C.c_int(max(m, 1)); info = C.c_int(0)
    getattr(lib, pre + "getrf_")(C.byref(m_), C.byref(n_), ag, C.byref(lda), ipiv, C.byref(info))
    arrays[name + "lu"] = ag
    arrays[name + "ipiv"] = ipiv[: min(m, n)]
    return dict(spec, kind="getrf", getrf_info=int(info.value))


def llt_case(spec: dict, arrays: dict, name: str) -> dict:
    a = gen(spec)
    n = spec["n"]
    upper = spec.get("upper", False)
    nrhs = spec.get("nrhs", 2)
    b = rhs(spec, nrhs)
    fact, info, x, rc = O.ref_llt(a, b, upper=upper)
    lib = O.ref()
    pre = "d" if a.dtype == np.float64 else "s"
    ag = np.array(a, order="F", copy=True)
    n_ = C.c_int(n); lda = C.c_int(max(n, 1)); pinfo = C.c_int(0)
    getattr(lib, pre + "potrf_")(b"U" if upper else b"L", C.byref(n_), ag, C.byref(lda), C.byref(pinfo))
    out = dict(spec, kind="llt", info=info, potrf_info=int(pinfo.value),
               rcond=(rc if info == 0 else None), l1_norm=O.sym_l1_norm(a, upper))
    tri = np.triu(fact) if upper else np.tril(fact)
    if info == 0:
        arrays[name + "x"] = x
    if n <= FULL_MAX:
        arrays[name + "fact"] = tri
    else:
        idx = sample_idx(n)
        arrays[name + "fact_idx"] = idx
        arrays[name + "fact_val"] = tri.reshape(-1, order="F")[idx]
        arrays[name + "fact_diag"] = np.diag(fact).copy()
        arrays[name + "fact_sketch"] = tri.astype(np.float64) @ sketch_matrix(n)
    f_o, info_o = O.llt(a, upper=upper)
    tri_o = np.triu(f_o) if upper else np.tril(f_o)
    out["factor_floor"] = rel(tri_o, tri)
    if info == 0:
        out["x_floor"] = rel(O.llt_solve(f_o, b, upper=upper), x)
    return out


def ldlt_case(spec: dict, arrays: dict, name: str) -> dict:
    """LDLT<MatrixX?, Lower|Upper>(A): matrixLDLT(), transpositionsP(), info(),
    isPositive(), isNegative(), solve(B), rcond(); and the C restatement's
    distance to them (the noise floor)."""
    a = gen(spec)
    n = spec["n"]
    upper = spec.get("upper", False)
    nrhs = spec.get("nrhs", 2)
    b = rhs(spec, nrhs)
    fact, tr, info, pos, neg, x, rc = O.ref_ldlt(a, b, upper=upper)
    out = dict(spec, kind="ldlt", info=info, is_positive=pos, is_negative=neg,
               rcond=rc if np.isfinite(rc) else None, l1_norm=O.sym_l1_norm(a, upper))
    tri = np.triu(fact) if upper else np.tril(fact)
    arrays[name + "tr"] = tr.astype(np.int32)
    arrays[name + "x"] = x
    if n <= FULL_MAX:
        arrays[name + "fact"] = fact
    else:
        idx = sample_idx(n)
        arrays[name + "fact_idx"] = idx
        arrays[name + "fact_val"] = tri.reshape(-1, order="F")[idx]
        arrays[name + "fact_diag"] = np.diag(fact).copy()
        arrays[name + "fact_sketch"] = tri.astype(np.float64) @ sketch_matrix(n)
    f_o, tr_o, ok_o, sign_o = O.ldlt(a, upper=upper)
    tri_o = np.triu(f_o) if upper else np.tril(f_o)
    out["transpositions_oracle_equal"] = bool(np.array_equal(tr_o, tr))
    out["sign_oracle"] = O.SIGN_NAMES[sign_o]
    out["factor_floor"] = rel(tri_o, tri) if np.all(np.isfinite(tri)) else None
    xo = O.ldlt_solve(f_o, tr_o, b, upper=upper)
    out["x_floor"] = rel(xo, x) if np.all(np.isfinite(x)) else None
    return out


def blas_inputs(spec: dict):
    """Operands of a BLAS case, rebuilt from seeds.  gemm: A (op(A) m x k), B
    (op(B) k x n), C; trsm: A (a well-conditioned triangle; with diag 'U' its
    diagonal holds NaN, which the routine must not read), B; syrk: A (op(A)
    n x k), C.  C holds NaN when beta = 0, which the routine must not read."""
    s, dt = spec["seed"], (np.float32 if spec.get("dtype") == "f32" else np.float64)
    f = lambda x: np.asfortranarray(x.astype(dt))
    if spec["op"] == "gemm":
        m, n, k = spec["m"], spec["n"], spec["k"]
        a = O.gauss(s, m, k) if spec["opa"] in "Nn" else O.gauss(s, k, m)
        b = O.gauss(s + 1, k, n) if spec["opb"] in "Nn" else O.gauss(s + 1, n, k)
        c = O.gauss(s + 2, m, n)
        if spec["beta"] == 0:
            c[::3, ::2] = np.nan
        return f(a), f(b), f(c)
    if spec["op"] == "trsm":
        m, n = spec["m"], spec["n"]
        na = m if spec["side"] in "Ll" else n
        a = O.gauss(s, na, na) / np.sqrt(na)
        a[np.diag_indices(na)] = 2.0 + np.abs(np.diag(a))
        tri = np.tril(a) if spec["uplo"] in "Ll" else np.triu(a)
        other = O.gauss(s + 3, na, na)            # the unused triangle: garbage the routine must not read
        a = tri + (np.triu(other, 1) if spec["uplo"] in "Ll" else np.tril(other, -1))
        if spec["diag"] in "Uu":
            a[np.diag_indices(na)] = np.nan
        return f(a), f(O.gauss(s + 1, m, n)), None
    n, k = spec["n"], spec["k"]
    a = O.gauss(s, n, k) if spec["opa"] in "Nn" else O.gauss(s, k, n)
    c = O.gauss(s + 2, n, n)
    if spec["beta"] == 0:
        c[::3, ::2] = np.nan
    return f(a), f(c), None


def blas_case(spec: dict, arrays: dict, name: str) -> dict:
    """The reference's BLAS shim (blas/level3_impl.h) on seeded operands; the
    output in full up to 129^2 entries, else as a sketch; the noise floor is
    the distance of a plain numpy restatement of the same formula."""
    x, y, z = blas_inputs(spec)
    op = spec["op"]
    if op == "gemm":
        out = O.ref_gemm(spec["opa"], spec["opb"], spec["alpha"], x, y, spec["beta"], z)
        oa = x if spec["opa"] in "Nn" else x.T
        ob = y if spec["opb"] in "Nn" else y.T
        zz = np.zeros_like(z) if spec["beta"] == 0 else spec["beta"] * z
        other = spec["alpha"] * (oa.astype(np.float64) @ ob.astype(np.float64)) + zz
    elif op == "trsm":
        out = O.ref_trsm(spec["side"], spec["uplo"], spec["opa"], spec["diag"], spec["alpha"], x, y)
        t = np.tril(x) if spec["uplo"] in "Ll" else np.triu(x)
        t = t.astype(np.float64)
        if spec["diag"] in "Uu":
            t[np.diag_indices(t.shape[0])] = 1.0
        t = t if spec["opa"] in "Nn" else t.T
        other = spec["alpha"] * (np.linalg.solve(t, y) if spec["side"] in "Ll" else np.linalg.solve(t.T, y.T).T)
    else:
        out = O.ref_syrk(spec["uplo"], spec["opa"], spec["alpha"], x, spec["beta"], y)
        oa = (x if spec["opa"] in "Nn" else x.T).astype(np.float64)
        zz = np.zeros_like(y) if spec["beta"] == 0 else spec["beta"] * y
        full = spec["alpha"] * (oa @ oa.T) + zz
        keep = np.tril if spec["uplo"] in "Ll" else np.triu
        return_floor = rel(keep(full), keep(out))
    if out.size <= FULL_MAX * FULL_MAX:
        arrays[name + "out"] = out
    else:
        arrays[name + "out_sketch"] = out.astype(np.float64) @ sketch_matrix(out.shape[1])
    return dict(spec, kind="blas", floor=return_floor if op == "syrk" else rel(other, out))


def rank_update_case(spec: dict, arrays: dict, name: str) -> dict:
    """LLT<Matrix, Lower|Upper>(A).rankUpdate(v, sigma) of the reference."""
    a = O.spd(spec["seed"], spec["n"])
    v = O.gauss(spec["seed"] + 1, spec["n"], 1)[:, 0]
    fact, info = O.ref_llt_rank_update(a, v, spec["sigma"], spec.get("upper", False))
    if spec["n"] <= FULL_MAX:
        arrays[name + "fact"] = fact
    else:
        tri = np.triu(fact) if spec.get("upper") else np.tril(fact)
        arrays[name + "fact_sketch"] = tri @ sketch_matrix(spec["n"])
    f0, _ = O.llt(a, upper=spec.get("upper", False))
    fo, ro = O.llt_rank_update(f0, v, spec["sigma"], spec.get("upper", False))
    tri = (np.triu if spec.get("upper") else np.tril)
    return dict(spec, kind="rank_update", info=info, floor=rel(tri(fo), tri(fact)))


def cases():
    lu_sizes = [1, 2, 3, 4, 5, 8, 15, 16, 17, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129, 200, 256, 257, 300,
                512, 1000, 2048]
    for n in lu_sizes:
        yield "lu", dict(gen="gauss", seed=100 + n, m=n, n=n)
    for n in [7, 33, 129, 300]:
        yield "lu", dict(gen="uniform", seed=200 + n, m=n, n=n, dtype="f32")
    for n in [8, 16, 24, 40]:
        yield "lu", dict(gen="int", seed=300 + n, m=n, n=n)
    for n, col in [(5, 2), (40, 0), (100, 57), (300, 299)]:
        yield "lu", dict(gen="zero_col", seed=400 + n, m=n, n=n, col=col)
    yield "lu", dict(gen="ones", seed=0, m=20, n=20)
    for n, pairs, c0 in [(512, 16, 300), (2048, 32, 1500)]:
        yield "lu", dict(gen="tie_rows", seed=1100 + n, m=n, n=n, pairs=pairs, c0=c0)
        yield "lu", dict(gen="near_tie_rows", seed=1200 + n, m=n, n=n, pairs=pairs, c0=c0)
    yield "lu", dict(gen="gauss", seed=8192, m=8192, n=8192, nrhs=2)
    for m, n in [(10, 4), (100, 37), (300, 129), (400, 70)]:
        yield "getrf", dict(gen="gauss", seed=500 + m, m=m, n=n)
    llt_sizes = [1, 2, 3, 5, 8, 16, 17, 31, 32, 33, 64, 65, 100, 128, 129, 200, 257, 512, 1000, 2048]
    for n in llt_sizes:
        yield "llt", dict(gen="spd", seed=600 + n, m=n, n=n)
    for n in [3, 33, 129, 257]:
        yield "llt", dict(gen="spd", seed=700 + n, m=n, n=n, upper=True)
    for n in [9, 65, 200]:
        yield "llt", dict(gen="spd", seed=800 + n, m=n, n=n, dtype="f32")
    for n in [4, 40]:
        yield "llt", dict(gen="neg_spd", seed=900 + n, m=n, n=n)
    for n, col in [(10, 6), (100, 77), (300, 130)]:
        yield "llt", dict(gen="late_fail", seed=950 + n, m=n, n=n, col=col)
    yield "llt", dict(gen="late_fail", seed=990, m=150, n=150, col=20, upper=True)
    for n in [1, 2, 3, 5, 16, 17, 31, 32, 33, 64, 65, 100, 200, 512, 1000, 2048]:
        yield "ldlt", dict(gen="spd", seed=1300 + n, m=n, n=n)
    for n in [3, 33, 129, 257]:
        yield "ldlt", dict(gen="spd", seed=1400 + n, m=n, n=n, upper=True)
    for n in [9, 65, 200]:
        yield "ldlt", dict(gen="spd", seed=1500 + n, m=n, n=n, dtype="f32")
    for n in [5, 17, 64, 200]:
        yield "ldlt", dict(gen="sym_gauss", seed=1600 + n, m=n, n=n)
    yield "ldlt", dict(gen="sym_gauss", seed=1700, m=40, n=40, upper=True)
    for pat in LDLT_EXACT:
        k = len(LDLT_EXACT[pat])
        yield "ldlt", dict(gen="ldlt_exact", pattern=pat, seed=1800, m=k, n=k)
        yield "ldlt", dict(gen="ldlt_exact", pattern=pat, seed=1801, m=k, n=k, upper=True)
    # BLAS level 3 (the reference's shim): every op combination, special alpha / beta
    sd = 2000
    for opa in "NT":
        for opb in "NT":
            for (m, n, k), (al, be) in [((7, 5, 3), (1.0, 0.0)), ((64, 33, 17), (-1.0, 1.0)),
                                        ((129, 100, 65), (0.3, 0.7)), ((40, 30, 0), (2.0, 3.0))]:
                sd += 10
                yield "blas", dict(gen="blas", op="gemm", opa=opa, opb=opb, m=m, n=n, k=k, alpha=al, beta=be, seed=sd)
    yield "blas", dict(gen="blas", op="gemm", opa="C", opb="N", m=50, n=40, k=30, alpha=0.0, beta=2.0, seed=2300)
    yield "blas", dict(gen="blas", op="gemm", opa="N", opb="T", m=1000, n=700, k=600, alpha=-1.0, beta=1.0, seed=2310)
    yield "blas", dict(gen="blas", op="gemm", opa="T", opb="N", m=300, n=200, k=100, alpha=0.5, beta=0.0,
                       seed=2320, dtype="f32")
    for side in "LR":
        for uplo in "LU":
            for opa in "NT":
                for diag in "NU":
                    sd += 10
                    yield "blas", dict(gen="blas", op="trsm", side=side, uplo=uplo, opa=opa, diag=diag, m=37, n=23,
                                       alpha=1.5, seed=sd)
    yield "blas", dict(gen="blas", op="trsm", side="L", uplo="L", opa="N", diag="N", m=700, n=300, alpha=1.0,
                       seed=2400)
    yield "blas", dict(gen="blas", op="trsm", side="R", uplo="U", opa="T", diag="N", m=200, n=500, alpha=-2.0,
                       seed=2410)
    yield "blas", dict(gen="blas", op="trsm", side="L", uplo="U", opa="N", diag="U", m=90, n=40, alpha=1.0,
                       seed=2420, dtype="f32")
    for uplo in "LU":
        for opa in "NT":
            for al, be in [(-1.0, 0.5), (1.0, 0.0)]:
                sd += 10
                yield "blas", dict(gen="blas", op="syrk", uplo=uplo, opa=opa, n=40, k=25, alpha=al, beta=be, seed=sd)
    yield "blas", dict(gen="blas", op="syrk", uplo="L", opa="N", n=600, k=300, alpha=-1.0, beta=1.0, seed=2500)
    # LLT::rankUpdate: updates and downdates, lower and upper, a failing downdate
    for n in [1, 5, 40, 300, 1000]:
        for upper in (False, True):
            for sigma in (0.7, -0.001, -1e4):
                if n == 1000 and (upper or sigma == -1e4):
                    continue
                yield "rank_update", dict(gen="rank_update", seed=2600 + n, m=n, n=n, sigma=sigma, upper=upper)


def main() -> None:
    arrays: dict[str, np.ndarray] = {}
    meta = []
    t0 = time.time()
    for i, (kind, spec) in enumerate(cases()):
        name = f"c{i}_"
        if kind == "lu":
            rec = lu_case(spec, arrays, name)
        elif kind == "getrf":
            rec = lu_rect_case(spec, arrays, name)
        elif kind == "ldlt":
            rec = ldlt_case(spec, arrays, name)
        elif kind == "blas":
            rec = blas_case(spec, arrays, name)
        elif kind == "rank_update":
            rec = rank_update_case(spec, arrays, name)
        else:
            rec = llt_case(spec, arrays, name)
        rec["name"] = name
        meta.append(rec)
        print(f"{name:6s} {kind:5s} n={spec['n']:5d} {spec['gen']:9s} {time.time() - t0:6.1f}s", flush=True)
    np.savez_compressed(OUT / "eigen_dense.npz", **arrays)
    with open(OUT / "eigen_dense.json", "w") as f:
        json.dump({"generator": "oracle.gauss/uniform/spd (counter-based splitmix64, Irwin-Hall(12))",
                   "reference": "Eigen 3.3.90 (PX4/eigen), g++ -O3 -mavx2 -mfma",
                   "sample_positions": "numpy default_rng(1000+n).choice(n*n, 2048) -- stored as *_idx",
                   "cases": meta}, f, indent=1)
    print("wrote", OUT / "eigen_dense.npz", (OUT / "eigen_dense.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
