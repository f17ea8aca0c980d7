"""Learned precision router for batches of general systems (n <= 512).

Pipeline (every numeric step runs in libgb300solve kernels):
  * ``MediumBatch``    packs matrices back to back (gbs_mbatch_*)
  * labels             log10(1 / rcond) from the method itself: FP64
                       PartialPivLU + Hager/Higham rcond (gbs_mbatch_lu_rcond)
  * features           size, diagonal / row-norm statistics and four
                       power-iteration estimates (gbs_mbatch_features)
  * ``Router``         3-layer width-64 MLP trained on the GPU by its own
                       forward / backward / Adam kernels (gbs_mlp_*), routing
                       each system to FP32 + FP64 refinement or to FP64
  * ``solve_*``        routed solve, always-FP64, and try-FP32-then-FP64
                       fallback; the FP64 tier decides every result the FP32
                       tier cannot bring to the backward-error bound
"""
from __future__ import annotations

import ctypes as C
import json
import time

import numpy as np

from . import _lib as L

LABEL_SCALE = 10.0     # network target = log10(kappa) / LABEL_SCALE


class MediumBatch:
    def __init__(self, sizes):
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        self.count = len(self.sizes)
        self._h = C.c_void_p()
        L.check(L.lib().gbs_mbatch_create(C.byref(self._h), self.count, self.sizes.ctypes.data_as(C.c_void_p)),
                "mbatch.create")
        self.a_off = np.zeros(max(self.count, 1), dtype=np.int64)
        self.v_off = np.zeros(max(self.count, 1), dtype=np.int64)
        L.lib().gbs_mbatch_offsets(self._h, self.a_off.ctypes.data_as(C.c_void_p),
                                   self.v_off.ctypes.data_as(C.c_void_p))
        self.a_elems = int(L.lib().gbs_mbatch_matrix_elements(self._h))
        self.v_elems = int(L.lib().gbs_mbatch_vector_elements(self._h))

    def __del__(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().gbs_mbatch_destroy(self._h)
            self._h = C.c_void_p()

    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr()) if t is not None else None

    @staticmethod
    def _sel(items):
        """(device pointer, count) of an int32 CUDA tensor of item indices, or all items."""
        if items is None:
            return None, 0
        assert items.dtype.is_floating_point is False and items.element_size() == 4 and items.is_cuda
        return C.c_void_p(items.data_ptr()), int(items.numel())

    def lu_rcond(self, d_a, d_piv, d_rhs, d_rcond, d_info, items=None, stream=0):
        sp, sn = self._sel(items)
        if items is not None and sn == 0:
            return
        L.check(L.lib().gbs_mbatch_lu_rcond(self._h, sp, sn, self._p(d_a), self._p(d_piv), self._p(d_rhs),
                                            self._p(d_rcond), self._p(d_info), C.c_void_p(stream)), "mbatch.lu_rcond")

    def ir(self, d_a, d_work, d_piv, d_rhs, d_x, d_status, tol=1e-13, max_iter=10, items=None, stream=0):
        sp, sn = self._sel(items)
        if items is not None and sn == 0:
            return
        L.check(L.lib().gbs_mbatch_ir(self._h, sp, sn, self._p(d_a), self._p(d_work), self._p(d_piv), self._p(d_rhs),
                                      self._p(d_x), tol, max_iter, self._p(d_status), C.c_void_p(stream)),
                "mbatch.ir")

    def features(self, d_a, d_feat, items=None, stream=0):
        sp, sn = self._sel(items)
        if items is not None and sn == 0:
            return
        L.check(L.lib().gbs_mbatch_features(self._h, sp, sn, self._p(d_a), self._p(d_feat), C.c_void_p(stream)),
                "mbatch.features")

    def matrix(self, d_a, i):
        n = int(self.sizes[i])
        return d_a[self.a_off[i]:self.a_off[i] + n * n].reshape(n, n).t()   # column-major view

    def vector(self, d_v, i):
        n = int(self.sizes[i])
        return d_v[self.v_off[i]:self.v_off[i] + n]


def feature_count() -> int:
    return int(L.lib().gbs_router_feature_count())


def haar(k, n, generator):
    """k Haar-random n x n orthogonal matrices: the Q factor (diag(R) > 0) of
    seeded Gaussian matrices, computed as Cholesky-QR applied twice (G = Q R
    with R = chol(G^T G), once more on Q for orthogonality to rounding level);
    batched Cholesky and triangular solves instead of one QR per matrix."""
    import torch
    q = torch.randn(k, n, n, dtype=torch.float64, device="cuda", generator=generator)
    for _ in range(2):
        r = torch.linalg.cholesky(q.transpose(-1, -2) @ q, upper=True)
        q = torch.linalg.solve_triangular(r, q, upper=True, left=False)
    return q


def generate(count, seed, nmin=32, nmax=512, logk=(1.0, 12.0)):
    """A = U diag(s) V^T with Haar-random orthogonal U, V and s log-spaced
    from 1 to 1/kappa, log10(kappa) uniform in logk; b iid N(0, 1).
    Returns (batch, packed A, packed b, log10 kappa)."""
    import torch
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, count).astype(np.int32)
    logkappa = rng.uniform(logk[0], logk[1], count)
    mb = MediumBatch(sizes)
    g = torch.Generator(device="cuda").manual_seed(int(seed))
    A = torch.empty(mb.a_elems, dtype=torch.float64, device="cuda")
    B = torch.randn(mb.v_elems, dtype=torch.float64, device="cuda", generator=g)
    a_off = torch.as_tensor(mb.a_off[:count], device="cuda")
    for n in np.unique(sizes):
        n = int(n)
        idx = np.nonzero(sizes == n)[0]
        for c0 in range(0, len(idx), 256):
            sel = idx[c0:c0 + 256]
            u = haar(len(sel), n, g)
            v = haar(len(sel), n, g)
            lk = torch.as_tensor(logkappa[sel], dtype=torch.float64, device="cuda")
            t = torch.linspace(0, 1, n, dtype=torch.float64, device="cuda")
            s = torch.pow(10.0, -lk[:, None] * t[None, :])
            mats = (u * s[:, None, :]) @ v.transpose(-1, -2)
            flat = mats.transpose(-1, -2).reshape(len(sel), -1)      # column-major per matrix
            offs = a_off[torch.as_tensor(sel, device="cuda")]
            ar = torch.arange(n * n, device="cuda")
            A[(offs[:, None] + ar[None, :]).reshape(-1)] = flat.reshape(-1)
    torch.cuda.synchronize()
    return mb, A, B, logkappa


def labels(mb, A):
    """log10(1 / rcond) from the FP64 LU + rcond of each item (on a copy)."""
    import torch
    a = A.clone()
    piv = torch.empty(mb.v_elems, dtype=torch.int32, device="cuda")
    rc = torch.empty(mb.count, dtype=torch.float64, device="cuda")
    info = torch.empty(mb.count, dtype=torch.int32, device="cuda")
    mb.lu_rcond(a, piv, None, rc, info)
    torch.cuda.synchronize()
    del a
    return torch.log10(1.0 / rc.clamp_min(1e-300)).float()


def features(mb, A):
    import torch
    f = torch.empty(mb.count, feature_count(), dtype=torch.float32, device="cuda")
    mb.features(A, f)
    return f


def route_and_solve(router, mb, A, B):
    """The routed solve: features, network, tier per item (on the GPU), then
    FP32 + refinement for the items routed low and FP64 for the rest and for
    every low item that did not reach the bound."""
    import torch
    tier = router.route(router.predict(features(mb, A)))
    lo = torch.nonzero(tier == 1).flatten().to(torch.int32)
    return solve_with_fallback(mb, A, B, lo)


class Router:
    def __init__(self, seed=0, threshold=6.0):
        self._h = C.c_void_p()
        L.check(L.lib().gbs_mlp_create(C.byref(self._h), feature_count(), 64, seed), "mlp.create")
        self.threshold = threshold      # route to FP32 + refinement when predicted log10 kappa <= threshold

    def __del__(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().gbs_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def params(self):
        p = np.zeros(L.lib().gbs_mlp_param_count(self._h), dtype=np.float32)
        L.check(L.lib().gbs_mlp_get_params(self._h, p.ctypes.data_as(C.c_void_p)), "mlp.get")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        L.check(L.lib().gbs_mlp_set_params(self._h, p.ctypes.data_as(C.c_void_p)), "mlp.set")

    def gradients(self, X, T):
        g = np.zeros(L.lib().gbs_mlp_param_count(self._h), dtype=np.float32)
        loss = C.c_double()
        L.check(L.lib().gbs_mlp_gradients(self._h, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()), X.shape[0],
                                          g.ctypes.data_as(C.c_void_p), C.byref(loss)), "mlp.gradients")
        return g, loss.value

    def fit(self, X, logk, epochs=20, batch=1024, lr=2e-3, seed=1):
        T = (logk / LABEL_SCALE).float().contiguous()
        loss = C.c_double()
        L.check(L.lib().gbs_mlp_fit(self._h, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()), X.shape[0], epochs,
                                    batch, lr, seed, C.byref(loss)), "mlp.fit")
        return loss.value

    def predict(self, X):
        import torch
        y = torch.empty(X.shape[0], dtype=torch.float32, device="cuda")
        L.check(L.lib().gbs_mlp_predict(self._h, C.c_void_p(X.data_ptr()), X.shape[0], C.c_void_p(y.data_ptr()),
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream)), "mlp.predict")
        return y * LABEL_SCALE

    def route(self, pred_logk):
        import torch
        tier = torch.empty(pred_logk.shape[0], dtype=torch.int32, device="cuda")
        L.check(L.lib().gbs_router_route(C.c_void_p(pred_logk.data_ptr()), pred_logk.shape[0], self.threshold,
                                         C.c_void_p(tier.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream)),
                "router.route")
        return tier

    def save(self, path):
        with open(path, "w") as f:
            json.dump({"in_dim": feature_count(), "width": 64, "threshold": self.threshold,
                       "label_scale": LABEL_SCALE, "params": self.params().tolist()}, f)

    def load(self, path):
        with open(path) as f:
            d = json.load(f)
        self.threshold = d["threshold"]
        self.set_params(np.asarray(d["params"], dtype=np.float32))


# ----------------------------------------------------------------- solving strategies
def _items(idx):
    import torch
    if hasattr(idx, "is_cuda"):
        return idx.to(torch.int32).contiguous()
    return torch.as_tensor(np.asarray(idx, dtype=np.int32), device="cuda")


def solve_fp64(mb, A, B, items=None, X=None):
    """FP64 LU + solve of the items (all by default) on a copy of A: returns X
    (packed; B's values for the items not solved unless X is given)."""
    import torch
    a = A.clone()
    x = B.clone() if X is None else X
    piv = torch.empty(mb.v_elems, dtype=torch.int32, device="cuda")
    info = torch.empty(mb.count, dtype=torch.int32, device="cuda")
    mb.lu_rcond(a, piv, x, None, info, items=None if items is None else _items(items))
    return x


def solve_fp32_ir(mb, A, B, tol=1e-13, max_iter=10, items=None, X=None):
    """FP32 LU + FP64 refinement; returns (X, status) with status -1 for the
    items that did not reach tol (their X entries are left as they were) and
    -2 for items not attempted."""
    import torch
    work = torch.empty(mb.a_elems, dtype=torch.float32, device="cuda")
    piv = torch.empty(mb.v_elems, dtype=torch.int32, device="cuda")
    x = torch.zeros(mb.v_elems, dtype=torch.float64, device="cuda") if X is None else X
    st = torch.full((mb.count,), -2, dtype=torch.int32, device="cuda")
    mb.ir(A, work, piv, B, x, st, tol, max_iter, items=None if items is None else _items(items))
    return x, st


def solve_with_fallback(mb, A, B, first_fp32_idx):
    """FP32 + refinement on first_fp32_idx (host indices or an int CUDA
    tensor), FP64 on the rest and on every item the FP32 tier did not bring to
    the bound.  Returns (X, stats)."""
    import torch
    X = B.clone()
    lo = _items(first_fp32_idx)
    _, st = solve_fp32_ir(mb, A, B, items=lo, X=X)
    redo = torch.nonzero(st < 0).flatten().to(torch.int32)
    solve_fp64(mb, A, B, items=redo, X=X)
    failed = int((st == -1).sum().item())
    return X, {"fp32_attempts": int(lo.numel()), "fp32_failed": failed, "fp64_solves": int(redo.numel())}


def backward_errors(mb, A, X, B):
    """Per-item normwise backward error (FP64, on the GPU)."""
    errs = np.zeros(mb.count)
    for i in range(mb.count):
        a = mb.matrix(A, i)
        x = mb.vector(X, i)
        b = mb.vector(B, i)
        r = b - a @ x
        den = a.abs().sum(dim=1).max() * x.abs().max() + b.abs().max()
        errs[i] = float((r.abs().max() / den).item())
    return errs


def timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0
