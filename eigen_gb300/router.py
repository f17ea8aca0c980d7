"""Learned precision router for batches of general systems (n <= 512).

Pipeline (every numeric step runs in libgb300solve kernels):
  * ``MediumBatch``    packs matrices back to back (gbs_mbatch_*)
  * labels             log10(1 / rcond) from the method itself: FP64
                       PartialPivLU + Hager/Higham rcond (gbs_mbatch_lu_rcond)
  * features           size, diagonal / row-norm statistics and four
                       power-iteration estimates (gbs_mbatch_features)
  * ``Router``         3-layer width-64 MLP trained on the GPU by its own
                       forward / backward / Adam kernels (gbs_mlp_*), routing
                       each system to FP32 LU + FP64 refinement, FP32 LU +
                       GMRES-IR, or FP64 LU
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

    def ir(self, d_a, d_work, d_piv, d_rhs, d_x, d_status, tol=1e-13, max_iter=10, items=None, factored=False,
           stream=0):
        sp, sn = self._sel(items)
        if items is not None and sn == 0:
            return
        L.check(L.lib().gbs_mbatch_ir(self._h, sp, sn, self._p(d_a), self._p(d_work), self._p(d_piv), self._p(d_rhs),
                                      self._p(d_x), tol, max_iter, int(factored), self._p(d_status),
                                      C.c_void_p(stream)), "mbatch.ir")

    def gmres_ir(self, d_a, d_work, d_piv, d_rhs, d_x, d_status, tol=1e-13, max_outer=6, restart=16, d_inner=None,
                 items=None, factored=False, stream=0):
        sp, sn = self._sel(items)
        if items is not None and sn == 0:
            return
        L.check(L.lib().gbs_mbatch_gmres_ir(self._h, sp, sn, self._p(d_a), self._p(d_work), self._p(d_piv),
                                            self._p(d_rhs), self._p(d_x), tol, max_outer, restart, int(factored),
                                            self._p(d_status), self._p(d_inner), C.c_void_p(stream)),
                "mbatch.gmres_ir")

    def largest_first(self, idx):
        """idx (int32 CUDA tensor) reordered by decreasing n (shorter launch tail)."""
        import torch
        if getattr(self, "_sizes_dev", None) is None:
            self._sizes_dev = torch.as_tensor(self.sizes, device="cuda")
        return idx[torch.argsort(self._sizes_dev[idx.long()], descending=True, stable=True)].contiguous()

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


class HaarPool:
    """k Haar matrices per size, drawn once; ``draw`` composes one of them with
    a random signed permutation (Q P is Haar-distributed when Q is), so a large
    training set costs one n^3 product per system instead of two QRs."""

    def __init__(self, k, generator):
        self.k = k
        self.g = generator
        self.pool = {}

    def draw(self, count, n):
        import torch
        if n not in self.pool:
            self.pool[n] = haar(self.k, n, self.g)
        q = self.pool[n][torch.randint(0, self.k, (count,), device="cuda", generator=self.g)]
        perm = torch.argsort(torch.rand(count, n, device="cuda", generator=self.g), dim=1)
        sign = torch.where(torch.rand(count, n, device="cuda", generator=self.g) < 0.5, -1.0, 1.0).to(q.dtype)
        return torch.gather(q, 2, perm[:, None, :].expand(count, n, n)) * sign[:, None, :]


def generate(count, seed, nmin=32, nmax=512, logk=(1.0, 12.0), pool=None):
    """A = U diag(s) V^T with Haar-random orthogonal U, V and s log-spaced
    from 1 to 1/kappa, log10(kappa) uniform in logk; b iid N(0, 1).  With a
    HaarPool, U and V come from it (training sets); otherwise each is a fresh
    Haar matrix.  Returns (batch, packed A, packed b, log10 kappa)."""
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
            u = pool.draw(len(sel), n) if pool else haar(len(sel), n, g)
            v = pool.draw(len(sel), n) if pool else haar(len(sel), n, g)
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
    """The routed solve: features, network and tier per item (on the GPU),
    then each tier on its items and FP64 for every item a refinement tier did
    not bring to the bound."""
    tier = router.route(router.predict(features(mb, A)))
    return solve_tiers(mb, A, B, tier)


class Router:
    def __init__(self, seed=0, t_ir=7.3, t_gmres=8.5):
        self._h = C.c_void_p()
        L.check(L.lib().gbs_mlp_create(C.byref(self._h), feature_count(), 64, seed), "mlp.create")
        self.t_ir = t_ir          # FP32 + refinement when predicted log10 kappa <= t_ir
        self.t_gmres = t_gmres    # FP32 + GMRES-IR when <= t_gmres, FP64 above

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
        L.check(L.lib().gbs_router_route(C.c_void_p(pred_logk.data_ptr()), pred_logk.shape[0], self.t_ir, self.t_gmres,
                                         C.c_void_p(tier.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream)),
                "router.route")
        return tier

    def save(self, path):
        with open(path, "w") as f:
            json.dump({"in_dim": feature_count(), "width": 64, "t_ir": self.t_ir, "t_gmres": self.t_gmres,
                       "label_scale": LABEL_SCALE, "params": self.params().tolist()}, f)

    @classmethod
    def pretrained(cls):
        """The network shipped with the package: trained on 1,000,000 systems
        of the n 32..512, log10 kappa 1..12 distribution with rcond labels
        from gbs_mbatch_lu_rcond (bench.py --config router --save-router)."""
        import os
        r = cls()
        r.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "router_weights.json"))
        return r

    def load(self, path):
        with open(path) as f:
            d = json.load(f)
        self.t_ir, self.t_gmres = d["t_ir"], d["t_gmres"]
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


class Fp32Work:
    """FP32 factor storage shared by the refinement tiers of one batch."""

    def __init__(self, mb):
        import torch
        self.work = torch.empty(mb.a_elems, dtype=torch.float32, device="cuda")
        self.piv = torch.empty(mb.v_elems, dtype=torch.int32, device="cuda")
        self.status = torch.full((mb.count,), NOT_ATTEMPTED, dtype=torch.int32, device="cuda")
        self.inner = torch.zeros(mb.count, dtype=torch.int32, device="cuda")


NOT_ATTEMPTED = -3      # status of items no refinement tier was asked to solve


def solve_fp32_ir(mb, A, B, tol=1e-13, max_iter=10, items=None, X=None, ws=None):
    """FP32 LU + FP64 refinement; returns (X, status): status >= 0 converged,
    -1 not converged, -2 FP32 zero pivot (X entries left as they were),
    NOT_ATTEMPTED for items not in `items`."""
    import torch
    ws = ws or Fp32Work(mb)
    x = torch.zeros(mb.v_elems, dtype=torch.float64, device="cuda") if X is None else X
    mb.ir(A, ws.work, ws.piv, B, x, ws.status, tol, max_iter, items=None if items is None else _items(items))
    return x, ws.status


def solve_fp32_gmres(mb, A, B, tol=1e-13, max_outer=4, restart=16, items=None, X=None, ws=None, factored=False):
    """FP32 LU preconditioning FP64 GMRES-IR; returns (X, status, inner
    iterations).  factored=True continues from ws's FP32 factors (the items
    a solve_fp32_ir call left at -1)."""
    import torch
    ws = ws or Fp32Work(mb)
    x = torch.zeros(mb.v_elems, dtype=torch.float64, device="cuda") if X is None else X
    mb.gmres_ir(A, ws.work, ws.piv, B, x, ws.status, tol, max_outer, restart, ws.inner,
                items=None if items is None else _items(items), factored=factored)
    return x, ws.status, ws.inner


def _fp64_rest(mb, A, B, X, status):
    """FP64 LU + solve of every item whose status is negative."""
    import torch
    redo = torch.nonzero(status < 0).flatten().to(torch.int32)
    solve_fp64(mb, A, B, items=mb.largest_first(redo), X=X)
    return int(redo.numel())


def solve_with_fallback(mb, A, B, first_fp32_idx):
    """FP32 + refinement on first_fp32_idx (host indices or an int CUDA
    tensor), FP64 on the rest and on every item the FP32 tier did not bring to
    the bound.  Returns (X, stats)."""
    X = B.clone()
    ws = Fp32Work(mb)
    lo = mb.largest_first(_items(first_fp32_idx))
    solve_fp32_ir(mb, A, B, items=lo, X=X, ws=ws)
    failed = int(((ws.status == -1) | (ws.status == -2)).sum().item())
    fp64 = _fp64_rest(mb, A, B, X, ws.status)
    return X, {"fp32_attempts": int(lo.numel()), "fp32_failed": failed, "fp64_solves": fp64}


def solve_cascade(mb, A, B):
    """Try-lowest-then-fallback without a router: every item FP32 + IR, the
    items it leaves unconverged FP32 GMRES-IR on the same factors, the rest
    FP64.  Returns (X, stats)."""
    import torch
    X = B.clone()
    ws = Fp32Work(mb)
    solve_fp32_ir(mb, A, B, X=X, ws=ws)
    ir_ok = int((ws.status >= 0).sum().item())
    retry = mb.largest_first(torch.nonzero(ws.status == -1).flatten().to(torch.int32))
    solve_fp32_gmres(mb, A, B, items=retry, X=X, ws=ws, factored=True)
    gm_ok = int((ws.status >= 0).sum().item()) - ir_ok
    fp64 = _fp64_rest(mb, A, B, X, ws.status)
    return X, {"ir_converged": ir_ok, "gmres_attempts": int(retry.numel()), "gmres_converged": gm_ok,
               "fp64_solves": fp64}


def solve_tiers(mb, A, B, tier):
    """Per-item tiers (int CUDA tensor: 1 FP32 + IR, 2 FP32 + GMRES-IR, 0
    FP64); every item a refinement tier leaves unconverged is solved in FP64.
    Returns (X, stats)."""
    import torch
    X = B.clone()
    ws = Fp32Work(mb)
    t1 = mb.largest_first(torch.nonzero(tier == 1).flatten().to(torch.int32))
    t2 = mb.largest_first(torch.nonzero(tier == 2).flatten().to(torch.int32))
    solve_fp32_ir(mb, A, B, items=t1, X=X, ws=ws)
    solve_fp32_gmres(mb, A, B, items=t2, X=X, ws=ws)
    st = ws.status
    stats = {"ir_routed": int(t1.numel()), "gmres_routed": int(t2.numel()),
             "ir_failed": int(((st < 0) & (st != NOT_ATTEMPTED) & (tier == 1)).sum().item()),
             "gmres_failed": int(((st < 0) & (st != NOT_ATTEMPTED) & (tier == 2)).sum().item())}
    stats["fp64_solves"] = _fp64_rest(mb, A, B, X, st)
    return X, stats


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
