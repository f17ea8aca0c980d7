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

    def lu_rcond(self, d_a, d_piv, d_rhs, d_rcond, d_info, stream=0):
        L.check(L.lib().gbs_mbatch_lu_rcond(self._h, self._p(d_a), self._p(d_piv), self._p(d_rhs), self._p(d_rcond),
                                            self._p(d_info), C.c_void_p(stream)), "mbatch.lu_rcond")

    def ir(self, d_a, d_work, d_piv, d_rhs, d_x, d_status, tol=1e-13, max_iter=10, stream=0):
        L.check(L.lib().gbs_mbatch_ir(self._h, self._p(d_a), self._p(d_work), self._p(d_piv), self._p(d_rhs),
                                      self._p(d_x), tol, max_iter, self._p(d_status), C.c_void_p(stream)),
                "mbatch.ir")

    def features(self, d_a, d_feat, stream=0):
        L.check(L.lib().gbs_mbatch_features(self._h, self._p(d_a), self._p(d_feat), C.c_void_p(stream)),
                "mbatch.features")

    def matrix(self, d_a, i):
        n = int(self.sizes[i])
        return d_a[self.a_off[i]:self.a_off[i] + n * n].reshape(n, n).t()   # column-major view

    def vector(self, d_v, i):
        n = int(self.sizes[i])
        return d_v[self.v_off[i]:self.v_off[i] + n]


def feature_count() -> int:
    return int(L.lib().gbs_router_feature_count())


def generate(count, seed, nmin=32, nmax=512, logk=(1.0, 12.0)):
    """A = U diag(s) V^T with Haar-random orthogonal U, V (QR of seeded
    Gaussians, signs fixed by diag(R)) and s log-spaced from 1 to 1/kappa,
    log10(kappa) uniform in logk.  Returns (batch, packed A, packed b, log10 kappa)."""
    import torch
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, count).astype(np.int32)
    logkappa = rng.uniform(logk[0], logk[1], count)
    mb = MediumBatch(sizes)
    g = torch.Generator(device="cuda").manual_seed(int(seed))
    A = torch.empty(mb.a_elems, dtype=torch.float64, device="cuda")
    B = torch.randn(mb.v_elems, dtype=torch.float64, device="cuda", generator=g)
    for n in np.unique(sizes):
        idx = np.nonzero(sizes == n)[0]
        k = len(idx)
        for c0 in range(0, k, 512):
            sel = idx[c0:c0 + 512]
            q1, r1 = torch.linalg.qr(torch.randn(len(sel), n, n, dtype=torch.float64, device="cuda", generator=g))
            q1 = q1 * torch.sign(torch.diagonal(r1, dim1=-2, dim2=-1)).unsqueeze(-2)
            q2, r2 = torch.linalg.qr(torch.randn(len(sel), n, n, dtype=torch.float64, device="cuda", generator=g))
            q2 = q2 * torch.sign(torch.diagonal(r2, dim1=-2, dim2=-1)).unsqueeze(-2)
            lk = torch.as_tensor(logkappa[sel], dtype=torch.float64, device="cuda")
            t = torch.linspace(0, 1, int(n), dtype=torch.float64, device="cuda")
            s = torch.pow(10.0, -lk[:, None] * t[None, :])
            mats = (q1 * s[:, None, :]) @ q2.transpose(-1, -2)
            flat = mats.transpose(-1, -2).reshape(len(sel), -1)      # column-major per matrix
            offs = torch.as_tensor(mb.a_off[sel], device="cuda")
            ar = torch.arange(int(n) * int(n), device="cuda")
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
def _subset(mb, A, B, idx):
    """Gather items idx into a new packed batch (device copies)."""
    import torch
    sizes = mb.sizes[idx]
    sub = MediumBatch(sizes)
    a_src = np.concatenate([np.arange(mb.a_off[i], mb.a_off[i] + int(mb.sizes[i]) ** 2) for i in idx]) if len(idx) \
        else np.zeros(0, dtype=np.int64)
    v_src = np.concatenate([np.arange(mb.v_off[i], mb.v_off[i] + int(mb.sizes[i])) for i in idx]) if len(idx) \
        else np.zeros(0, dtype=np.int64)
    a_idx = torch.as_tensor(a_src, device="cuda")
    v_idx = torch.as_tensor(v_src, device="cuda")
    return sub, A[a_idx].contiguous(), B[v_idx].contiguous(), v_idx


def solve_fp64(mb, A, B):
    """FP64 LU + solve of every item: returns X (packed)."""
    import torch
    a = A.clone()
    x = B.clone()
    piv = torch.empty(mb.v_elems, dtype=torch.int32, device="cuda")
    rc = torch.empty(mb.count, dtype=torch.float64, device="cuda")
    info = torch.empty(mb.count, dtype=torch.int32, device="cuda")
    mb.lu_rcond(a, piv, x, rc, info)
    return x


def solve_fp32_ir(mb, A, B, tol=1e-13, max_iter=10):
    import torch
    work = torch.empty(mb.a_elems, dtype=torch.float32, device="cuda")
    piv = torch.empty(mb.v_elems, dtype=torch.int32, device="cuda")
    x = torch.zeros(mb.v_elems, dtype=torch.float64, device="cuda")
    st = torch.empty(mb.count, dtype=torch.int32, device="cuda")
    mb.ir(A, work, piv, B, x, st, tol, max_iter)
    return x, st


def solve_with_fallback(mb, A, B, first_fp32_idx):
    """FP32 + refinement on first_fp32_idx, FP64 on the rest and on every item
    the FP32 tier did not bring to the bound.  Returns (X, stats)."""
    import torch
    X = torch.empty(mb.v_elems, dtype=torch.float64, device="cuda")
    all_idx = np.arange(mb.count)
    lo = np.asarray(first_fp32_idx, dtype=np.int64)
    hi = np.setdiff1d(all_idx, lo)
    failed = np.zeros(0, dtype=np.int64)
    if len(lo):
        sub, a, b, v_idx = _subset(mb, A, B, lo)
        x, st = solve_fp32_ir(sub, a, b)
        X[v_idx] = x
        failed = lo[(st.cpu().numpy() < 0)]
    redo = np.concatenate([hi, failed]).astype(np.int64)
    if len(redo):
        sub, a, b, v_idx = _subset(mb, A, B, redo)
        X[v_idx] = solve_fp64(sub, a, b)
    return X, {"fp32_attempts": int(len(lo)), "fp32_failed": int(len(failed)), "fp64_solves": int(len(redo))}


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
