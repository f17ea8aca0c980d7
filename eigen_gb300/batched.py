"""Batched small-system solver (gbs_batched_*): LLT + solve for SPD items,
PartialPivLU + solve for general items, n in [1, 64], one launch per call
(a CUDA graph), buffers packed back to back on the device."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class BatchedSolver:
    def __init__(self, sizes, kinds, dtype=np.float64, use_graph=True):
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        self.kinds = np.ascontiguousarray(kinds, dtype=np.int32)
        self.dtype = np.dtype(dtype)
        self._h = C.c_void_p()
        code = L.GBS_F64 if self.dtype == np.float64 else L.GBS_F32
        L.check(L.lib().gbs_batched_create(C.byref(self._h), code, len(self.sizes),
                                           self.sizes.ctypes.data_as(C.c_void_p),
                                           self.kinds.ctypes.data_as(C.c_void_p), int(use_graph)), "batched.create")
        n = len(self.sizes)
        self.a_off = np.zeros(max(n, 1), dtype=np.int64)
        self.b_off = np.zeros(max(n, 1), dtype=np.int64)
        L.lib().gbs_batched_offsets(self._h, self.a_off.ctypes.data_as(C.c_void_p),
                                    self.b_off.ctypes.data_as(C.c_void_p))
        self.a_elems = int(L.lib().gbs_batched_matrix_elements(self._h))
        self.b_elems = int(L.lib().gbs_batched_rhs_elements(self._h))

    def __del__(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().gbs_batched_destroy(self._h)
            self._h = C.c_void_p()

    def pack(self, mats, rhs):
        """Lists of numpy matrices / vectors -> packed 1-D host arrays."""
        a = np.empty(self.a_elems, dtype=self.dtype)
        b = np.empty(self.b_elems, dtype=self.dtype)
        for i, (m, v) in enumerate(zip(mats, rhs)):
            n = self.sizes[i]
            a[self.a_off[i]:self.a_off[i] + n * n] = np.asarray(m, dtype=self.dtype).reshape(-1, order="F")
            b[self.b_off[i]:self.b_off[i] + n] = v
        return a, b

    def unpack(self, a, b, i):
        n = self.sizes[i]
        return (a[self.a_off[i]:self.a_off[i] + n * n].reshape((n, n), order="F"),
                b[self.b_off[i]:self.b_off[i] + n])

    def solve(self, d_a, d_b, d_info, d_piv, stream=None):
        """Device torch tensors (flat): factors/solutions in place."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        L.check(L.lib().gbs_batched_solve(self._h, C.c_void_p(d_a.data_ptr()), C.c_void_p(d_b.data_ptr()),
                                          C.c_void_p(d_info.data_ptr()), C.c_void_p(d_piv.data_ptr()),
                                          C.c_void_p(s)), "batched.solve")

    def solve_host(self, a, b, info, piv=None, x=None):
        """Host buffers (numpy arrays or CPU torch tensors, flat, packed): the
        solutions go to x (default: b, in place), info (int32) gets the
        per-item status, piv (int32, optional) the LU items' transpositions;
        a is read only.  The copies overlap the solve when the buffers are
        pinned."""
        def ptr(t):
            if t is None:
                return None
            return C.c_void_p(t.data_ptr() if hasattr(t, "data_ptr") else t.ctypes.data)
        L.check(L.lib().gbs_batched_solve_host(self._h, ptr(a), ptr(b), ptr(b if x is None else x), ptr(info),
                                               ptr(piv)), "batched.solve_host")

    def autotune(self, d_a, d_b, d_info, d_piv, persist=False):
        """Chooses each size group's kernel variant by timing the whole batch
        on these buffers; every run starts from their contents, which are
        restored on return.  Returns config()."""
        L.check(L.lib().gbs_batched_autotune(self._h, C.c_void_p(d_a.data_ptr()), C.c_void_p(d_b.data_ptr()),
                                             C.c_void_p(d_info.data_ptr()), C.c_void_p(d_piv.data_ptr()),
                                             int(persist)), "batched.autotune")
        return self.config()

    def buckets(self):
        """The plan's buckets: kind, size class, items, largest n, variant."""
        cnt = C.c_int()
        L.check(L.lib().gbs_batched_buckets(self._h, 0, C.byref(cnt), None), "batched.buckets")
        d = np.zeros(7 * max(cnt.value, 1), dtype=np.int32)
        L.check(L.lib().gbs_batched_buckets(self._h, cnt.value, C.byref(cnt),
                                            d.ctypes.data_as(C.POINTER(C.c_int))),
                "batched.buckets")
        keys = ("kind", "n_lo", "n_hi", "items", "max_n", "lanes_per_system", "warps_per_cta")
        return [dict(zip(keys, map(int, d[7 * i:7 * i + 7]))) for i in range(cnt.value)]

    def set_variant(self, bucket, lanes_per_system, warps_per_cta=1):
        L.check(L.lib().gbs_batched_set_variant(self._h, int(bucket), int(lanes_per_system), int(warps_per_cta)),
                "batched.set_variant")

    def config(self):
        ws, wl = C.c_int(), C.c_int()
        L.lib().gbs_batched_config(self._h, C.byref(ws), C.byref(wl))
        return {"warps_per_cta_n<=32": ws.value, "warps_per_cta_n<=64": wl.value, "buckets": self.buckets()}
