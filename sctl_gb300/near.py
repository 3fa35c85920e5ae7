"""Batched near-field direct sums (BoundaryIntegralOp's per-block near work,
boundary_integral.txx:1165-1240 and :1311-1381) over the C ABI's plan API.

    plan = NearPlan("Laplace3D_DxU", blocks, ns, nt, mode="mixed", digits=10)
    plan.execute(r_trg, r_src, n_src, v_src, v_out, w_src=None)   # torch CUDA tensors

`blocks` is an (nblk, 4) int64 array of (src_begin, src_count, trg_begin,
trg_count) rows into the concatenated source / target arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi


class NearPlan:
    def __init__(self, kernel, blocks, ns: int, nt: int, mode="mixed", digits: int = -1, trg_map=None,
                 n_out: int | None = None, trg_index=None):
        """trg_index (optional): block target ranges index this list of target indices in [0, nt)
        (a near list); results then scatter to the listed targets."""
        self.kernel = capi.KERNEL_IDS[kernel] if isinstance(kernel, str) else int(kernel)
        self.mode = capi.MODE_IDS[mode] if isinstance(mode, str) else int(mode)
        self.blocks = np.ascontiguousarray(blocks, dtype=np.int64).reshape(-1, 4)
        self.ns, self.nt = int(ns), int(nt)
        lib = capi.load()
        h = ctypes.c_void_p()
        tm = None
        if trg_map is not None:
            self._map = np.ascontiguousarray(trg_map, dtype=np.int64)
            tm = self._map.ctypes.data
        ti, n_index = None, 0
        if trg_index is not None:
            self._index = np.ascontiguousarray(trg_index, dtype=np.int64)
            ti, n_index = self._index.ctypes.data, self._index.size
        rc = lib.sctlgpu_near_plan_create_indexed(ctypes.byref(h), self.kernel, self.mode, int(digits),
                                                  self.blocks.shape[0],
                                                  self.blocks.ctypes.data if self.blocks.size else None,
                                                  self.ns, self.nt, ti, n_index, tm,
                                                  int(n_out if n_out is not None else -1))
        capi.check(rc, "sctlgpu_near_plan_create")
        self._h = h

    def execute(self, r_trg, r_src, n_src, v_src, v_out, w_src=None, accumulate=False, stream=None):
        import torch
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        p = lambda t: None if t is None or t.numel() == 0 else t.data_ptr()  # noqa: E731
        flags = capi.DEVICE_PTRS | (capi.ACCUMULATE if accumulate else 0)
        rc = capi.load().sctlgpu_near_plan_execute(self._h, p(r_trg), p(r_src), p(n_src), p(v_src), p(w_src),
                                                   p(v_out), flags, stream)
        capi.check(rc, "sctlgpu_near_plan_execute")
        return v_out

    def info(self):
        n, q, g = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        capi.check(capi.load().sctlgpu_near_plan_info(self._h, ctypes.byref(n), ctypes.byref(q), ctypes.byref(g)))
        return {"items": n.value, "interactions": q.value, "graph_kernels": g.value}

    def status(self, stream=None):
        return capi.load().sctlgpu_near_plan_status(self._h, stream)

    def close(self):
        if getattr(self, "_h", None):
            capi.load().sctlgpu_near_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(kernel, mode="mixed", digits=-1):
    k = capi.KERNEL_IDS[kernel] if isinstance(kernel, str) else int(kernel)
    m = capi.MODE_IDS[mode] if isinstance(mode, str) else int(mode)
    out = (ctypes.c_int * capi.NEAR_CLASSES)()
    capi.check(capi.load().sctlgpu_near_autotune(k, m, int(digits), out), "sctlgpu_near_autotune")
    return list(out)
