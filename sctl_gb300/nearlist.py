"""Near lists on the GPU (BuildNearList, boundary_integral.txx:50-522), through
`sctlgpu_near_list_build`.

    L = NearList(r_trg, elem_nds_cnt, elem_nds_dsp, r_src, src_radius)
    L.arrays()   # near_elem_cnt, near_elem_dsp, near_trg_idx, near_scatter_index,
                 # near_trg_cnt, near_trg_dsp, near_trg_elem (numpy or CUDA tensors)

Inputs are numpy arrays (host) or CUDA tensors (device).  Target t is near
element e when some node s of e has |x_t - x_s| < src_radius[s].
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi

FIELDS = ("near_elem_cnt", "near_elem_dsp", "near_trg_idx", "near_scatter_index", "near_trg_cnt", "near_trg_dsp",
          "near_trg_elem")


def _is_dev(a):
    return hasattr(a, "is_cuda") and a.is_cuda


class NearList:
    def __init__(self, r_trg, elem_nds_cnt, elem_nds_dsp, r_src, src_radius, stream=None):
        lib = capi.load()
        arrs = [r_trg, elem_nds_cnt, elem_nds_dsp, r_src, src_radius]
        dev = [_is_dev(a) for a in arrs]
        if any(dev) and not all(dev):
            raise capi.SctlGpuError(capi.ERR_INVALID_ARGUMENT, "near list inputs: all host or all device")
        self.device = all(dev)
        if self.device:
            import torch
            conv = [a.contiguous() for a in arrs]
            conv[1] = conv[1].to(torch.int64)
            conv[2] = conv[2].to(torch.int64)
            ptr = lambda a: a.data_ptr() if a.numel() else None  # noqa: E731
            size = lambda a: a.numel()  # noqa: E731
            if stream is None:
                stream = torch.cuda.current_stream().cuda_stream
        else:
            conv = [np.ascontiguousarray(arrs[0], np.float64), np.ascontiguousarray(arrs[1], np.int64),
                    np.ascontiguousarray(arrs[2], np.int64), np.ascontiguousarray(arrs[3], np.float64),
                    np.ascontiguousarray(arrs[4], np.float64)]
            ptr = lambda a: a.ctypes.data if a.size else None  # noqa: E731
            size = lambda a: a.size  # noqa: E731
        self._keep = conv
        xt, cnt, dsp, xs, rad = conv
        self.nt, self.n_elem, ns = size(xt) // 3, size(cnt), size(xs) // 3
        if size(dsp) != self.n_elem or size(rad) != ns or size(xt) % 3 or size(xs) % 3:
            raise capi.SctlGpuError(capi.ERR_INVALID_SIZE, "near list input sizes")
        h = ctypes.c_void_p()
        capi.check(lib.sctlgpu_near_list_build(ctypes.byref(h), self.nt, ptr(xt), self.n_elem, ptr(cnt), ptr(dsp), ns,
                                               ptr(xs), ptr(rad), capi.DEVICE_PTRS if self.device else 0, stream),
                   "sctlgpu_near_list_build")
        self._h = h
        n = ctypes.c_int64()
        capi.check(lib.sctlgpu_near_list_sizes(h, ctypes.byref(n), None, None))
        self.n_near = n.value

    def arrays(self, device=None):
        """The seven arrays, as CUDA tensors (device=True) or numpy arrays."""
        device = self.device if device is None else device
        sizes = {"near_elem_cnt": self.n_elem, "near_elem_dsp": self.n_elem, "near_trg_idx": self.n_near,
                 "near_scatter_index": self.n_near, "near_trg_cnt": self.nt, "near_trg_dsp": self.nt,
                 "near_trg_elem": self.n_near}
        if device:
            import torch
            out = {k: torch.empty(max(sizes[k], 1), dtype=torch.int64, device="cuda") for k in FIELDS}
            ptrs = [out[k].data_ptr() for k in FIELDS]
            stream = torch.cuda.current_stream().cuda_stream
        else:
            out = {k: np.empty(max(sizes[k], 1), np.int64) for k in FIELDS}
            ptrs = [out[k].ctypes.data for k in FIELDS]
            stream = None
        capi.check(capi.load().sctlgpu_near_list_get(self._h, *ptrs, stream), "sctlgpu_near_list_get")
        return {k: out[k][:sizes[k]] for k in FIELDS}

    def close(self):
        if getattr(self, "_h", None):
            capi.load().sctlgpu_near_list_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
