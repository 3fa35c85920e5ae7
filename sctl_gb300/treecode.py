"""Far field by a barycentric Lagrange treecode over the C ABI (sctlgpu_treecode_*):
the fast path ParticleFMM::Eval takes for 40,000 targets or more (EvalPVFMM,
fmm-wrapper.txx:854-1038; Eval at :542-549), for the four hot-path kernels.

    tc = Treecode("Laplace3D_DxU", r_src, r_trg, n_src=n_src, digits=10)   # geometry: numpy or tensors
    u = tc.eval(v_src)                                                     # CUDA tensor densities

The geometry calls play SetSrcCoord / SetTrgCoord (fmm-wrapper.txx:505-540):
they build both trees and the interaction blocks once; `eval` is
SetDensitySL/DL + Eval on the device, `eval_host` the same from host arrays.  Accuracy follows `digits` (interpolation
degree and acceptance parameter), or explicit `order` / `theta`.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi

EVAL_DIRECT_BELOW = 40000  # ParticleFMM::EvalPVFMM's cut-over to EvalDirect (fmm-wrapper.txx:864-867)


def _host(a):
    if a is None:
        return None
    if type(a).__module__.startswith("torch"):
        a = a.detach().to("cpu").numpy()
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1)


def _params(order, theta, leaf_max, batch_max, dual=True, theta_trg=0.0, moment_bytes=0.0):
    return capi.TreecodeParams(float(theta or 0.0), int(order or 0), int(leaf_max or 0), int(batch_max or 0),
                               1 if dual else 0, float(theta_trg or 0.0), float(moment_bytes or 0.0))


_SIZE_KEYS = ("blocks", "source_slots", "slots", "clusters", "direct_interactions", "proxy_interactions", "order",
              "target_list", "target_clusters", "direct_fallback")


class Treecode:
    def __init__(self, kernel, r_src, r_trg, n_src=None, digits: int = 10, mode="mixed", order=0, theta=0.0,
                 leaf_max=0, batch_max=0, dual=True, theta_trg=0.0, moment_bytes=0.0):
        self.kernel = capi.KERNEL_IDS[kernel] if isinstance(kernel, str) else int(kernel)
        self.mode = capi.MODE_IDS[mode] if isinstance(mode, str) else int(mode)
        self.digits = int(digits)
        xs, xt, ns_ = _host(r_src), _host(r_trg), _host(n_src)
        self.ns, self.nt = xs.size // 3, xt.size // 3
        _, nd, sd, td = capi.kernel_dims(self.kernel)
        self.sd, self.td = sd, td
        lib = capi.load()
        h = ctypes.c_void_p()
        prm = _params(order, theta, leaf_max, batch_max, dual, theta_trg, moment_bytes)
        rc = lib.sctlgpu_treecode_create(ctypes.byref(h), self.kernel, self.mode, self.digits, self.ns,
                                         xs.ctypes.data if xs.size else None,
                                         ns_.ctypes.data if ns_ is not None and ns_.size else None, self.nt,
                                         xt.ctypes.data if xt.size else None, ctypes.byref(prm))
        capi.check(rc, "sctlgpu_treecode_create")
        self._h = h

    def eval(self, v_src, out=None, accumulate=False, stream=None):
        """Potentials at the targets (nt * TrgDim, FP64, CUDA) for densities v_src (ns * SrcDim, CUDA)."""
        import torch
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        v = v_src.reshape(-1).contiguous()
        if v.dtype != torch.float64 or not v.is_cuda or v.numel() != self.ns * self.sd:
            raise ValueError("v_src must be a CUDA float64 tensor of ns * SrcDim entries")
        if out is None:
            out = torch.empty(self.nt * self.td, dtype=torch.float64, device=v.device)
            accumulate = False
        flags = capi.DEVICE_PTRS | (capi.ACCUMULATE if accumulate else 0)
        rc = capi.load().sctlgpu_treecode_execute(self._h, v.data_ptr() if v.numel() else None,
                                                  out.data_ptr() if out.numel() else None, flags, stream)
        capi.check(rc, "sctlgpu_treecode_execute")
        return out

    def eval_host(self, v_src, out=None, accumulate=False):
        """The same from host arrays (ParticleFMM's Eval on SCTL vectors): densities copied in and
        potentials copied out by the library, synchronously; numpy float64 in and out."""
        v = np.ascontiguousarray(v_src, dtype=np.float64).reshape(-1)
        if v.size != self.ns * self.sd:
            raise ValueError("v_src must hold ns * SrcDim entries")
        if out is None:
            out = np.zeros(self.nt * self.td)
            accumulate = False
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != self.nt * self.td:
            raise ValueError("out must be a contiguous float64 array of nt * TrgDim entries")
        flags = capi.ACCUMULATE if accumulate else 0
        rc = capi.load().sctlgpu_treecode_execute(self._h, v.ctypes.data if v.size else None,
                                                  out.ctypes.data if out.size else None, flags, None)
        capi.check(rc, "sctlgpu_treecode_execute")
        return out

    def info(self):
        sizes = (ctypes.c_int64 * 10)()
        th = ctypes.c_double()
        capi.check(capi.load().sctlgpu_treecode_info(self._h, sizes, ctypes.byref(th)), "sctlgpu_treecode_info")
        d = dict(zip(_SIZE_KEYS, list(sizes)))
        d["theta"] = th.value
        d["direct_sum_interactions"] = self.ns * self.nt
        return d

    def status(self, stream=None):
        return capi.load().sctlgpu_treecode_status(self._h, stream)

    def close(self):
        if getattr(self, "_h", None):
            capi.load().sctlgpu_treecode_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def layout(kernel, r_src, r_trg, digits: int = 10, order=0, theta=0.0, leaf_max=0, batch_max=0, dual=True,
           theta_trg=0.0):
    """The host-only part of Treecode (no device): sizes, blocks (rows of src_begin, src_count,
    trg_begin, trg_count; sources index the source slots, targets the target list of sorted
    targets then target proxies), the source of every slot (-1 padding, -2 proxy), the target
    order, per source cluster with proxies (slot begin, end, proxy begin, end, grid points along
    x, y, z) and per target cluster with proxies (target begin, end, proxy begin, end, grid
    points along x, y, z)."""
    k = capi.KERNEL_IDS[kernel] if isinstance(kernel, str) else int(kernel)
    xs, xt = _host(r_src), _host(r_trg)
    ns, nt = xs.size // 3, xt.size // 3
    lib = capi.load()
    prm = _params(order, theta, leaf_max, batch_max, dual, theta_trg)
    sizes = (ctypes.c_int64 * 10)()
    th = ctypes.c_double()
    args = (k, ns, xs.ctypes.data if ns else None, nt, xt.ctypes.data if nt else None, ctypes.byref(prm), int(digits))
    capi.check(lib.sctlgpu_treecode_layout(*args, sizes, ctypes.byref(th), None, None, None, None, None),
               "sctlgpu_treecode_layout")
    s = dict(zip(_SIZE_KEYS, list(sizes)))
    blocks = np.zeros((s["blocks"], 4), np.int64)
    slot_src = np.zeros(s["slots"], np.int64)
    trg_order = np.zeros(nt, np.int64)
    clusters = np.zeros((s["clusters"], 7), np.int64)
    tclusters = np.zeros((s["target_clusters"], 7), np.int64)
    p = lambda a: a.ctypes.data if a.size else None  # noqa: E731
    capi.check(lib.sctlgpu_treecode_layout(*args, sizes, ctypes.byref(th), p(blocks), p(slot_src), p(trg_order),
                                           p(clusters), p(tclusters)), "sctlgpu_treecode_layout")
    s["theta"] = th.value
    return s, blocks, slot_src, trg_order, clusters, tclusters
