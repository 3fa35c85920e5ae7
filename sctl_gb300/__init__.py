"""sctl_gb300 -- GB300 (sm_103a) drop-in for SCTL's particle-kernel hot path.

Python mirror of sctl::GenericKernel (include/sctl/generic-kernel.hpp) for the
micro-kernels of include/sctl/kernel_functions.hpp: the four that
BoundaryIntegralOp and ParticleFMM evaluate on the hot path (Laplace3D_FxU,
Laplace3D_DxU, Stokes3D_FxU, Stokes3D_DxU; every precision mode) and the other
twelve (Laplace gradient / Hessian, BiotSavart, Helmholtz, Stokes traction /
source-sink / pressure; FP64 and FP32).  The Helmholtz kernels need their
wavenumber, the reference's ctx_ptr: GenericKernel("Helmholtz3D_FxU", ctx=k).
All compute runs in libsctlgpu.so through its C ABI (include/sctlgpu.h).

Arguments follow the reference: flat array-of-structures coordinates
(r_trg[nt*3], r_src[ns*3], n_src[ns*3] for double-layer kernels), densities
v_src[ns*SrcDim()], potentials v_trg[nt*TrgDim()].  Eval re-initialises and
zeroes v_trg when its size is wrong and otherwise adds into it
(generic-kernel.txx:129-132).  Host arrays are numpy; CUDA torch tensors are
passed as device pointers on the current torch stream.
"""
from __future__ import annotations

import numpy as np

from . import capi
from .capi import F32, F64, MIXED, SctlGpuError, kernel_dims, launch_count  # noqa: F401

__all__ = ["GenericKernel", "Laplace3D_FxU", "Laplace3D_DxU", "Stokes3D_FxU", "Stokes3D_DxU", "Laplace3D_FxdU",
           "Laplace3D_Fxd2U", "Laplace3D_DxdU", "BiotSavart3D_FxU", "BiotSavart3D_FxdU", "Stokes3D_FxT",
           "Stokes3D_FSxU", "Stokes3D_FxUP", "SctlGpuError", "F64", "F32", "MIXED", "eval_device",
           "kernel_matrix_device", "digits_for_tolerance"]


def digits_for_tolerance(tol: float) -> int:
    """The `digits` a boundary-integral operator passes to its far-field evaluator for accuracy
    `tol`: BoundaryIntegralOp::SetAccuracy (boundary_integral.txx:588-595) uses
    (Integer)(log(tol) / log(0.1)) + 1, truncation toward zero."""
    import math
    if not tol > 0:
        raise ValueError("tolerance must be positive")
    return int(math.log(tol) / math.log(0.1)) + 1


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _mode_for(dtype, mode):
    if mode is not None:
        return capi.MODE_IDS[mode] if isinstance(mode, str) else int(mode)
    return F32 if np.dtype(dtype) == np.float32 else F64


def _real(mode):
    return np.float32 if mode == F32 else np.float64


def _ctx_arg(mode, ctx):
    """Host value of the call's real type holding the kernel context (or None)."""
    import ctypes
    if ctx is None:
        return None, None
    v = ctypes.c_float(ctx) if mode == F32 else ctypes.c_double(ctx)
    return v, ctypes.addressof(v)


def eval_device(kernel: int, mode: int, digits: int, nt: int, r_trg: int, ns: int, r_src: int, n_src: int,
                v_src: int, v_trg: int, accumulate: bool, stream: int = 0, ctx=None) -> None:
    """Raw device-pointer entry (asynchronous on `stream`)."""
    flags = capi.DEVICE_PTRS | (capi.ACCUMULATE if accumulate else 0)
    keep, cp = _ctx_arg(mode, ctx)
    capi.check(capi.load().sctlgpu_eval_ctx(kernel, mode, digits, nt, r_trg, ns, r_src, n_src or None, v_src, v_trg,
                                            flags, cp, stream or None), "sctlgpu_eval")


def kernel_matrix_device(kernel: int, mode: int, digits: int, nt: int, r_trg: int, ns: int, r_src: int, n_src: int,
                         M: int, stream: int = 0, ctx=None) -> None:
    keep, cp = _ctx_arg(mode, ctx)
    capi.check(capi.load().sctlgpu_kernel_matrix_ctx(kernel, mode, digits, nt, r_trg, ns, r_src, n_src or None, M,
                                                     capi.DEVICE_PTRS, cp, stream or None), "sctlgpu_kernel_matrix")


class GenericKernel:
    """One micro-kernel behind the GenericKernel API."""

    def __init__(self, name: str, ctx=None):
        self.name = name
        self.kernel_id = capi.KERNEL_IDS[name]
        self.ctx = ctx  # the reference's ctx_ptr target (Helmholtz wavenumber)

    def SetCtx(self, ctx):
        """GenericKernel::SetCtxPtr (generic-kernel.hpp:79), by value."""
        self.ctx = ctx
        return self

    # dims are constexpr in the reference (generic-kernel.hpp:54-74)
    def CoordDim(self) -> int:
        return 3

    def NormalDim(self) -> int:
        return _DIMS[self.kernel_id][0]

    def SrcDim(self) -> int:
        return _DIMS[self.kernel_id][1]

    def TrgDim(self) -> int:
        return _DIMS[self.kernel_id][2]

    def Name(self) -> str:
        return self.name.replace("_", "-")

    def ScaleFactor(self) -> float:
        return float(capi.load().sctlgpu_scale_factor(self.kernel_id))

    def Eval(self, v_trg, r_trg, r_src, n_src, v_src, digits: int = -1, mode=None):
        """GenericKernel<uK>::Eval<Real,true>(v_trg, r_trg, r_src, n_src, v_src, digits, self).

        Returns v_trg (the same object when it was correctly sized, else a new
        zero-initialised array/tensor holding the result).
        """
        nd, sd, td = _DIMS[self.kernel_id]
        if _is_torch(r_trg) and r_trg.is_cuda:
            return self._eval_torch(v_trg, r_trg, r_src, n_src, v_src, digits, mode)
        m = _mode_for(np.asarray(r_trg).dtype, mode)
        dt = _real(m)
        r_trg = np.ascontiguousarray(r_trg, dt).reshape(-1)
        r_src = np.ascontiguousarray(r_src, dt).reshape(-1)
        v_src = np.ascontiguousarray(v_src, dt).reshape(-1)
        n_src = np.ascontiguousarray(n_src, dt).reshape(-1) if nd else None
        nt, ns = r_trg.size // 3, r_src.size // 3
        if r_trg.size != nt * 3 or r_src.size != ns * 3 or v_src.size != ns * sd or (nd and n_src.size != ns * nd):
            raise SctlGpuError(capi.ERR_INVALID_SIZE, "Eval: array sizes do not match the kernel dimensions")
        accumulate = v_trg is not None and np.asarray(v_trg).size == nt * td
        if accumulate:
            out = v_trg if (isinstance(v_trg, np.ndarray) and v_trg.dtype == dt and v_trg.flags.c_contiguous) \
                else np.ascontiguousarray(v_trg, dt)
        else:
            out = np.zeros(nt * td, dt)
        ptr = lambda a: None if a is None or a.size == 0 else a.ctypes.data  # noqa: E731
        keep, cp = _ctx_arg(m, self.ctx)
        rc = capi.load().sctlgpu_eval_ctx(self.kernel_id, m, int(digits), nt, ptr(r_trg), ns, ptr(r_src),
                                          ptr(n_src), ptr(v_src), ptr(out), capi.ACCUMULATE if accumulate else 0, cp,
                                          None)
        capi.check(rc, f"{self.name}.Eval")
        if accumulate and out is not v_trg:
            np.copyto(np.asarray(v_trg).reshape(-1), out.reshape(np.asarray(v_trg).reshape(-1).shape))
            return v_trg
        return out

    def _eval_torch(self, v_trg, r_trg, r_src, n_src, v_src, digits, mode):
        import torch
        nd, sd, td = _DIMS[self.kernel_id]
        m = _mode_for(np.float32 if r_trg.dtype == torch.float32 else np.float64, mode)
        tdt = torch.float32 if m == F32 else torch.float64
        r_trg = r_trg.contiguous().to(tdt).reshape(-1)
        r_src = r_src.contiguous().to(tdt).reshape(-1)
        v_src = v_src.contiguous().to(tdt).reshape(-1)
        n_src = n_src.contiguous().to(tdt).reshape(-1) if nd else None
        nt, ns = r_trg.numel() // 3, r_src.numel() // 3
        accumulate = v_trg is not None and v_trg.numel() == nt * td
        if accumulate:
            if v_trg.dtype != tdt or not v_trg.is_contiguous():
                raise SctlGpuError(capi.ERR_INVALID_ARGUMENT, "Eval: v_trg must be contiguous and of the Real type")
            out = v_trg
        else:
            out = torch.zeros(nt * td, dtype=tdt, device=r_trg.device)
        stream = torch.cuda.current_stream(r_trg.device).cuda_stream
        eval_device(self.kernel_id, m, int(digits), nt, r_trg.data_ptr(), ns, r_src.data_ptr(),
                    n_src.data_ptr() if n_src is not None else 0, v_src.data_ptr(), out.data_ptr(), accumulate,
                    stream, self.ctx)
        return out

    def KernelMatrix(self, Xt, Xs, Xn, digits: int = -1, mode=None):
        """GenericKernel<uK>::KernelMatrix<Real,omp,digits>(M, Xt, Xs, Xn): returns M of shape
        (Ns*SrcDim, Nt*TrgDim), source-major and scaled."""
        nd, sd, td = _DIMS[self.kernel_id]
        if _is_torch(Xt) and Xt.is_cuda:
            import torch
            m = _mode_for(np.float32 if Xt.dtype == torch.float32 else np.float64, mode)
            tdt = torch.float32 if m == F32 else torch.float64
            Xt = Xt.contiguous().to(tdt).reshape(-1)
            Xs = Xs.contiguous().to(tdt).reshape(-1)
            Xn = Xn.contiguous().to(tdt).reshape(-1) if nd else None
            nt, ns = Xt.numel() // 3, Xs.numel() // 3
            M = torch.empty((ns * sd, nt * td), dtype=tdt, device=Xt.device)
            kernel_matrix_device(self.kernel_id, m, int(digits), nt, Xt.data_ptr(), ns, Xs.data_ptr(),
                                 Xn.data_ptr() if Xn is not None else 0, M.data_ptr(),
                                 torch.cuda.current_stream(Xt.device).cuda_stream, self.ctx)
            return M
        m = _mode_for(np.asarray(Xt).dtype, mode)
        dt = _real(m)
        Xt = np.ascontiguousarray(Xt, dt).reshape(-1)
        Xs = np.ascontiguousarray(Xs, dt).reshape(-1)
        Xn = np.ascontiguousarray(Xn, dt).reshape(-1) if nd else None
        nt, ns = Xt.size // 3, Xs.size // 3
        M = np.zeros((ns * sd, nt * td), dt)
        ptr = lambda a: None if a is None or a.size == 0 else a.ctypes.data  # noqa: E731
        keep, cp = _ctx_arg(m, self.ctx)
        rc = capi.load().sctlgpu_kernel_matrix_ctx(self.kernel_id, m, int(digits), nt, ptr(Xt), ns, ptr(Xs),
                                                   ptr(Xn), ptr(M), 0, cp, None)
        capi.check(rc, f"{self.name}.KernelMatrix")
        return M


# (NormalDim, SrcDim, TrgDim) of each kernel id -- generic-kernel.hpp:54-74 with kernel_functions.hpp.
_DIMS = {capi.LAPLACE3D_FXU: (0, 1, 1), capi.LAPLACE3D_DXU: (3, 1, 1),
         capi.STOKES3D_FXU: (0, 3, 3), capi.STOKES3D_DXU: (3, 3, 3),
         4: (0, 1, 3), 5: (0, 1, 9), 6: (3, 1, 3), 7: (0, 3, 3), 8: (0, 3, 9), 9: (0, 2, 2), 10: (3, 2, 2),
         11: (0, 2, 6), 12: (0, 2, 6), 13: (0, 3, 9), 14: (0, 4, 3), 15: (0, 3, 4)}

Laplace3D_FxU = GenericKernel("Laplace3D_FxU")
Laplace3D_DxU = GenericKernel("Laplace3D_DxU")
Stokes3D_FxU = GenericKernel("Stokes3D_FxU")
Stokes3D_DxU = GenericKernel("Stokes3D_DxU")
Laplace3D_FxdU = GenericKernel("Laplace3D_FxdU")
Laplace3D_Fxd2U = GenericKernel("Laplace3D_Fxd2U")
Laplace3D_DxdU = GenericKernel("Laplace3D_DxdU")
BiotSavart3D_FxU = GenericKernel("BiotSavart3D_FxU")
BiotSavart3D_FxdU = GenericKernel("BiotSavart3D_FxdU")
Stokes3D_FxT = GenericKernel("Stokes3D_FxT")
Stokes3D_FSxU = GenericKernel("Stokes3D_FSxU")
Stokes3D_FxUP = GenericKernel("Stokes3D_FxUP")
