"""ctypes binding of libsctlgpu (the C ABI declared in include/sctlgpu.h).

The product path: every call goes to the CUDA library.  If the library is
missing or cannot be loaded the import of the entry points raises -- there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsctlgpu.so")

# Mirrors of the enums in include/sctlgpu.h
LAPLACE3D_FXU, LAPLACE3D_DXU, STOKES3D_FXU, STOKES3D_DXU = 0, 1, 2, 3
F64, F32, MIXED = 0, 1, 2
ACCUMULATE, DEVICE_PTRS = 1, 2
OK = 0
ERR_INVALID_KERNEL, ERR_INVALID_MODE, ERR_INVALID_SIZE, ERR_NULL_POINTER = -1, -2, -3, -4
ERR_CUDA, ERR_NO_DEVICE, ERR_DEVICE_TIMEOUT, ERR_INVALID_ARGUMENT, ERR_TOO_LARGE = -5, -6, -7, -8, -9

KERNEL_IDS = {"Laplace3D_FxU": LAPLACE3D_FXU, "Laplace3D_DxU": LAPLACE3D_DXU,
              "Stokes3D_FxU": STOKES3D_FXU, "Stokes3D_DxU": STOKES3D_DXU,
              "Laplace3D_FxdU": 4, "Laplace3D_Fxd2U": 5, "Laplace3D_DxdU": 6, "BiotSavart3D_FxU": 7,
              "BiotSavart3D_FxdU": 8, "Helmholtz3D_FxU": 9, "Helmholtz3D_DxU": 10, "Helmholtz3D_FxdU": 11,
              "HelmholtzDiff3D_FxdU": 12, "Stokes3D_FxT": 13, "Stokes3D_FSxU": 14, "Stokes3D_FxUP": 15}
HELMHOLTZ_IDS = (9, 10, 11, 12)
MODE_IDS = {"f64": F64, "f32": F32, "mixed": MIXED}

# Every symbol include/*.h declares, with its ctypes signature.
_i, _i64, _u, _vp, _d, _cp = ctypes.c_int, ctypes.c_int64, ctypes.c_uint, ctypes.c_void_p, ctypes.c_double, ctypes.c_char_p
_ip = ctypes.POINTER(ctypes.c_int)
SIGNATURES = {
    "sctlgpu_kernel_dims": (_i, [_i, _ip, _ip, _ip, _ip]),
    "sctlgpu_scale_factor": (_d, [_i]),
    "sctlgpu_eval": (_i, [_i, _i, _i, _i64, _vp, _i64, _vp, _vp, _vp, _vp, _u, _vp]),
    "sctlgpu_kernel_matrix": (_i, [_i, _i, _i, _i64, _vp, _i64, _vp, _vp, _vp, _u, _vp]),
    "sctlgpu_eval_ctx": (_i, [_i, _i, _i, _i64, _vp, _i64, _vp, _vp, _vp, _vp, _u, _vp, _vp]),
    "sctlgpu_kernel_matrix_ctx": (_i, [_i, _i, _i, _i64, _vp, _i64, _vp, _vp, _vp, _u, _vp, _vp]),
    "sctlgpu_strerror": (_cp, [_i]),
    "sctlgpu_last_cuda_error": (_cp, []),
    "sctlgpu_device_status": (_i, [_vp]),
    "sctlgpu_launch_count": (_i64, []),
    "sctlgpu_set_timing": (_i, [_i]),
    "sctlgpu_last_kernel_ms": (_d, []),
    "sctlgpu_newton_steps": (_i, [_i, _i]),
    "sctlgpu_eval_mixed_noalloc": (_i, [_i, _i, _i64, _vp, _i64, _vp, _vp, _vp, _vp, _u, _vp]),
    "sctlgpu_near_plan_create": (_i, [ctypes.POINTER(_vp), _i, _i, _i, _i64, _vp, _i64, _i64, _vp, _i64]),
    "sctlgpu_near_plan_create_indexed": (_i, [ctypes.POINTER(_vp), _i, _i, _i, _i64, _vp, _i64, _i64, _vp, _i64,
                                              _vp, _i64]),
    "sctlgpu_near_plan_execute": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _u, _vp]),
    "sctlgpu_near_plan_info": (_i, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64), _ip]),
    "sctlgpu_near_plan_status": (_i, [_vp, _vp]),
    "sctlgpu_near_plan_destroy": (_i, [_vp]),
    "sctlgpu_near_autotune": (_i, [_i, _i, _i, _ip]),
    "sctlgpu_panel_near_weights": (_i, [_i, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _d, _i, _vp, _vp]),
    "sctlgpu_mlp_create": (_i, [ctypes.POINTER(_vp), _i, _i, _i, ctypes.c_uint64]),
    "sctlgpu_mlp_destroy": (_i, [_vp]),
    "sctlgpu_mlp_num_params": (_i64, [_vp]),
    "sctlgpu_mlp_get_params": (_i, [_vp, _vp]),
    "sctlgpu_mlp_set_params": (_i, [_vp, _vp]),
    "sctlgpu_mlp_forward": (_i, [_vp, _i, _vp, _vp, _vp]),
    "sctlgpu_mlp_forward_dot": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp]),
    "sctlgpu_mlp_train_step": (_i, [_vp, _i, _vp, _vp, ctypes.c_float, _vp, _vp]),
    "sctlgpu_mlp_gradients": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "sctlgpu_near_list_build": (_i, [ctypes.POINTER(_vp), _i64, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _u, _vp]),
    "sctlgpu_near_list_sizes": (_i, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "sctlgpu_near_list_get": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "sctlgpu_near_list_elem_index": (_i, [_vp, _vp, _vp]),
    "sctlgpu_near_list_destroy": (_i, [_vp]),
    "sctlgpu_far_densities": (_i, [_i64, _i, _vp, _vp, _vp, _vp]),
    "sctlgpu_near_matrix_apply": (_i, [_i, _i, _i64, _vp, _i64, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _i64, _vp,
                                      _vp, _vp]),
    "sctlgpu_near_matrix_apply_pairs": (_i, [_i, _i, _i64, _vp, _i64, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp,
                                            _i64, _vp, _vp, _vp]),
    "sctlgpu_to_float_pairs": (_i, [_i64, _vp, _vp, _vp]),
    "sctlgpu_near_matrix_resolve": (_i, [_i, _i, _i64, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _i64, _i64, _vp, _vp]),
    "sctlgpu_near_matrix_apply_resolved": (_i, [_i, _i, _i64, _vp, _i64, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp]),
    "sctlgpu_device_status_word": (_i, [_vp, ctypes.POINTER(ctypes.c_uint)]),
    "sctlgpu_panel_arithmetic": (_i, [_i]),
    "sctlgpu_tc_gemm_bf16": (_i, [_i, _i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _i, _vp]),
    "sctlgpu_panel_near_correction": (_i, [_i, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _i64, _d,
                                           _i, _i, _vp, _vp]),
    "sctlgpu_treecode_create": (_i, [ctypes.POINTER(_vp), _i, _i, _i, _i64, _vp, _vp, _i64, _vp, _vp]),
    "sctlgpu_treecode_execute": (_i, [_vp, _vp, _vp, _u, _vp]),
    "sctlgpu_treecode_info": (_i, [_vp, _vp, ctypes.POINTER(_d)]),
    "sctlgpu_treecode_status": (_i, [_vp, _vp]),
    "sctlgpu_treecode_destroy": (_i, [_vp]),
    "sctlgpu_treecode_layout": (_i, [_i, _i64, _vp, _i64, _vp, _vp, _i, _vp, ctypes.POINTER(_d), _vp, _vp, _vp, _vp,
                                     _vp]),
}


class TreecodeParams(ctypes.Structure):
    """sctlgpu_treecode_params."""
    _fields_ = [("theta", ctypes.c_double), ("order", ctypes.c_int), ("leaf_max", ctypes.c_int),
                ("batch_max", ctypes.c_int), ("dual", ctypes.c_int), ("theta_trg", ctypes.c_double),
                ("moment_bytes", ctypes.c_double)]
NEAR_CLASSES = 10
NOALLOC_SCRATCH_BYTES = 64 << 20

_lib = None


class SctlGpuError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        lib = _lib
        msg = lib.sctlgpu_strerror(status).decode() if lib is not None else str(status)
        if status == ERR_CUDA and lib is not None:
            msg += ": " + lib.sctlgpu_last_cuda_error().decode()
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


def load(path: str | None = None):
    """Load libsctlgpu.so (built in-tree by sctl_gb300.build); raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"libsctlgpu.so not built ({p}); run `python -m sctl_gb300.build`")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise SctlGpuError(status, what)


def kernel_dims(kernel) -> tuple[int, int, int, int]:
    k = KERNEL_IDS[kernel] if isinstance(kernel, str) else int(kernel)
    c, n, s, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(load().sctlgpu_kernel_dims(k, ctypes.byref(c), ctypes.byref(n), ctypes.byref(s), ctypes.byref(t)),
          "sctlgpu_kernel_dims")
    return c.value, n.value, s.value, t.value


def launch_count() -> int:
    return int(load().sctlgpu_launch_count())


def set_timing(enable: bool) -> None:
    load().sctlgpu_set_timing(1 if enable else 0)


def last_kernel_ms() -> float:
    return float(load().sctlgpu_last_kernel_ms())


def newton_steps(mode, digits) -> int:
    m = MODE_IDS[mode] if isinstance(mode, str) else int(mode)
    return int(load().sctlgpu_newton_steps(m, int(digits)))
