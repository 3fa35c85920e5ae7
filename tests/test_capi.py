"""The C-ABI library loads, exports every symbol include/*.h declares, and
rejects bad arguments with status codes -- no GPU needed (the argument checks
run before any device call)."""
import os
import re

import numpy as np
import pytest

import sctl_gb300 as S
from sctl_gb300 import capi

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for fn in os.listdir(INCLUDE):
        if fn.endswith(".h"):
            src = open(os.path.join(INCLUDE, fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(sctlgpu_\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    names = declared_symbols()
    assert "sctlgpu_eval" in names and "sctlgpu_kernel_matrix" in names
    for n in names:
        assert hasattr(lib, n), n
    assert names <= set(capi.SIGNATURES), names - set(capi.SIGNATURES)


def test_kernel_dims_match_reference():
    assert capi.kernel_dims(0) == (3, 0, 1, 1)
    assert capi.kernel_dims(1) == (3, 3, 1, 1)
    assert capi.kernel_dims(2) == (3, 0, 3, 3)
    assert capi.kernel_dims(3) == (3, 3, 3, 3)
    with pytest.raises(S.SctlGpuError):
        capi.kernel_dims(16)
    for k, v in ((0, 1 / (4 * np.pi)), (1, 1 / (4 * np.pi)), (2, 1 / (8 * np.pi)), (3, 3 / (4 * np.pi))):
        assert abs(capi.load().sctlgpu_scale_factor(k) - v) < 1e-17
    # the other twelve micro-kernels (kernel_functions.hpp:81-659): dims and uKerScaleFactor
    from oracle import oracle as O
    for k in range(4, 16):
        assert capi.kernel_dims(k)[1:] == O.DIMS[k], k
        assert abs(capi.load().sctlgpu_scale_factor(k) - O.scale_factor(k)) < 1e-17, k


def test_argument_errors_without_gpu():
    lib = capi.load()
    x = np.zeros(6)
    p = x.ctypes.data
    assert lib.sctlgpu_eval(16, 0, -1, 1, p, 1, p, None, p, p, 0, None) == capi.ERR_INVALID_KERNEL
    assert lib.sctlgpu_eval(0, 7, -1, 1, p, 1, p, None, p, p, 0, None) == capi.ERR_INVALID_MODE
    assert lib.sctlgpu_eval(0, 0, -1, -1, p, 1, p, None, p, p, 0, None) == capi.ERR_INVALID_SIZE
    assert lib.sctlgpu_eval(0, 0, -1, 1, None, 1, p, None, p, p, 0, None) == capi.ERR_NULL_POINTER
    assert lib.sctlgpu_eval(1, 0, -1, 1, p, 1, p, None, p, p, 0, None) == capi.ERR_NULL_POINTER  # DxU needs normals
    assert lib.sctlgpu_eval(0, 0, -1, 1 << 62, p, 1, p, None, p, p, 0, None) == capi.ERR_INVALID_SIZE
    assert lib.sctlgpu_kernel_matrix(0, 0, -1, 1, p, 1, p, None, None, 0, None) == capi.ERR_NULL_POINTER
    # the Helmholtz kernels need their wavenumber (ctx); the hot-path-only entries refuse ids >= 4
    assert lib.sctlgpu_eval(9, 0, -1, 1, p, 1, p, None, p, p, 0, None) == capi.ERR_NULL_POINTER
    assert lib.sctlgpu_kernel_matrix(11, 0, -1, 1, p, 1, p, None, p, 0, None) == capi.ERR_NULL_POINTER
    assert lib.sctlgpu_eval_mixed_noalloc(4, 10, 1, p, 1, p, None, p, p, 2, None) == capi.ERR_INVALID_KERNEL
    # zero targets is a no-op that needs no device
    assert lib.sctlgpu_eval(0, 0, -1, 0, None, 5, p, None, p, None, 0, None) == capi.OK
    # near-matrix application: TrgDim must be 1, 2, 3, 4 or 9; pointers checked before any launch
    na = lambda k1, nt, tdsp, n_near=0, tp=None: lib.sctlgpu_near_matrix_apply(  # noqa: E731
        1, k1, nt, tdsp, n_near, tp, 1, p, p, 1, p, p, 6, p, 6, p, p, None)
    assert na(5, 1, p) == capi.ERR_INVALID_SIZE
    assert na(1, -1, p) == capi.ERR_INVALID_SIZE
    assert na(1, 1, p, n_near=2) == capi.ERR_INVALID_SIZE  # identity order needs n_near <= n_pairs
    assert na(1, 1, None) == capi.ERR_NULL_POINTER
    assert na(1, 0, None) == capi.OK
    # the float-pair form: same checks, plus 8-byte alignment of the pairs
    nb = lambda k1, nt, tdsp, K2=p: lib.sctlgpu_near_matrix_apply_pairs(  # noqa: E731
        1, k1, nt, tdsp, 0, None, 1, p, p, 1, p, p, 6, K2, 6, p, p, None)
    assert nb(5, 1, p) == capi.ERR_INVALID_SIZE
    assert nb(1, 1, None) == capi.ERR_NULL_POINTER
    assert nb(1, 1, p, K2=None) == capi.ERR_NULL_POINTER
    assert nb(1, 1, p, K2=p + 4) == capi.ERR_INVALID_SIZE
    assert nb(1, 0, None) == capi.OK
    assert lib.sctlgpu_to_float_pairs(-1, p, p, None) == capi.ERR_INVALID_SIZE
    assert lib.sctlgpu_to_float_pairs(3, None, p, None) == capi.ERR_NULL_POINTER
    assert lib.sctlgpu_to_float_pairs(3, p, p + 4, None) == capi.ERR_INVALID_SIZE
    assert lib.sctlgpu_to_float_pairs(0, None, None, None) == capi.OK
    for code in (0, -1, -2, -3, -4, -5, -6, -7, -8, -9):
        assert lib.sctlgpu_strerror(code)


def test_python_eval_rejects_mismatched_sizes():
    with pytest.raises(S.SctlGpuError):
        S.Laplace3D_FxU.Eval(None, np.zeros(3), np.zeros(6), None, np.ones(3))


def test_newton_schedule():
    # rsqrt.approx seed ~ 6.89 digits: FP32 full (6 digits) needs no step, FP64 full two.
    assert capi.newton_steps("f32", -1) == 0
    assert capi.newton_steps("f64", -1) == 2
    assert capi.newton_steps("f64", 16) == 2
    assert capi.newton_steps("f64", 4) == 0
    assert capi.newton_steps("f64", 6) == 1   # the f64 seed is 2^-20.1 with a margin for r^-5
    assert capi.newton_steps("f64", 10) == 1
    assert capi.newton_steps("mixed", 6) == 0
    assert capi.newton_steps("mixed", 10) == 1


def test_launch_counter_starts_readable():
    assert isinstance(capi.launch_count(), int)
    assert capi.load().sctlgpu_last_kernel_ms() < 0 or True


def test_digits_for_tolerance_follows_set_accuracy():
    """BoundaryIntegralOp::SetAccuracy's tolerance -> digits rule (boundary_integral.txx:588-595),
    on tolerances away from exact powers of ten (where the floating log ratio may fall either side
    of the integer)."""
    import sctl_gb300 as S
    assert S.digits_for_tolerance(3e-7) == 7
    assert S.digits_for_tolerance(5e-11) == 11
    assert S.digits_for_tolerance(0.5) == 1
    assert S.digits_for_tolerance(2.0) == 1  # log(2)/log(0.1) = -0.30 truncates to 0, plus one
    with pytest.raises(ValueError):
        S.digits_for_tolerance(0.0)
