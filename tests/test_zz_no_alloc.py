"""sctlgpu_eval_mixed_noalloc: the direct sum for callers that cannot allocate
device memory (a host whose device memory belongs to another allocator, code
running after allocations are frozen, real-time loops).  It must agree with
sctlgpu_eval on the same inputs, also when called twice in a row (its fixed
scratch array keeps the previous call's contents), and must refuse problems
larger than its 64 MiB array before launching anything.

Collected last (file name) so a failure here does not hide other results."""
import numpy as np
import pytest

from oracle import oracle as O
from sctl_gb300 import capi
from sctl_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _dev(torch, d):
    return {a: torch.from_numpy(np.ascontiguousarray(v)).cuda() for a, v in d.items()}


def _ptr(t):
    return t.data_ptr() if t.numel() else None


def _existing(torch, k, dd, digits, nt, ns, td):
    out = torch.zeros(nt * td, dtype=torch.float64, device="cuda")
    rc = capi.load().sctlgpu_eval(k, capi.MIXED, digits, nt, _ptr(dd["r_trg"]), ns, _ptr(dd["r_src"]),
                                  _ptr(dd["n_src"]), _ptr(dd["v_src"]), out.data_ptr(), capi.DEVICE_PTRS, None)
    assert rc == capi.OK
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _noalloc(torch, k, dd, digits, nt, ns, td, out=None, flags=0):
    if out is None:
        out = torch.full((nt * td,), 7.0, dtype=torch.float64, device="cuda")  # stale values must not leak in
    stream = torch.cuda.current_stream().cuda_stream
    rc = capi.load().sctlgpu_eval_mixed_noalloc(k, digits, nt, _ptr(dd["r_trg"]), ns, _ptr(dd["r_src"]),
                                                _ptr(dd["n_src"]), _ptr(dd["v_src"]), out.data_ptr(), flags,
                                                stream)
    assert rc == capi.OK, capi.load().sctlgpu_strerror(rc)
    return out.cpu().numpy()


@pytest.mark.parametrize("k,digits", [(1, 10), (3, 10), (0, 6), (2, 12)])
def test_noalloc_matches_existing_entry_twice(cuda, k, digits):
    torch = cuda
    td = 3 if k >= 2 else 1
    nt, ns = 3001, 5003
    d = W.sphere_ball(ns, nt, k, 40 + k)
    dd = _dev(torch, d)
    ref = _existing(torch, k, dd, digits, nt, ns, td)
    tol = 10.0 ** (-digits) if digits > 6 else 2e-6
    first = _noalloc(torch, k, dd, digits, nt, ns, td)
    second = _noalloc(torch, k, dd, digits, nt, ns, td)
    assert O.rel_l2(first, ref) < tol * 1e-2
    assert O.rel_l2(second, ref) < tol * 1e-2
    np.testing.assert_array_equal(first, second)
    oracle = O.eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    assert O.rel_l2(second, oracle) < tol


def test_noalloc_different_kernels_in_a_row_and_accumulate(cuda):
    torch = cuda
    d1 = W.sphere_ball(2000, 999, 3, 50)
    d0 = W.sphere_ball(7000, 1500, 0, 51)
    dd1, dd0 = _dev(torch, d1), _dev(torch, d0)
    r1 = _existing(torch, 3, dd1, 10, 999, 2000, 3)
    r0 = _existing(torch, 0, dd0, 10, 1500, 7000, 1)
    a = _noalloc(torch, 3, dd1, 10, 999, 2000, 3)
    b = _noalloc(torch, 0, dd0, 10, 1500, 7000, 1)
    c = _noalloc(torch, 3, dd1, 10, 999, 2000, 3)
    assert O.rel_l2(a, r1) < 1e-12 and O.rel_l2(c, r1) < 1e-12 and O.rel_l2(b, r0) < 1e-12
    acc = torch.ones(1500, dtype=torch.float64, device="cuda")
    got = _noalloc(torch, 0, dd0, 10, 1500, 7000, 1, out=acc, flags=capi.ACCUMULATE)
    assert O.rel_l2(got, r0 + 1.0) < 1e-12


def test_noalloc_rejects_oversize_before_launch(cuda):
    torch = cuda
    x = torch.zeros(3, dtype=torch.float64, device="cuda")
    # 2^20 Stokes DxU sources need 80 MiB of packed records: refused, nothing launched
    n0 = capi.launch_count()
    rc = capi.load().sctlgpu_eval_mixed_noalloc(3, 10, 1, x.data_ptr(), 1 << 20, x.data_ptr(), x.data_ptr(),
                                                x.data_ptr(), x.data_ptr(), 0, None)
    assert rc == capi.ERR_TOO_LARGE
    assert capi.launch_count() == n0
    assert capi.load().sctlgpu_eval_mixed_noalloc(9, 10, 1, x.data_ptr(), 1, x.data_ptr(), None, x.data_ptr(),
                                                  x.data_ptr(), 0, None) == capi.ERR_INVALID_KERNEL


@pytest.mark.parametrize("digits", list(range(0, 16)) + [-1])
def test_noalloc_routing_matches_existing_entry_every_digits(cuda, digits):
    """Both entries pick the arithmetic and Newton schedule from one rule: equal results for every digits."""
    torch = cuda
    d = W.sphere_ball(1200, 700, 2, 60)
    dd = _dev(torch, d)
    ref = _existing(torch, 2, dd, digits, 700, 1200, 3)
    got = _noalloc(torch, 2, dd, digits, 700, 1200, 3)
    assert O.rel_l2(got, ref) < 1e-13


def test_noalloc_just_under_the_limit(cuda):
    """2^20 Laplace FxU sources and 2^20 targets: 32 MiB of records plus the partial sums of as many
    source slices as fit in the rest of the 64 MiB array (fewer slices than sctlgpu_eval would use)."""
    torch = cuda
    n = 1 << 20
    d = W.sphere_ball(n, n, 0, 61)
    dd = _dev(torch, d)
    ref = _existing(torch, 0, dd, 10, n, n, 1)
    got = _noalloc(torch, 0, dd, 10, n, n, 1)
    assert O.rel_l2(got, ref) < 1e-12
    # 8 Mi targets: their partial sums alone (one slice, 64 MiB) no longer fit beside the records:
    # refused before anything launches (the buffers are real, so nothing could read out of bounds)
    big_nt = (64 << 20) // 8
    xt = torch.zeros(big_nt * 3, dtype=torch.float64, device="cuda")
    vt = torch.zeros(big_nt, dtype=torch.float64, device="cuda")
    n0 = capi.launch_count()
    rc = capi.load().sctlgpu_eval_mixed_noalloc(0, 10, big_nt, xt.data_ptr(), n, _ptr(dd["r_src"]), None,
                                                _ptr(dd["v_src"]), vt.data_ptr(), 0, None)
    assert rc == capi.ERR_TOO_LARGE and capi.launch_count() == n0
