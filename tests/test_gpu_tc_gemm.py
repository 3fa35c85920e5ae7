"""tcgen05 BF16 GEMM (FP32 accumulation in tensor memory) against a torch FP32
reference on the same BF16-rounded inputs."""
import math

import pytest

from sctl_gb300 import capi

pytestmark = pytest.mark.gpu


def gemm(torch, A, Bt, bias=None, act=0, c32=True, pre=False, c16=False):
    M, K = A.shape
    N = Bt.shape[0]
    C32 = torch.full((M, N), float("nan"), device="cuda") if c32 else None
    P32 = torch.full((M, N), float("nan"), device="cuda") if pre else None
    C16 = torch.zeros((M, N), dtype=torch.bfloat16, device="cuda") if c16 else None
    p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    rc = capi.load().sctlgpu_tc_gemm_bf16(M, N, K, A.data_ptr(), Bt.data_ptr(), p(bias), act, p(C32), p(P32), p(C16),
                                          0, torch.cuda.current_stream().cuda_stream)
    assert rc == capi.OK, capi.load().sctlgpu_strerror(rc)
    torch.cuda.synchronize()
    return C32, P32, C16


def ref(torch, A, Bt, bias, act):
    x = A.float() @ Bt.float().T
    if bias is not None:
        x = x + bias
    pre = x.clone()
    if act:
        x = 0.5 * x * (1 + torch.tanh(math.sqrt(2 / math.pi) * (x + 0.044715 * x ** 3)))
    return x, pre


@pytest.mark.parametrize("M,N,K", [(128, 16, 64), (128, 256, 64), (256, 96, 128), (384, 112, 256)])
def test_tc_gemm_matches_fp32_reference(cuda, M, N, K):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    Bt = (torch.randn(N, K, device="cuda", generator=g) / math.sqrt(K)).to(torch.bfloat16)
    C32, _, _ = gemm(torch, A, Bt)
    want, _ = ref(torch, A, Bt, None, 0)
    err = ((C32 - want).abs().max() / want.abs().max()).item()
    assert err < 1e-5, err


def test_tc_gemm_bias_gelu_outputs(cuda):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(7)
    A = torch.randn(256, 128, device="cuda", generator=g).to(torch.bfloat16)
    Bt = (torch.randn(256, 128, device="cuda", generator=g) / 11).to(torch.bfloat16)
    bias = torch.randn(256, device="cuda", generator=g)
    C32, P32, C16 = gemm(torch, A, Bt, bias, act=1, pre=True, c16=True)
    want, pre = ref(torch, A, Bt, bias, 1)
    assert ((P32 - pre).abs().max() / pre.abs().max()).item() < 1e-5
    assert ((C32 - want).abs().max() / want.abs().max()).item() < 1e-5
    assert ((C16.float() - want).abs().max() / want.abs().max()).item() < 1e-2
    assert capi.load().sctlgpu_device_status(None) == capi.OK


def test_tc_gemm_rejects_bad_shapes(cuda):
    torch = cuda
    A = torch.zeros(100, 64, dtype=torch.bfloat16, device="cuda")
    assert capi.load().sctlgpu_tc_gemm_bf16(100, 16, 64, A.data_ptr(), A.data_ptr(), None, 0, A.data_ptr(), None,
                                            None, 0, None) == capi.ERR_INVALID_SIZE


@pytest.mark.parametrize("M,N,K,acc", [(512, 256, 4096, 0), (256, 64, 16384, 0), (128, 128, 8192, 1),
                                       (1024, 16, 640, 0)])
def test_tc_gemm_ring_wraparound_and_split_k(cuda, M, N, K, acc):
    """Many more K chunks than ring stages (the producer waits for stages the MMAs released),
    and small-M plain FP32 outputs that take the split-K path (partials reduced in slice order),
    with and without accumulation into C."""
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    Bt = (torch.randn(N, K, device="cuda", generator=g) / math.sqrt(K)).to(torch.bfloat16)
    C0 = torch.randn(M, N, device="cuda", generator=g)
    C = C0.clone()
    rc = capi.load().sctlgpu_tc_gemm_bf16(M, N, K, A.data_ptr(), Bt.data_ptr(), None, 0, C.data_ptr(), None, None,
                                          acc, torch.cuda.current_stream().cuda_stream)
    assert rc == capi.OK, capi.load().sctlgpu_strerror(rc)
    torch.cuda.synchronize()
    want = A.float() @ Bt.float().T + (C0 if acc else 0)
    err = ((C - want).abs().max() / want.abs().max()).item()
    assert err < 1e-5, err
    assert capi.load().sctlgpu_device_status(None) == capi.OK


def test_tc_gemm_rejects_misaligned_outputs(cuda):
    torch = cuda
    A = torch.zeros(128, 64, dtype=torch.bfloat16, device="cuda")
    Bt = torch.zeros(16, 64, dtype=torch.bfloat16, device="cuda")
    C = torch.zeros(128 * 16 + 4, device="cuda")
    rc = capi.load().sctlgpu_tc_gemm_bf16(128, 16, 64, A.data_ptr(), Bt.data_ptr(), None, 0, C.data_ptr() + 4, None,
                                          None, 0, None)
    assert rc == capi.ERR_INVALID_ARGUMENT
