"""The twelve micro-kernels beyond the hot-path four (Laplace gradient / Hessian,
BiotSavart, Helmholtz, Stokes traction / source-sink / pressure) on the GPU,
through the C ABI, against the reference's own Eval / KernelMatrix outputs
(tests/golden/reference_ext.npz) and the oracle."""
import os
import sys

import numpy as np
import pytest

import sctl_gb300 as S
from oracle import oracle as O
from sctl_gb300 import capi

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_ext_golden import KERNELS, MU, ext_case  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_ext.npz"))
NAMES = {v: k for k, v in capi.KERNEL_IDS.items()}


def kern(k):
    return S.GenericKernel(NAMES[k], ctx=MU if k in capi.HELMHOLTZ_IDS else None)


@pytest.mark.parametrize("k", KERNELS)
def test_ext_eval_f64_f32_mixed_match_reference(cuda, k):
    xt, xs, n, f = ext_case(k)
    K = kern(k)
    got = K.Eval(None, xt, xs, n, f, digits=-1, mode="f64")
    assert O.rel_l2(got, GOLDEN[f"{k}/eval_f64"]) < 1e-12
    mixed = K.Eval(None, xt, xs, n, f, digits=10, mode="mixed")  # FP64 path for these kernels
    assert O.rel_l2(mixed, GOLDEN[f"{k}/eval_f64"]) < 1e-10
    g32 = K.Eval(None, xt.astype(np.float32), xs.astype(np.float32), n.astype(np.float32), f.astype(np.float32),
                 digits=-1, mode="f32")
    assert O.rel_l2(g32, GOLDEN[f"{k}/eval_f32"]) < 5e-6
    assert O.rel_l2(g32, GOLDEN[f"{k}/eval_f64"]) < 5e-6
    d6 = K.Eval(None, xt, xs, n, f, digits=6, mode="f64")
    assert O.rel_l2(d6, GOLDEN[f"{k}/eval_f64"]) < 1e-6


@pytest.mark.parametrize("k", KERNELS)
def test_ext_kernel_matrix_matches_reference(cuda, k):
    xt, xs, n, _ = ext_case(k, nt=20, ns=25, seed=1)
    K = kern(k)
    want = GOLDEN[f"{k}/kmat_f64"]
    M = K.KernelMatrix(xt, xs, n, mode="f64")
    assert M.shape == want.shape
    assert np.abs(M - want).max() <= 1e-13 * np.abs(want).max()
    M32 = K.KernelMatrix(xt.astype(np.float32), xs.astype(np.float32), n.astype(np.float32), mode="f32")
    assert np.abs(M32 - want).max() <= 2e-5 * np.abs(want).max()


def test_ext_device_pointers_accumulate_and_large(cuda):
    torch = cuda
    rng = np.random.default_rng(3)
    for k in (5, 8, 11, 14):
        nd, sd, td = O.DIMS[k]
        xs, xt = rng.uniform(-1, 1, (20000, 3)), rng.uniform(-1, 1, (3000, 3))
        n = rng.normal(size=(20000, 3)) if nd else np.zeros((0, 3))
        f = rng.normal(size=20000 * sd)
        ref = O.eval(k, xt, xs, n if nd else None, f, mu=MU)
        d = {a: torch.from_numpy(np.ascontiguousarray(v)).cuda() for a, v in (("xt", xt), ("xs", xs), ("n", n), ("f", f))}
        v0 = torch.ones(3000 * td, dtype=torch.float64, device="cuda")
        out = kern(k).Eval(v0, d["xt"], d["xs"], d["n"], d["f"], digits=-1, mode="f64")
        torch.cuda.synchronize()
        assert out.data_ptr() == v0.data_ptr()  # sized v_trg: added into
        assert O.rel_l2(out.cpu().numpy() - 1.0, ref) < 1e-12
    assert capi.load().sctlgpu_device_status(None) == capi.OK


def test_helmholtz_needs_its_wavenumber(cuda):
    xt, xs, n, f = ext_case(9)
    with pytest.raises(S.SctlGpuError):
        S.GenericKernel("Helmholtz3D_FxU").Eval(None, xt, xs, None, f)
    a = S.GenericKernel("Helmholtz3D_FxU", ctx=MU).Eval(None, xt, xs, None, f)
    b = S.GenericKernel("Helmholtz3D_FxU").SetCtx(0.0).Eval(None, xt, xs, None, f)
    assert O.rel_l2(a, GOLDEN["9/eval_f64"]) < 1e-12
    # mu = 0: the real part is the Laplace single layer, the imaginary part (f_im G0) the same for f_im
    lap = S.Laplace3D_FxU.Eval(None, xt, xs, None, f.reshape(-1, 2)[:, 0].copy())
    assert O.rel_l2(b.reshape(-1, 2)[:, 0], lap) < 1e-12
