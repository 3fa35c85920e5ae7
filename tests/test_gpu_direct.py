"""GPU parity of the direct sums and kernel matrices, through the C ABI,
against the CPU oracle and the reference's golden outputs."""
import json
import math
import os
import threading

import numpy as np
import pytest

import sctl_gb300 as S
from oracle import oracle as O
from sctl_gb300 import capi
from sctl_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NAMES = ["Laplace3D_FxU", "Laplace3D_DxU", "Stokes3D_FxU", "Stokes3D_DxU"]
KER = [S.Laplace3D_FxU, S.Laplace3D_DxU, S.Stokes3D_FxU, S.Stokes3D_DxU]
META = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_eval.json")))
PI = math.pi

# Tolerances (relative l2 against the FP64 oracle / the reference's output):
TOL_F64 = 1e-12          # plain FP64 vs the reference's FP64 Eval
TOL_F32_SMALL = 1e-6     # plain FP32 vs the reference's FP32 Eval, small N
TOL_MIXED = {6: 2e-6, 7: 1e-6, 8: 1e-8, 10: 1e-10, 11: 1e-11, 12: 1e-12}


def case(name, tag):
    c = META["cases"][f"{name}/{tag}"]
    return W.GENERATORS[c["generator"]](c["n_src"], c["n_trg"], NAMES.index(name), c["seed"])


def run(k, d, mode, digits, dtype=np.float64):
    return KER[k].Eval(None, d["r_trg"].astype(dtype), d["r_src"].astype(dtype), d["n_src"].astype(dtype),
                       d["v_src"].astype(dtype), digits=digits, mode=mode)


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("tag", ["ragged", "one_target"])
def test_f64_matches_reference(cuda, golden, k, tag):
    d = case(NAMES[k], tag)
    out = run(k, d, "f64", -1)
    assert O.rel_l2(out, golden[f"{NAMES[k]}/{tag}/eval_f64_d-1"]) < TOL_F64


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("digits", [6, 10])
def test_f64_reduced_digits_within_budget(cuda, golden, k, digits):
    d = case(NAMES[k], "ragged")
    out = run(k, d, "f64", digits)
    assert O.rel_l2(out, golden[f"{NAMES[k]}/ragged/eval_f64_d-1"]) < 10.0 ** (-digits)


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("tag", ["ragged", "one_target"])
def test_f32_matches_reference_f32(cuda, golden, k, tag):
    """FP32 against the reference's FP32 Eval: within 1e-6 wherever the reference's own FP32 sum
    is within 5e-7 of the FP64 result for the same FP32 inputs; and never further from the FP64
    oracle than the reference's FP32 Eval is (both carry their FP32 summation error)."""
    d = case(NAMES[k], tag)
    out = run(k, d, "f32", -1, np.float32)
    assert out.dtype == np.float32
    ref32, ref64 = golden[f"{NAMES[k]}/{tag}/eval_f32"], golden[f"{NAMES[k]}/{tag}/eval_f64_d-1"]
    f64r = O.eval(k, *(np.asarray(d[a], np.float32).astype(np.float64) for a in ("r_trg", "r_src", "n_src", "v_src")))
    if O.rel_l2(ref32, f64r) <= 5e-7:
        assert O.rel_l2(out, ref32) < TOL_F32_SMALL
    assert O.rel_l2(out, ref64) <= max(1.5 * O.rel_l2(ref32, ref64), TOL_F32_SMALL)


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("digits", sorted(TOL_MIXED))
def test_mixed_meets_digits(cuda, golden, k, digits):
    d = case(NAMES[k], "ragged")
    out = run(k, d, "mixed", digits)
    assert out.dtype == np.float64
    assert O.rel_l2(out, golden[f"{NAMES[k]}/ragged/eval_f64_d-1"]) < TOL_MIXED[digits]


@pytest.mark.parametrize("k", range(4))
def test_small_deterministic_eval_and_matrix(cuda, golden, k):
    name = NAMES[k]
    Xt, Xs, Xn, Vs = (golden[f"{name}/small/{a}"] for a in ("Xt", "Xs", "Xn", "Vs"))
    for mode, tol in (("f64", 1e-13), ("mixed", 1e-11)):
        v = KER[k].Eval(None, Xt, Xs, Xn, Vs, mode=mode, digits=-1 if mode == "f64" else 12)
        assert O.rel_l2(v, golden[f"{name}/small/eval_f64"]) < tol
        M = KER[k].KernelMatrix(Xt, Xs, Xn, mode=mode, digits=-1 if mode == "f64" else 12)
        assert M.shape == golden[f"{name}/small/kmat_f64"].shape
        assert O.rel_l2(M, golden[f"{name}/small/kmat_f64"]) < tol
        # Eval == KernelMatrix applied to the densities (test-kernel_functions.cpp:487-526)
        np.testing.assert_allclose(v, Vs @ M, rtol=1e-10, atol=1e-12)
    M32 = KER[k].KernelMatrix(Xt.astype(np.float32), Xs.astype(np.float32), Xn.astype(np.float32))
    assert M32.dtype == np.float32 and O.rel_l2(M32, golden[f"{name}/small/kmat_f64"]) < 1e-6


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("mode", ["f64", "f32", "mixed"])
def test_kernel_matrix_matches_reference(cuda, golden, k, mode):
    d = case(NAMES[k], "kmat40x50")
    dt = np.float32 if mode == "f32" else np.float64
    M = KER[k].KernelMatrix(d["r_trg"].astype(dt), d["r_src"].astype(dt), d["n_src"].astype(dt), mode=mode,
                            digits=-1 if mode != "mixed" else 12)
    assert O.rel_l2(M, golden[f"{NAMES[k]}/kmat40x50/kmat_f64"]) < (1e-6 if mode == "f32" else 1e-12)


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("digits", [6, 10, 11])
def test_kernel_matrix_mixed_double_float(cuda, golden, k, digits):
    """Mixed KernelMatrix at digits <= 11: double-float entries rounded to FP64 by integer
    operations.  Against the reference's FP64 matrix, a larger FP64 matrix entry by entry, and
    zero entries for coincident points (r = 0)."""
    d = case(NAMES[k], "kmat40x50")
    M = KER[k].KernelMatrix(d["r_trg"], d["r_src"], d["n_src"], mode="mixed", digits=digits)
    assert O.rel_l2(M, golden[f"{NAMES[k]}/kmat40x50/kmat_f64"]) < 1e-12
    e = W.sphere_ball(700, 300, k, seed=21)
    xt = np.concatenate([e["r_trg"], e["r_src"][:5]])  # 5 targets on top of sources
    M = KER[k].KernelMatrix(xt, e["r_src"], e["n_src"], mode="mixed", digits=digits)
    M64 = KER[k].KernelMatrix(xt, e["r_src"], e["n_src"], mode="f64")
    assert np.abs(M - M64).max() <= 1e-12 * np.abs(M64).max()
    k0, k1 = O.DIMS[k][1], O.DIMS[k][2]
    for i in range(5):  # source i coincides with target 300 + i
        blk = M[i * k0:(i + 1) * k0, (300 + i) * k1:(301 + i) * k1]
        assert np.all(blk == 0.0)


def test_cube8192_f64_digits14(cuda, golden):
    d = W.cube(8192, 8192, 0, 0)
    out = run(0, d, "f64", 14)
    assert O.rel_l2(out, golden["Laplace3D_FxU/cube8192/eval_f64_d14"]) < TOL_F64


def test_known_answers(cuda):
    """The reference's analytic single-pair tests (src/test-kernel_functions.cpp:36-132), tol 1e-9."""
    z = np.zeros(0)
    for mode in ("f64", "mixed"):
        v = S.Laplace3D_FxU.Eval(None, np.array([2.0, 0, 0]), np.zeros(3), z, np.array([3.0]), mode=mode)
        assert abs(v[0] - 3.0 / (4 * PI * 2.0)) < 1e-9
        v = S.Laplace3D_DxU.Eval(None, np.array([2.0, 0, 0]), np.zeros(3), np.array([1.0, 0, 0]), np.array([1.0]),
                                 mode=mode)
        assert abs(v[0] - 1.0 / (16 * PI)) < 1e-9
        v = S.Stokes3D_FxU.Eval(None, np.array([2.0, 0, 0]), np.zeros(3), z, np.array([1.0, 0, 0]), mode=mode)
        assert abs(v[0] - 1.0 / (4 * PI * 2.0)) < 1e-9 and abs(v[1]) < 1e-12 and abs(v[2]) < 1e-12
        v = S.Stokes3D_DxU.Eval(None, np.array([3.0, 0, 0]), np.zeros(3), np.array([0, 1.0, 0]),
                                np.array([1.0, 0, 0]), mode=mode)
        assert v.shape == (3,)
        v = S.Laplace3D_FxU.Eval(None, np.array([1.0, 0, 0, 2, 0, 0, 3, 0, 0, 5, 0, 0]), np.zeros(3), z,
                                 np.array([1.0]), mode=mode)
        np.testing.assert_allclose(v, [1 / (4 * PI * r) for r in (1, 2, 3, 5)], rtol=1e-9)


@pytest.mark.parametrize("mode", ["f64", "f32", "mixed"])
@pytest.mark.parametrize("k", range(4))
def test_self_interaction_masked(cuda, mode, k):
    """A target sitting exactly on a source gets nothing from it (r^2 == 0 mask)."""
    d = W.sphere_ball(257, 33, k, 21)
    d["r_trg"][:10] = d["r_src"][5:15]
    dt = np.float32 if mode == "f32" else np.float64
    out = run(k, d, mode, -1 if mode != "mixed" else 10, dt)
    assert np.all(np.isfinite(out))
    ref = O.eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    # FP32: neighbours of an on-surface target cancel in r.n, so FP32 keeps ~1e-5 here
    assert O.rel_l2(out, ref) < (1e-4 if mode == "f32" else 1e-10)


@pytest.mark.parametrize("mode", ["f64", "mixed"])
def test_accumulate_and_reinit_semantics(cuda, mode):
    d = W.sphere_ball(500, 70, 2, 4)
    a = run(2, d, mode, 12)
    v = np.ones(70 * 3)
    out = S.Stokes3D_FxU.Eval(v, d["r_trg"], d["r_src"], d["n_src"], d["v_src"], digits=12, mode=mode)
    assert out is v
    np.testing.assert_allclose(v, a + 1.0, rtol=1e-11, atol=1e-13)
    wrong = np.ones(5)
    out2 = S.Stokes3D_FxU.Eval(wrong, d["r_trg"], d["r_src"], d["n_src"], d["v_src"], digits=12, mode=mode)
    assert out2.shape == (210,)
    np.testing.assert_allclose(out2, a, rtol=1e-12)


def test_empty_inputs(cuda):
    v = S.Laplace3D_FxU.Eval(None, np.zeros((4, 3)), np.zeros((0, 3)), None, np.zeros(0))
    assert v.shape == (4,) and np.all(v == 0)
    v = np.full(4, 2.0)
    S.Laplace3D_FxU.Eval(v, np.zeros((4, 3)), np.zeros((0, 3)), None, np.zeros(0))
    assert np.all(v == 2.0)
    v = S.Laplace3D_FxU.Eval(None, np.zeros((0, 3)), np.ones((3, 3)), None, np.ones(3))
    assert v.shape == (0,)


@pytest.mark.parametrize("k", range(4))
def test_device_pointer_path(cuda, k):
    torch = cuda
    d = W.sphere_ball(3000, 1111, k, 8)
    ref = O.eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    dev = {a: torch.from_numpy(np.ascontiguousarray(v)).cuda() for a, v in d.items()}
    out = KER[k].Eval(None, dev["r_trg"], dev["r_src"], dev["n_src"], dev["v_src"], digits=10, mode="mixed")
    torch.cuda.synchronize()
    assert O.rel_l2(out.cpu().numpy(), ref) < 1e-10
    acc = out.clone()
    KER[k].Eval(acc, dev["r_trg"], dev["r_src"], dev["n_src"], dev["v_src"], digits=-1, mode="f64")
    torch.cuda.synchronize()
    assert O.rel_l2(acc.cpu().numpy(), 2 * ref) < 1e-10
    assert capi.load().sctlgpu_device_status(None) == capi.OK


def test_concurrent_host_threads(cuda):
    """Re-entrant from several host threads (BIO calls KernelMatrix inside an OpenMP region)."""
    d = W.sphere_ball(2000, 300, 1, 9)
    ref = O.eval(1, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    errs = []

    def work():
        for _ in range(5):
            out = run(1, d, "mixed", 10)
            errs.append(O.rel_l2(out, ref))

    th = [threading.Thread(target=work) for _ in range(6)]
    [t.start() for t in th]
    [t.join() for t in th]
    assert len(errs) == 30 and max(errs) < 1e-10


@pytest.mark.parametrize("k", [0, 3])
def test_large_sources_subset_of_targets(cuda, k):
    """2^20 sources (the sphere/ball workload's source count) against a target subset, vs the oracle."""
    d = W.sphere_ball(1 << 20, 256, k, 0)
    ref = O.eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    for mode, digits, tol in (("mixed", 10, 1e-10), ("f64", -1, 1e-12), ("mixed", 6, 2e-6)):
        assert O.rel_l2(run(k, d, mode, digits), ref) < tol


def test_packed_records_beyond_2gib(cuda):
    """2^25 Stokes3D_DxU sources: the packed double-float records (80 B each, 2.7 GB) and the FP64
    records are addressed past 2^31 bytes; 64-bit offsets in the pack, tile and slice arithmetic."""
    torch = cuda
    k, ns, nt = 3, 1 << 25, 96
    rng = np.random.default_rng(21)
    xs = rng.normal(size=(ns, 3))
    xs /= np.linalg.norm(xs, axis=1, keepdims=True)
    xt = rng.uniform(-1.5, 1.5, (nt, 3))
    f = rng.normal(size=ns * 3)
    dev = [torch.from_numpy(np.ascontiguousarray(a).reshape(-1)).cuda() for a in (xt, xs, xs, f)]
    ref = O.eval(k, xt[:16], xs, xs, f)
    for mode, digits, tol in (("mixed", 10, 1e-10), ("f64", -1, 1e-12)):
        out = S.Stokes3D_DxU.Eval(None, dev[0], dev[1], dev[2], dev[3], digits=digits, mode=mode)
        torch.cuda.synchronize()
        assert O.rel_l2(out.cpu().numpy()[:16 * 3], ref) < tol, mode
    del dev
    torch.cuda.empty_cache()


@pytest.mark.parametrize("k", [0, 2])
def test_clusters_precision_stress(cuda, k):
    d = W.clusters(1 << 14, 512, k, 0)
    ref = O.eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"], precision="ld")
    for digits in (8, 10, 11, 12):
        assert O.rel_l2(run(k, d, "mixed", digits), ref) < 10.0 ** (-digits) * 2


def test_linearity_full_size_property(cuda):
    """Size-independent property at 2^18 x 2^18: Eval is linear in the densities."""
    torch = cuda
    d = W.sphere_ball(1 << 18, 1 << 18, 3, 2)
    dev = {a: torch.from_numpy(np.ascontiguousarray(v)).cuda() for a, v in d.items()}
    f2 = torch.randn_like(dev["v_src"])
    a = S.Stokes3D_DxU.Eval(None, dev["r_trg"], dev["r_src"], dev["n_src"], dev["v_src"], digits=10, mode="mixed")
    b = S.Stokes3D_DxU.Eval(None, dev["r_trg"], dev["r_src"], dev["n_src"], f2, digits=10, mode="mixed")
    c = S.Stokes3D_DxU.Eval(None, dev["r_trg"], dev["r_src"], dev["n_src"], 2 * dev["v_src"] - 3 * f2, digits=10,
                            mode="mixed")
    torch.cuda.synchronize()
    lhs, rhs = c.cpu().numpy(), (2 * a - 3 * b).cpu().numpy()
    assert O.rel_l2(lhs, rhs) < 1e-10


def test_launch_count_and_timing(cuda):
    d = W.sphere_ball(4096, 4096, 0, 1)
    n0 = capi.launch_count()
    capi.set_timing(True)
    run(0, d, "mixed", 10)
    ms = capi.last_kernel_ms()
    capi.set_timing(False)
    assert capi.launch_count() - n0 >= 3
    assert ms > 0
