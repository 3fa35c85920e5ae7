"""Pins the CPU oracle (oracle/sctl_oracle.c) to the reference: golden outputs of
the reference's own Eval/KernelMatrix (tests/golden, made by make_golden.py)
and the reference's known-answer tests."""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from sctl_gb300 import workloads as W

NAMES = ["Laplace3D_FxU", "Laplace3D_DxU", "Stokes3D_FxU", "Stokes3D_DxU"]
META = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_eval.json")))
PI = math.pi


def case_inputs(name, tag):
    c = META["cases"][f"{name}/{tag}"]
    k = NAMES.index(name)
    return W.GENERATORS[c["generator"]](c["n_src"], c["n_trg"], k, c["seed"])


@pytest.mark.parametrize("k", range(4))
def test_small_deterministic_eval_and_matrix(golden, k):
    name = NAMES[k]
    Xt, Xs, Xn, Vs = (golden[f"{name}/small/{a}"] for a in ("Xt", "Xs", "Xn", "Vs"))
    assert O.rel_l2(O.eval(k, Xt, Xs, Xn, Vs), golden[f"{name}/small/eval_f64"]) < 1e-14
    assert O.rel_l2(O.kernel_matrix(k, Xt, Xs, Xn), golden[f"{name}/small/kmat_f64"]) < 1e-14
    f32 = O.eval(k, Xt.astype(np.float32), Xs.astype(np.float32), Xn.astype(np.float32), Vs.astype(np.float32),
                 precision="f32")
    assert O.rel_l2(f32, golden[f"{name}/small/eval_f32"]) < 1e-6


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("tag", ["ragged", "one_target"])
def test_seeded_eval_matches_reference(golden, k, tag):
    name = NAMES[k]
    d = case_inputs(name, tag)
    mine = O.eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    assert O.rel_l2(mine, golden[f"{name}/{tag}/eval_f64_d-1"]) < 1e-14
    # the reference's reduced-digits results sit within their digit budget of the oracle
    for digits in (6, 10):
        assert O.rel_l2(golden[f"{name}/{tag}/eval_f64_d{digits}"], mine) < 10.0 ** (-digits)
    mine32 = O.eval(k, *(d[a].astype(np.float32) for a in ("r_trg", "r_src", "n_src", "v_src")), precision="f32")
    assert O.rel_l2(mine32, golden[f"{name}/{tag}/eval_f32"]) < 2e-6


@pytest.mark.parametrize("k", range(4))
def test_kernel_matrix_matches_reference(golden, k):
    d = case_inputs(NAMES[k], "kmat40x50")
    M = O.kernel_matrix(k, d["r_trg"], d["r_src"], d["n_src"])
    assert O.rel_l2(M, golden[f"{NAMES[k]}/kmat40x50/kmat_f64"]) < 1e-14


def test_cube8192_digits14(golden):
    d = W.cube(8192, 8192, 0, 0)
    mine = O.eval(0, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    assert O.rel_l2(mine, golden["Laplace3D_FxU/cube8192/eval_f64_d14"]) < 1e-13


# --- the reference's known-answer tests (src/test-kernel_functions.cpp:36-132,
# src/test-generic-kernel.cpp:55-103), tolerance 1e-9 as there.
def test_known_answers():
    z = np.zeros(0)
    v = O.eval(0, [2, 0, 0], [0, 0, 0], z, [3.0])
    assert abs(v[0] - 3.0 / (4 * PI * 2.0)) < 1e-9
    v = O.eval(1, [2, 0, 0], [0, 0, 0], [1, 0, 0], [1.0])
    assert abs(v[0] - 1.0 / (16 * PI)) < 1e-9
    v = O.eval(2, [2, 0, 0], [0, 0, 0], z, [1.0, 0, 0])
    assert abs(v[0] - 1.0 / (4 * PI * 2.0)) < 1e-9 and abs(v[1]) < 1e-12 and abs(v[2]) < 1e-12
    v = O.eval(3, [3, 0, 0], [0, 0, 0], [0, 1, 0], [1.0, 0, 0])
    assert v.shape == (3,)
    M = O.kernel_matrix(0, [1, 0, 0], [0, 0, 0], z)
    assert M.shape == (1, 1) and abs(M[0, 0] - 1 / (4 * PI)) < 1e-9
    v = O.eval(0, [1, 0, 0, 2, 0, 0, 3, 0, 0, 5, 0, 0], [0, 0, 0], z, [1.0])
    np.testing.assert_allclose(v, [1 / (4 * PI * r) for r in (1, 2, 3, 5)], rtol=1e-9)
    v = O.eval(0, [2, 0, 0], [0, 0, 0, 4, 0, 0], z, [1.0, 1.0])
    assert abs(v[0] - 2 * (1 / (4 * PI * 2))) < 1e-9


def test_self_interaction_is_masked():
    v = O.eval(0, [0.5, 0.5, 0.5], [0.5, 0.5, 0.5, 1.5, 0.5, 0.5], np.zeros(0), [7.0, 1.0])
    assert abs(v[0] - 1 / (4 * PI)) < 1e-15


def test_eval_accumulates():
    d = W.cube(50, 20, 0, 1)
    a = O.eval(0, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    b = O.eval(0, d["r_trg"], d["r_src"], d["n_src"], d["v_src"], v_trg=a.copy())
    np.testing.assert_allclose(b, 2 * a, rtol=1e-15)


@pytest.mark.parametrize("k", range(4))
def test_eval_equals_matrix_apply(k):
    """Eval vs KernelMatrix on the reference test's 7x5 inputs (test-kernel_functions.cpp:487-526)."""
    nd, sd, td = O.DIMS[k]
    Xs = np.array([0.1 * (i + 1) - 0.35 for i in range(7 * 3)])
    Vs = np.array([0.3 * (i % 5) - 0.4 for i in range(7 * sd)])
    Xt = np.array([1.7 + 0.2 * i for i in range(5 * 3)])
    Xn = np.tile([0.0, 1.0, 0.0], 7) if nd else np.zeros(0)
    v = O.eval(k, Xt, Xs, Xn, Vs)
    M = O.kernel_matrix(k, Xt, Xs, Xn)
    np.testing.assert_allclose(v, Vs @ M, rtol=1e-10, atol=1e-12)


def test_newton_schedule_matches_reference_table():
    # AVX-512 rsqrt14 (4.2144 digits): <=4 -> 0, 5-8 -> 1, 9-16 -> 2  (intrin-wrapper.hpp:3384)
    assert [O.newton_steps(d, 1, 4.2144199393) for d in (3, 4, 5, 8, 9, 15)] == [0, 0, 1, 1, 2, 2]
    # 12-bit rsqrtps / NEON: <=3 -> 0, 4-6 -> 1, 7-13 -> 2, 14+ -> 3 (:1566)
    assert [O.newton_steps(d, 1, 3.4362686889) for d in (3, 4, 6, 7, 13, 14)] == [0, 1, 1, 2, 2, 3]
    assert O.newton_steps(-1, 1, 3.4362686889) == 3 and O.newton_steps(-1, 0, 3.4362686889) == 1


@pytest.mark.parametrize("steps", [1, 2, 3])
def test_deferred_scaling_newton_equals_plain_newton(steps):
    rng = np.random.default_rng(5)
    for x in rng.uniform(1e-3, 1e3, 50):
        y0 = (1.0 / math.sqrt(x)) * (1 + 2.0 ** -12)
        y = y0
        for _ in range(steps):
            y = y * (1.5 - 0.5 * x * y * y)
        assert abs(O.rsqrt_newton(x, y0, steps) - y) <= 4e-16 * y
    assert O.rsqrt_newton(0.0, 1.0, 2) == 0.0
