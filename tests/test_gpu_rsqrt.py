"""Seed accuracy of sm_103a's rsqrt.approx.{f32,f64} as the kernels use it
(KernelMatrix of Laplace3D_FxU at digits 6 runs zero Newton steps), and the
reference's rsqrt contract (vec-test.hpp:431-465): digits 4 -> rel err < 2^-11,
digits 7 -> < 2^-22, masked lanes exactly 0."""
import math

import numpy as np
import pytest

import sctl_gb300 as S
from sctl_gb300 import capi

pytestmark = pytest.mark.gpu

# Measured on GB300: 2^-22.28 (f32) and 2^-20.1 (f64, MUFU.RSQ64H); the library's
# Newton schedule uses these (less log10 5 for r^-5).
SEED_BOUND = {"f32": 2.0 ** -22.0, "f64": 2.0 ** -20.0}


def pair_values(mode, digits, r):
    """scale/r for each distance r via a 1-source x n-target kernel matrix."""
    dt = np.float32 if mode == "f32" else np.float64
    xt = np.zeros((r.size, 3))
    xt[:, 0] = r
    M = S.Laplace3D_FxU.KernelMatrix(xt.astype(dt), np.zeros(3, dt), None, digits=digits, mode=mode)
    return np.asarray(M, np.float64).reshape(-1) * (4 * math.pi)


@pytest.mark.parametrize("mode", ["f32", "f64"])
def test_seed_accuracy(cuda, mode):
    rng = np.random.default_rng(0)
    r = np.exp(rng.uniform(math.log(1e-3), math.log(1e3), 200000))
    if mode == "f32":
        r = r.astype(np.float32).astype(np.float64)
    got = pair_values(mode, 6 if mode == "f64" else 5, r)
    exact = 1.0 / r
    err = np.max(np.abs(got - exact) / exact)
    print(f"rsqrt.approx seed ({mode}): max rel err {err:.3e} = 2^{math.log2(err):.2f}")
    assert err < SEED_BOUND[mode]


@pytest.mark.parametrize("digits,bound", [(4, 2.0 ** -11), (7, 2.0 ** -22), (10, 1e-10), (14, 1e-14)])
def test_reference_rsqrt_contract_f64(cuda, digits, bound):
    rng = np.random.default_rng(1)
    r = np.sqrt(rng.uniform(1.0, 2.0 ** 31, 50000))  # rand()-range squares as in vec-test.hpp
    got = pair_values("f64", digits, r)
    err = np.max(np.abs(got - 1.0 / r) * r)
    assert err < bound
    assert capi.newton_steps("f64", digits) == (0 if digits <= 5 else 1 if digits <= 10 else 2)


def test_masked_pair_is_exactly_zero(cuda):
    for mode in ("f32", "f64", "mixed"):
        assert pair_values(mode, -1, np.array([0.0, 1.0]))[0] == 0.0
