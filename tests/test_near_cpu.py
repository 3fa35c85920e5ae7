"""Plan creation rejects malformed block tables before touching a device."""
import ctypes

import numpy as np

from sctl_gb300 import capi
from sctl_gb300 import workloads as W


def create(blocks, ns, nt, kernel=1, mode=capi.MIXED, tmap=None, n_out=-1):
    h = ctypes.c_void_p()
    b = np.ascontiguousarray(blocks, np.int64).reshape(-1, 4)
    tm = None if tmap is None else np.ascontiguousarray(tmap, np.int64)
    return capi.load().sctlgpu_near_plan_create(ctypes.byref(h), kernel, mode, -1, b.shape[0], b.ctypes.data, ns, nt,
                                               None if tm is None else tm.ctypes.data, n_out)


def test_invalid_blocks_rejected():
    assert create([[0, 5, 0, 3]], 4, 3) == capi.ERR_INVALID_SIZE          # sources past the end
    assert create([[0, 4, 2, 3]], 4, 3) == capi.ERR_INVALID_SIZE          # targets past the end
    assert create([[0, -1, 0, 3]], 4, 3) == capi.ERR_INVALID_SIZE
    assert create([[0, 4, 0, 3]], 4, 3, kernel=9) == capi.ERR_INVALID_KERNEL
    assert create([[0, 4, 0, 3]], 4, 3, mode=7) == capi.ERR_INVALID_MODE
    assert create([[0, 4, 0, 3]], 4, 3, tmap=[0, 1, 5], n_out=3) == capi.ERR_INVALID_ARGUMENT
    assert create([[0, 4, 0, 3]], 4, 3, mode=capi.F32, tmap=[0, 1, 2], n_out=3) == capi.ERR_INVALID_ARGUMENT


def test_near_blocks_generator_shapes():
    d = W.near_blocks(64, 1, seed=0)
    b = d["blocks"]
    assert b.shape == (64, 4)
    assert b[:, 1].min() >= 100 and b[:, 1].max() <= 6400 and b[:, 3].min() >= 16 and b[:, 3].max() <= 2048
    assert d["r_src"].shape[0] == b[:, 1].sum() and d["r_trg"].shape[0] == b[:, 3].sum()
    assert np.all(b[1:, 0] == np.cumsum(b[:, 1])[:-1])
    p = W.near_blocks(16, 0, seed=1, panel=True)
    assert set(np.unique(p["blocks"][:, 1])) <= {100 * k * k for k in range(1, 9)}


def test_torus_pair_features_device_form_matches_numpy():
    """The torch form of the learned path's pair features (run where the pairs live) equals the
    numpy form used to define them."""
    import torch
    from sctl_gb300.torus import Torus, pair_features, pair_features_device
    T = Torus(seed=0)
    tg = T.targets(1500, seed=5)
    pt, pp = T.near_pairs(tg["r_trg"], 1.0)
    a = pair_features(T, tg["r_trg"], pt, pp)
    b = pair_features_device(T, torch.from_numpy(tg["r_trg"]).reshape(-1), torch.from_numpy(pt),
                             torch.from_numpy(pp)).numpy()
    assert a.shape == b.shape == (pt.size, 15)
    assert np.abs(a - b).max() < 1e-12


def test_torus_chebyshev_rule_and_interpolation():
    """The torus panels' 1-D rule is ChebQuadRule's (quadrule.txx:71-101): its 10 weights integrate
    x^k on [0, 1] exactly for k <= 9; the barycentric Lagrange matrix reproduces the nodes and
    interpolates degree-9 polynomials exactly."""
    from sctl_gb300.torus import cheb_bary_weights, cheb_rule, lagrange_matrix
    x, w = cheb_rule(10)
    for k in range(10):
        assert abs((w * x ** k).sum() - 1.0 / (k + 1)) < 1e-15
    bw = cheb_bary_weights(10)
    assert np.array_equal(lagrange_matrix(x, bw, x), np.eye(10))
    y = np.linspace(-0.2, 1.2, 37)
    c = np.random.default_rng(0).standard_normal(10)
    np.testing.assert_allclose(lagrange_matrix(x, bw, y) @ np.polyval(c, x), np.polyval(c, y), rtol=0, atol=1e-11)


def test_torus_singular_part_limits():
    """The learned path's singular part: the double layer's +-1/2 jump for targets just above and
    below a panel's interior (bases summing to one), the solid-angle fade-out far away, and its
    dot product equal to the explicit weights."""
    import torch
    from sctl_gb300.torus import Torus, pair_features_device, singular_dot, singular_weights
    T = Torus(seed=0)
    tg = T.targets(400, seed=3, hmin=1e-5, hmax=1e-5)
    pt = torch.arange(400)
    pp = torch.from_numpy(tg["panel"])
    f = pair_features_device(T, torch.from_numpy(tg["r_trg"]), pt, pp)
    inside = ((f[:, 0] > 0.05) & (f[:, 0] < 0.95) & (f[:, 1] > 0.05) & (f[:, 1] < 0.95)).numpy()
    J = singular_weights(T, f).numpy()
    side = tg["side"]
    np.testing.assert_allclose(J.sum(1)[inside], 0.5 * side[inside], atol=2e-3)
    far = T.targets(50, seed=4, hmin=0.9, hmax=0.9)
    ff = pair_features_device(T, torch.from_numpy(far["r_trg"]), torch.arange(50), torch.from_numpy(far["panel"]))
    assert np.abs(singular_weights(T, ff).numpy()).sum(1).max() < 0.05
    sig = torch.from_numpy(T.sigma)
    np.testing.assert_allclose(singular_dot(T, f, sig, pp).numpy(), (J * T.sigma[tg["panel"]]).sum(1), atol=1e-14)
