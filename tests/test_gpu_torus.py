"""Near-singular double-layer evaluation on the 64 x 32-panel torus.

Pins: Gauss's law for the double layer (sigma = 1 gives exactly -1 inside the
tube and 0 outside, for the kernel (r.n)/(4 pi r^3) with r = x_t - y and outward
n), self-convergence of the adaptive rule, and the smooth rule for far
targets."""
import numpy as np
import pytest

from sctl_gb300.nearquad import PanelSurface
from sctl_gb300.torus import Torus

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(cuda):
    torch = cuda
    T = Torus(seed=0)
    S = PanelSurface(T.X, T.N, T.Q, T.size)
    return torch, T, S


def test_gauss_law_double_layer(setup):
    torch, T, S = setup
    tg = T.targets(4000, seed=11, hmin=1e-4, hmax=1.0)
    xt = torch.from_numpy(tg["r_trg"]).cuda()
    one = torch.ones(T.np * T.p * T.p, dtype=torch.float64, device="cuda")
    v = S.evaluate(xt, one, kernel=1, mode="mixed", digits=10).cpu().numpy()
    exact = np.where(tg["side"] < 0, -1.0, 0.0)
    err = np.abs(v - exact)
    assert err.max() < 1e-8, (err.max(), tg["h"][err.argmax()])
    from sctl_gb300 import capi
    assert capi.load().sctlgpu_device_status(None) == capi.OK  # no queue overflow / bad index


def test_smooth_rule_alone_is_wrong_near_and_right_far(setup):
    torch, T, S = setup
    far = T.targets(500, seed=12, hmin=2.0, hmax=3.0)
    near = T.targets(500, seed=13, hmin=1e-3, hmax=1e-2)
    one = torch.ones(T.np * T.p * T.p, dtype=torch.float64, device="cuda")
    vf = S.far_field(torch.from_numpy(far["r_trg"]).cuda(), one).cpu().numpy()
    vn = S.far_field(torch.from_numpy(near["r_trg"]).cuda(), one).cpu().numpy()
    ef = np.abs(vf - np.where(far["side"] < 0, -1.0, 0.0))
    en = np.abs(vn - np.where(near["side"] < 0, -1.0, 0.0))
    assert ef.max() < 1e-9
    assert en.max() > 1e-3


def test_self_convergence_fourier_density(setup):
    torch, T, S = setup
    tg = T.targets(2000, seed=14)
    xt = torch.from_numpy(tg["r_trg"]).cuda()
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    a = S.evaluate(xt, sig, alpha=1.0).cpu().numpy()
    b = S.evaluate(xt, sig, alpha=2.0, near_factor=1.5).cpu().numpy()
    assert np.abs(a - b).max() / np.abs(b).max() < 1e-9


def test_green_identity_point_source(setup):
    """Green's representation on the solid torus: for u = 1/|y - x0| with x0 in the hole (harmonic
    inside the tube), SL[du/dn](x) - DL[u](x) = u(x) for targets inside the tube and 0 outside,
    with SL = Laplace3D_FxU and DL = Laplace3D_DxU through the near-singular path (near targets
    at 1e-4 .. 1 panel sizes)."""
    torch, T, S = setup
    x0 = np.array([0.0, 0.05, 0.02])
    Y, Nrm = T.X.reshape(-1, 3), T.N.reshape(-1, 3)
    d = Y - x0
    rr = np.linalg.norm(d, axis=1)
    u = 1.0 / rr
    dudn = -(d * Nrm).sum(1) / rr ** 3
    tg = T.targets(3000, seed=15, hmin=1e-4, hmax=1.0)
    xt = torch.from_numpy(tg["r_trg"]).cuda()
    sl = S.evaluate(xt, torch.from_numpy(dudn).cuda(), kernel=0, mode="mixed", digits=10).cpu().numpy()
    dl = S.evaluate(xt, torch.from_numpy(u).cuda(), kernel=1, mode="mixed", digits=10).cpu().numpy()
    ut = 1.0 / np.linalg.norm(tg["r_trg"] - x0, axis=1)
    exact = np.where(tg["side"] < 0, ut, 0.0)
    err = np.abs(sl - dl - exact) / np.abs(ut).max()
    assert err.max() < 1e-8, (err.max(), tg["h"][err.argmax()], tg["side"][err.argmax()])
