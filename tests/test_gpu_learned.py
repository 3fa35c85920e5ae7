"""Learned near-singular correction on the torus: trained on the GPU from
adaptive-quadrature labels, it must remove most of the smooth rule's
near-field error at negligible cost (the gain over the method without it),
and with a tight tolerance the disagreement check must hand the pairs back to
the plain path so the result still meets it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained(cuda):
    torch = cuda
    from sctl_gb300.learned import LearnedCorrection, panel_weights
    from sctl_gb300.nearquad import PanelSurface
    from sctl_gb300.torus import Torus, pair_features_device
    T = Torus(seed=0)
    S = PanelSurface(T.X, T.N, T.Q, T.size)
    tg = T.targets(24000, seed=100)
    xt = torch.from_numpy(tg["r_trg"]).cuda().reshape(-1).contiguous()
    pt, pp = S.near_pairs(xt, 1.5)
    W = panel_weights(1, pt, pp, xt, S.X)
    f = pair_features_device(T, xt, pt, pp)
    L = LearnedCorrection(max_batch=8192, singular=T)
    losses = L.fit(f, W, steps=4000, batch=8192, lr=3e-3)
    return torch, T, S, L, losses, (f, W)


def test_training_converged(trained):
    _, _, _, _, losses, _ = trained
    # the standardized MSE of the weights minus their singular part starts near 1.1; training
    # at least halves it
    assert all(l < 0.55 for l in losses), losses


def test_singular_part_sharpens_the_network_near_the_surface(trained):
    """Networks that learn the weights minus their singular part (solid angle x frozen density)
    are far more accurate below 1e-3 panel sizes than networks that learn the weights outright."""
    torch, T, S, L, _, (f, W) = trained
    from sctl_gb300.learned import LearnedCorrection
    L0 = LearnedCorrection(max_batch=8192)
    L0.fit(f, W, steps=4000, batch=8192, lr=3e-3)
    for b in (5, 6, 7):  # |log10 h| bins covering h in [1e-4, 1e-3] panel sizes
        assert L.calib[b] < 0.25 * L0.calib[b], (b, L.calib[b].item(), L0.calib[b].item())


def test_basis_inputs_lower_the_training_loss(trained):
    """Networks that also see the panel's Lagrange bases at the foot point fit the weights
    better than networks on the 15 geometric features alone."""
    torch, T, S, L, losses, (f, W) = trained
    from sctl_gb300.learned import LearnedCorrection
    Lb = LearnedCorrection(max_batch=8192, singular=T, basis_inputs=True)
    lb = Lb.fit(f, W, steps=4000, batch=8192, lr=3e-3)
    assert max(lb) < 0.8 * min(losses), (lb, losses)


def test_checkpoint_round_trip(trained, tmp_path):
    """A trained correction saved and loaded into a fresh object predicts the same weights; a
    checkpoint of another configuration is refused."""
    torch, T, S, L, _, (f, W) = trained
    from sctl_gb300.checkpoint import CheckpointError
    from sctl_gb300.learned import LearnedCorrection
    path = str(tmp_path / "corr.ckpt")
    L.save(path)
    L2 = LearnedCorrection(max_batch=8192, singular=T).load(path)
    x = f[:3000]
    assert torch.equal(L.predict_weights(x), L2.predict_weights(x))
    assert torch.equal(L.calib, L2.calib) and torch.equal(L.calib_sum, L2.calib_sum)
    with pytest.raises(CheckpointError):
        LearnedCorrection(max_batch=8192, singular=T, basis_inputs=True).load(path)


def test_learned_correction_gain_over_smooth_rule(trained):
    torch, T, S, L, _, _ = trained
    from sctl_gb300.learned import learned_near_field
    tg = T.targets(2000, seed=200)
    xt = torch.from_numpy(tg["r_trg"]).cuda()
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    plain = S.evaluate(xt, sig).cpu().numpy()
    smooth = S.far_field(xt.reshape(-1), sig).cpu().numpy()
    st = {}
    learned = learned_near_field(S, T, L, xt, sig, tol=1e30, stats=st).cpu().numpy()
    e_smooth = np.abs(smooth - plain).max()
    e_learned = np.abs(learned - plain).max()
    assert st["accepted"] == st["candidates"] and st["fallback"] == st["pairs"] - st["accepted"]
    assert e_learned < 1e-2 * e_smooth, (e_learned, e_smooth)


def test_tight_tolerance_falls_back_to_plain_path(trained):
    torch, T, S, L, _, _ = trained
    from sctl_gb300.learned import learned_near_field
    tg = T.targets(1000, seed=300)
    xt = torch.from_numpy(tg["r_trg"]).cuda()
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    plain = S.evaluate(xt, sig).cpu().numpy()
    st = {}
    out = learned_near_field(S, T, L, xt, sig, tol=1e-12, stats=st).cpu().numpy()
    assert st["fallback"] >= 0.99 * st["pairs"]
    assert st["inferred"] == 0  # the calibrated bound rules every pair out before any inference
    assert np.abs(out - plain).max() / np.abs(plain).max() < 1e-8


def test_calibrated_gate_bounds_the_error(trained):
    """At a moderate tolerance the accepted pairs' calibrated bounds hold: each target's deviation
    from the plain path stays below tol times its number of accepted pairs."""
    torch, T, S, L, _, _ = trained
    from sctl_gb300.learned import learned_near_field
    tg = T.targets(2000, seed=400)
    xt = torch.from_numpy(tg["r_trg"]).cuda()
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    plain = S.evaluate(xt, sig).cpu().numpy()
    assert L.calib is not None and bool((L.calib > 0).all())
    accepted = {}
    for tol in (1.0, 1e-1, 1e-3):
        st = {}
        out = learned_near_field(S, T, L, xt, sig, tol=tol, stats=st).cpu().numpy()
        dev = np.abs(out - plain)
        n_acc = st["accepted_per_target"].cpu().numpy()
        assert st["accepted"] <= st["inferred"] <= st["candidates"]
        assert np.all(dev <= tol * n_acc + 1e-12 * np.abs(plain).max()), (tol, (dev - tol * n_acc).max())
        accepted[tol] = st["accepted"]
    assert accepted[1.0] > 0 and accepted[1.0] >= accepted[1e-1] >= accepted[1e-3], accepted
