"""The near-field correction network on the tcgen05 kernels: forward and
gradients against a numpy FP64 restatement of the same network (same
BF16-rounded weights, inputs and inter-layer activations), Adam training,
the fused weight.density epilogue, and the label (weights-mode) quadrature."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C = math.sqrt(2 / math.pi)


def bf16(torch, a):
    return torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16).float().numpy().astype(np.float64)


def gelu(x):
    return 0.5 * x * (1 + np.tanh(C * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C * (x + 0.044715 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * C * (1 + 3 * 0.044715 * x * x)


def ref_forward(torch, layers, x):
    a = bf16(torch, np.pad(x, ((0, 0), (0, 64 - x.shape[1]))))
    zs, hs = [], [a]
    for li, (W, b) in enumerate(layers):
        z = a @ bf16(torch, W).T + b
        if li < 3:
            zs.append(z)
            a = bf16(torch, gelu(z))
            hs.append(a)
        else:
            y = z
    return y, zs, hs


def ref_grads(torch, layers, x, t, out_dim):
    y, zs, hs = ref_forward(torch, layers, x)
    B = x.shape[0]
    d = np.zeros_like(y)
    d[:, :out_dim] = 2 * (y[:, :out_dim] - t) / (B * out_dim)
    grads = [None] * 4
    dcur = bf16(torch, d)
    grads[3] = (dcur.T @ hs[3], d.sum(0))
    for l in (2, 1, 0):
        dh = dcur @ bf16(torch, layers[l + 1][0])
        g = dh * gelu_grad(zs[l])
        dz = bf16(torch, g)
        grads[l] = (dz.T @ hs[l], g.sum(0))
        dcur = dz
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    loss = np.mean((y[:, :out_dim] - t) ** 2)
    return flat, loss, y


@pytest.fixture(scope="module")
def mlp(cuda):
    from sctl_gb300.learned import MLP
    return MLP(in_dim=15, out_dim=100, max_batch=1024, seed=3)


def test_forward_matches_fp64_restatement(cuda, mlp):
    torch = cuda
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (256, 15)).astype(np.float32)
    y = mlp.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    yr, _, _ = ref_forward(torch, mlp.layers(), x.astype(np.float64))
    err = np.abs(y - yr[:, :100]).max() / np.abs(yr[:, :100]).max()
    assert err < 2e-3, err


def test_gradients_match_fp64_restatement(cuda, mlp):
    torch = cuda
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (256, 15)).astype(np.float32)
    t = rng.standard_normal((256, 100)).astype(np.float32)
    g, loss = mlp.gradients(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda())
    gr, lr, _ = ref_grads(torch, mlp.layers(), x.astype(np.float64), t.astype(np.float64), 100)
    assert abs(loss - lr) / lr < 1e-3
    rel = np.linalg.norm(g - gr) / np.linalg.norm(gr)
    cos = float(g @ gr / (np.linalg.norm(g) * np.linalg.norm(gr)))
    assert rel < 2e-2 and cos > 0.9998, (rel, cos)
    # every layer's weight and bias gradient is checked, not just the total
    o = 0
    for n, k in [(256, 64), (256, 256), (256, 256), (128, 256)]:
        for size in (n * k, n):
            a, b = g[o:o + size], gr[o:o + size]
            if np.linalg.norm(b) > 0:
                assert np.linalg.norm(a - b) / np.linalg.norm(b) < 5e-2
            o += size


def test_training_reduces_loss(cuda):
    torch = cuda
    from sctl_gb300.learned import MLP
    m = MLP(in_dim=4, out_dim=8, max_batch=1024, seed=5)
    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.randn(4, 8, device="cuda", generator=g)
    losses = []
    for it in range(400):
        x = torch.rand(1024, 4, device="cuda", generator=g) * 2 - 1
        t = torch.sin(2 * x @ A).contiguous()
        losses.append(m.train_step(x.contiguous(), t, 3e-3 * (0.5 + 0.5 * math.cos(math.pi * it / 400)),
                                   want_loss=(it in (0, 399))))
    assert losses[-1] < losses[0] / 30, (losses[0], losses[-1])


def test_forward_dot_epilogue(cuda, mlp):
    torch = cuda
    rng = np.random.default_rng(2)
    x = torch.from_numpy(rng.uniform(-1, 1, (300, 15)).astype(np.float32)).cuda()
    dens = torch.from_numpy(rng.standard_normal((7, 100))).cuda()
    idx = torch.from_numpy(rng.integers(0, 7, 300)).cuda()
    out = torch.ones(300, dtype=torch.float64, device="cuda")
    mlp.forward_dot(x, dens, idx, out)
    y = mlp.forward(x).double()
    want = 1 + (y * dens[idx]).sum(1)
    assert (out - want).abs().max().item() < 1e-5 * want.abs().max().item()


def test_weights_mode_equals_potential_mode(cuda):
    torch = cuda
    from sctl_gb300.learned import panel_weights
    from sctl_gb300.nearquad import PanelSurface
    from sctl_gb300.torus import Torus
    T = Torus(seed=0)
    S = PanelSurface(T.X, T.N, T.Q, T.size)
    tg = T.targets(300, seed=21)
    xt = torch.from_numpy(tg["r_trg"]).cuda().reshape(-1).contiguous()
    pt, pp = S.near_pairs(xt, 1.5)
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    W = panel_weights(1, pt, pp, xt, S.X)
    pot = (W * sig.reshape(T.np, 100)[pp]).sum(1)
    ref = torch.zeros(300, dtype=torch.float64, device="cuda").index_add_(0, pt, pot)
    got = S.near_correction(xt, sig, (pt, pp), subtract_smooth=False)
    assert ((got - ref).abs().max() / ref.abs().max()).item() < 1e-12
