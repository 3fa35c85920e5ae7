"""Batched near-field plans (persistent kernel + work queue + CUDA graph)
against the CPU oracle evaluated block by block."""
import numpy as np
import pytest

from oracle import oracle as O
from sctl_gb300 import capi
from sctl_gb300 import workloads as W
from sctl_gb300.near import NearPlan, autotune

pytestmark = pytest.mark.gpu


def oracle_blocks(k, d, w=None):
    nd, sd, td = O.DIMS[k]
    out = np.zeros((d["r_trg"].shape[0], td))
    f = d["v_src"] if w is None else d["v_src"] * w[:, None]
    for s0, ns, t0, nt in d["blocks"]:
        if nt == 0:
            continue
        out[t0:t0 + nt] = O.eval(k, d["r_trg"][t0:t0 + nt], d["r_src"][s0:s0 + ns],
                                 d["n_src"][s0:s0 + ns] if nd else np.zeros(0), f[s0:s0 + ns]).reshape(nt, td)
    return out


def dev(torch, d, dtype=None):
    return {a: torch.from_numpy(np.ascontiguousarray(v if dtype is None else v.astype(dtype))).cuda()
            for a, v in d.items() if a != "blocks"}


@pytest.mark.parametrize("k", range(4))
# FP32: blocks sit at |x| ~ 10 with targets 1e-3 off the patch, so FP32 coordinates alone
# carry ~1e-6 * 10 / 1e-3 = 1e-2 relative error on the closest double-layer pairs.
@pytest.mark.parametrize("mode,digits,tol", [("f64", -1, 1e-12), ("mixed", 10, 1e-10), ("mixed", 6, 2e-6),
                                             ("f32", -1, 2e-3)])
def test_near_batch_matches_oracle(cuda, k, mode, digits, tol):
    torch = cuda
    d = W.near_blocks(160, k, seed=k)
    ref = oracle_blocks(k, d)
    dt = np.float32 if mode == "f32" else np.float64
    dd = dev(torch, d, dt)
    td = O.DIMS[k][2]
    out = torch.zeros(d["r_trg"].shape[0] * td, dtype=torch.float32 if mode == "f32" else torch.float64,
                      device="cuda")
    plan = NearPlan(k, d["blocks"], d["r_src"].shape[0], d["r_trg"].shape[0], mode=mode, digits=digits)
    plan.execute(dd["r_trg"], dd["r_src"], dd["n_src"], dd["v_src"], out)
    torch.cuda.synchronize()
    assert O.rel_l2(out.cpu().numpy(), ref.reshape(-1)) < tol
    # replay of the captured graph gives the same numbers
    out2 = out.clone()
    plan.execute(dd["r_trg"], dd["r_src"], dd["n_src"], dd["v_src"], out2)
    torch.cuda.synchronize()
    assert torch.equal(out, out2)
    assert plan.status() == capi.OK
    info = plan.info()
    assert info["interactions"] == int((d["blocks"][:, 1] * d["blocks"][:, 3]).sum())
    assert info["items"] >= len(d["blocks"]) and info["graph_kernels"] >= 2


@pytest.mark.parametrize("mode,digits,tol", [("f64", -1, 1e-12), ("mixed", 10, 1e-10)])
def test_near_batch_panel_variant_matches_oracle(cuda, mode, digits, tol):
    """The panel form of the uneven blocks: 10 x 10 panels upsampled k x per side (Ns = 100 k^2,
    k = 1..8), Laplace3D_DxU."""
    torch = cuda
    d = W.near_blocks(96, 1, seed=11, panel=True)
    assert set(np.unique(d["blocks"][:, 1]) // 100) <= {k * k for k in range(1, 9)}
    ref = oracle_blocks(1, d)
    dd = dev(torch, d)
    out = torch.zeros(d["r_trg"].shape[0], dtype=torch.float64, device="cuda")
    plan = NearPlan(1, d["blocks"], d["r_src"].shape[0], d["r_trg"].shape[0], mode=mode, digits=digits)
    plan.execute(dd["r_trg"], dd["r_src"], dd["n_src"], dd["v_src"], out)
    torch.cuda.synchronize()
    assert O.rel_l2(out.cpu().numpy(), ref.reshape(-1)) < tol
    assert plan.status() == capi.OK


def test_near_batch_map_weights_accumulate_and_recapture(cuda):
    torch = cuda
    k = 1
    d = W.near_blocks(120, k, seed=7)
    nt_tot, ns_tot = d["r_trg"].shape[0], d["r_src"].shape[0]
    rng = np.random.default_rng(3)
    w = rng.uniform(-1.0, 2.0, ns_tot)
    n_out = nt_tot // 3 + 1
    tmap = rng.integers(0, n_out, nt_tot)
    per_t = oracle_blocks(k, d, w)[:, 0]
    ref = np.zeros(n_out)
    np.add.at(ref, tmap, per_t)
    dd = dev(torch, d)
    wd = torch.from_numpy(w).cuda()
    plan = NearPlan(k, d["blocks"], ns_tot, nt_tot, mode="mixed", digits=10, trg_map=tmap, n_out=n_out)
    out = torch.full((n_out,), 5.0, dtype=torch.float64, device="cuda")
    plan.execute(dd["r_trg"], dd["r_src"], dd["n_src"], dd["v_src"], out, w_src=wd)
    torch.cuda.synchronize()
    assert O.rel_l2(out.cpu().numpy(), ref) < 1e-10
    plan.execute(dd["r_trg"], dd["r_src"], dd["n_src"], dd["v_src"], out, w_src=wd, accumulate=True)
    torch.cuda.synchronize()
    assert O.rel_l2(out.cpu().numpy(), 2 * ref) < 1e-10
    # new buffers -> the graph is re-captured
    f2 = dd["v_src"] * 3.0
    out3 = torch.empty(n_out, dtype=torch.float64, device="cuda")
    plan.execute(dd["r_trg"], dd["r_src"], dd["n_src"], f2, out3, w_src=wd)
    torch.cuda.synchronize()
    assert O.rel_l2(out3.cpu().numpy(), 3 * ref) < 1e-10


def test_near_batch_empty_and_tiny_blocks(cuda):
    torch = cuda
    k = 0
    xs = np.random.default_rng(1).uniform(0, 1, (50, 3))
    xt = np.random.default_rng(2).uniform(0, 1, (30, 3))
    f = np.random.default_rng(3).standard_normal((50, 1))
    blocks = np.array([[0, 0, 0, 5], [0, 7, 5, 0], [7, 1, 5, 1], [8, 42, 6, 24]], np.int64)
    out = torch.full((30,), 9.0, dtype=torch.float64, device="cuda")
    dd = {a: torch.from_numpy(v).cuda() for a, v in (("r_trg", xt), ("r_src", xs), ("v_src", f))}
    plan = NearPlan(k, blocks, 50, 30, mode="f64")
    plan.execute(dd["r_trg"], dd["r_src"], None, dd["v_src"], out)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    assert np.all(o[:5] == 0)                      # no sources: zero
    assert np.allclose(o[5], O.eval(0, xt[5], xs[7:8], None, f[7:8])[0], rtol=1e-13)
    np.testing.assert_allclose(o[6:30], O.eval(0, xt[6:30], xs[8:50], None, f[8:50]), rtol=1e-12)


def test_autotune_table(cuda):
    t = autotune("Laplace3D_DxU", "mixed", 10)
    assert len(t) == capi.NEAR_CLASSES and all(s in (1, 2, 4, 8) for s in t)
    assert autotune("Laplace3D_DxU", "mixed", 10) == t  # cached
