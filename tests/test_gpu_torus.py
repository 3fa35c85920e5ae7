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


def test_gauss_law_with_treecode_far_field(setup):
    """The whole evaluation with the far field by the treecode (ParticleFMM::Eval's fast path):
    Gauss's law at 2^20 targets to 1e-9 (the direct-far-field evaluation reaches 9.2e-10 there),
    and within 1e-9 of the direct-far-field evaluation.  At this size target clusters carry
    proxies; their points must stay inside the bounding box of the inputs, or the treecode's
    mixed-precision frame differs from the subtraction plan's and the near panels' large
    smooth-rule terms no longer cancel term by term (5.9e-7 here when they did not)."""
    torch, T, S = setup
    tg = T.targets(1 << 20, seed=15, hmin=1e-4, hmax=1.0)
    xt = torch.from_numpy(tg["r_trg"]).cuda()
    one = torch.ones(T.np * T.p * T.p, dtype=torch.float64, device="cuda")
    pairs = S.near_pairs(xt)
    v = S.evaluate(xt, one, pairs=pairs, far="treecode").cpu().numpy()
    info = S.treecode(xt).info()
    assert info["proxy_interactions"] > 0 and info["target_clusters"] > 0
    exact = np.where(tg["side"] < 0, -1.0, 0.0)
    assert np.abs(v - exact).max() < 1e-9
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    a = S.evaluate(xt, sig, pairs=pairs, far="treecode").cpu().numpy()
    b = S.evaluate(xt, sig, pairs=pairs).cpu().numpy()
    assert np.abs(a - b).max() < 1e-9 * max(1.0, np.abs(b).max())


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


@pytest.mark.parametrize("float_pairs", [True, False])
def test_near_matrix_path_equals_adaptive_path(setup, float_pairs):
    """SetupNear once (stored accurate weights), ComputeNearInterac per application: the
    stored-matrix evaluation equals the matrix-free adaptive one, and keeps Gauss's law, with
    the weights stored in FP64 or as float pairs."""
    torch, T, S = setup
    tg = T.targets(3000, seed=16, hmin=1e-4, hmax=1.0)
    xt = torch.from_numpy(tg["r_trg"]).cuda().reshape(-1).contiguous()
    pairs = S.near_pairs(xt, 1.5)
    plan = S.smooth_subtraction_plan(3000, pairs)
    M = S.near_matrix(xt, pairs, float_pairs=float_pairs)
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    a = S.evaluate(xt, sig, pairs=pairs, plan=plan, matrix=M)
    b = S.evaluate(xt, sig, pairs=pairs, plan=plan)
    assert ((a - b).abs().max() / b.abs().max()).item() < 1e-12
    one = torch.ones_like(sig)
    v = S.evaluate(xt, one, pairs=pairs, plan=plan, matrix=M).cpu().numpy()
    assert np.abs(v - np.where(tg["side"] < 0, -1.0, 0.0)).max() < 1e-8
    from sctl_gb300 import capi
    assert capi.load().sctlgpu_device_status(None) == capi.OK


@pytest.mark.parametrize("k0,k1", [(1, 1), (3, 3), (1, 9), (4, 3), (2, 2), (1, 4)])
def test_near_matrix_apply_general_layout(cuda, k0, k1):
    """sctlgpu_near_matrix_apply against a numpy restatement of ComputeNearInterac: uneven
    elements (1..7 nodes), element-major blocks, a permuted target-major order, targets without
    pairs (left untouched), accumulation into U."""
    torch = cuda
    from sctl_gb300 import capi
    lib = capi.load()
    rng = np.random.default_rng(k0 * 10 + k1)
    n_elem, nt, n_pairs = 37, 53, 300
    cnt = rng.integers(1, 8, n_elem)
    dsp = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    F = rng.standard_normal(int(cnt.sum()) * k0)
    pe = rng.integers(0, n_elem, n_pairs)
    pt = rng.integers(0, nt - 5, n_pairs)          # the last 5 targets have no pairs
    sizes = cnt[pe] * k0 * k1
    kdsp = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    K = rng.standard_normal(int(sizes.sum()))
    order = np.argsort(pt, kind="stable")
    tdsp = np.concatenate([[0], np.cumsum(np.bincount(pt, minlength=nt))])
    U0 = rng.standard_normal(nt * k1)
    want = U0.copy()
    for j in range(n_pairs):
        n = cnt[pe[j]] * k0
        blk = K[kdsp[j]:kdsp[j] + n * k1].reshape(k1, n)
        want[pt[j] * k1:(pt[j] + 1) * k1] += blk @ F[dsp[pe[j]] * k0:dsp[pe[j]] * k0 + n]
    d = lambda a, dt=torch.int64: torch.from_numpy(np.ascontiguousarray(a)).to(dt).cuda()  # noqa: E731
    g = {"tdsp": d(tdsp), "ord": d(order), "pe": d(pe), "kd": d(kdsp), "ed": d(dsp), "ec": d(cnt),
         "K": d(K, torch.float64), "F": d(F, torch.float64), "U": d(U0, torch.float64)}
    rc = lib.sctlgpu_near_matrix_apply(k0, k1, nt, g["tdsp"].data_ptr(), n_pairs, g["ord"].data_ptr(),
                                       n_pairs, g["pe"].data_ptr(), g["kd"].data_ptr(), n_elem,
                                       g["ed"].data_ptr(), g["ec"].data_ptr(), K.size, g["K"].data_ptr(),
                                       F.size, g["F"].data_ptr(), g["U"].data_ptr(), None)
    assert rc == capi.OK
    got = g["U"].cpu().numpy()
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13)
    np.testing.assert_array_equal(got[(nt - 5) * k1:], U0[(nt - 5) * k1:])
    # the same blocks as float pairs (converted in place), double-float application
    K2 = g["K"].clone()
    assert lib.sctlgpu_to_float_pairs(K.size, K2.data_ptr(), K2.data_ptr(), None) == capi.OK
    hl = K2.cpu().numpy().view(np.float32).reshape(-1, 2).astype(np.float64)
    assert np.abs(hl.sum(1) - K).max() <= 2.0 ** -46 * np.abs(K).max()
    U2 = d(U0, torch.float64)
    rc = lib.sctlgpu_near_matrix_apply_pairs(k0, k1, nt, g["tdsp"].data_ptr(), n_pairs, g["ord"].data_ptr(),
                                             n_pairs, g["pe"].data_ptr(), g["kd"].data_ptr(), n_elem,
                                             g["ed"].data_ptr(), g["ec"].data_ptr(), K.size, K2.data_ptr(),
                                             F.size, g["F"].data_ptr(), U2.data_ptr(), None)
    assert rc == capi.OK
    got2 = U2.cpu().numpy()
    np.testing.assert_allclose(got2, want, rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(got2[(nt - 5) * k1:], U0[(nt - 5) * k1:])
    # the index chain resolved once: both forms of the blocks give the same sums as through the chain
    res = torch.empty(2 * n_pairs, dtype=torch.int64, device="cuda")
    assert lib.sctlgpu_near_matrix_resolve(k0, k1, n_pairs, g["ord"].data_ptr(), n_pairs, g["pe"].data_ptr(),
                                           g["kd"].data_ptr(), n_elem, g["ed"].data_ptr(), g["ec"].data_ptr(),
                                           K.size, F.size, res.data_ptr(), None) == capi.OK
    for kk, k2, ref in ((g["K"], None, got), (None, K2, got2)):
        U3 = d(U0, torch.float64)
        rc = lib.sctlgpu_near_matrix_apply_resolved(k0, k1, nt, g["tdsp"].data_ptr(), n_pairs, res.data_ptr(), K.size,
                                                    kk.data_ptr() if kk is not None else None,
                                                    k2.data_ptr() if k2 is not None else None, F.size,
                                                    g["F"].data_ptr(), U3.data_ptr(), None)
        assert rc == capi.OK
        np.testing.assert_array_equal(U3.cpu().numpy(), ref)
    assert lib.sctlgpu_near_matrix_apply_resolved(k0, k1, nt, g["tdsp"].data_ptr(), n_pairs, res.data_ptr(), K.size,
                                                  g["K"].data_ptr(), K2.data_ptr(), F.size, g["F"].data_ptr(),
                                                  U3.data_ptr(), None) == capi.ERR_INVALID_ARGUMENT
    assert capi.load().sctlgpu_device_status(None) == capi.OK
    # an element index out of range: resolved as invalid, skipped and flagged when applied
    bad = int(order[0])
    pe_bad = pe.copy()
    pe_bad[bad] = n_elem + 5
    g["pe_bad"] = d(pe_bad)
    assert lib.sctlgpu_near_matrix_resolve(k0, k1, n_pairs, g["ord"].data_ptr(), n_pairs, g["pe_bad"].data_ptr(),
                                           g["kd"].data_ptr(), n_elem, g["ed"].data_ptr(), g["ec"].data_ptr(),
                                           K.size, F.size, res.data_ptr(), None) == capi.OK
    U4 = d(U0, torch.float64)
    assert lib.sctlgpu_near_matrix_apply_resolved(k0, k1, nt, g["tdsp"].data_ptr(), n_pairs, res.data_ptr(), K.size,
                                                  g["K"].data_ptr(), None, F.size, g["F"].data_ptr(), U4.data_ptr(),
                                                  None) == capi.OK
    assert capi.load().sctlgpu_device_status(None) == capi.ERR_DEVICE_TIMEOUT  # status bit 4: a pair skipped
    assert capi.load().sctlgpu_device_status(None) == capi.OK  # reading clears it
    n = cnt[pe[bad]] * k0
    blk = K[kdsp[bad]:kdsp[bad] + n * k1].reshape(k1, n)
    want4 = want.copy()
    want4[pt[bad] * k1:(pt[bad] + 1) * k1] -= blk @ F[dsp[pe[bad]] * k0:dsp[pe[bad]] * k0 + n]
    np.testing.assert_allclose(U4.cpu().numpy(), want4, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("kernel", [0, 1])
def test_double_float_panel_quadrature_matches_fp64(setup, kernel):
    """The default double-float panel kernel against the FP64 one (both refine with the same FP32
    box test): corrections (with the smooth part subtracted in-kernel) and weights agree far below
    the quadrature's own error (1e-10 relative)."""
    torch, T, S = setup
    from sctl_gb300 import capi
    from sctl_gb300.learned import panel_weights
    lib = capi.load()
    tg = T.targets(1500, seed=18, hmin=1e-4, hmax=1.0)
    xt = torch.from_numpy(tg["r_trg"]).cuda().reshape(-1).contiguous()
    pairs = S.near_pairs(xt, 1.5)
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    res = {}
    for mode in (capi.F64, capi.MIXED):
        prev = lib.sctlgpu_panel_arithmetic(mode)
        try:
            c = S.near_correction(xt, sig, pairs, kernel=kernel).cpu().numpy()
            w = panel_weights(kernel, pairs[0][:3000].contiguous(), pairs[1][:3000].contiguous(), xt, S.X)
            res[mode] = (c, w.cpu().numpy())
        finally:
            lib.sctlgpu_panel_arithmetic(prev)
    (c64, w64), (cdf, wdf) = res[capi.F64], res[capi.MIXED]
    assert np.abs(cdf - c64).max() <= 1e-11 * np.abs(c64).max(), np.abs(cdf - c64).max() / np.abs(c64).max()
    assert np.abs(wdf - w64).max() <= 2e-11 * np.abs(w64).max()
    assert lib.sctlgpu_device_status(None) == capi.OK


@pytest.fixture(scope="module")
def oracle_pairs(setup):
    """Ten (target, panel) pairs -- targets 1e-4 .. 0.5 panel sizes off their own panel, each with
    its own and the next panel -- and their weights from the CPU restatement of the quadrature
    (oracle/panel_oracle.py: alpha = 2 and 14 x 14 Gauss points, converged to rounding)."""
    torch, T, S = setup
    from oracle import panel_oracle as PO
    hs = [1e-4, 1e-3, 1e-2, 0.1, 0.5]
    panels = [100, 777, 1500, 2047, 31]
    xt = np.concatenate([T.targets(1, seed=19 + i, hmin=h, hmax=h, panels=[p])["r_trg"]
                         for i, (h, p) in enumerate(zip(hs, panels))])
    pt, pp = [], []
    for i, p in enumerate(panels):
        pt += [i, i]
        pp += [p, p // T.n_phi * T.n_phi + (p % T.n_phi + 1) % T.n_phi]  # own panel, next along phi
    ref = {k: np.stack([PO.panel_weights(T.X[p], xt[i], kernel=k) for i, p in zip(pt, pp)]) for k in (0, 1)}
    return xt, np.array(pt), np.array(pp), ref


@pytest.mark.parametrize("arith", ["mixed", "f64"])
@pytest.mark.parametrize("alpha", [1.0, 2.0])
@pytest.mark.parametrize("kernel", [1, 0])
def test_panel_weights_match_cpu_oracle(setup, oracle_pairs, arith, alpha, kernel):
    """The GPU's near-singular weights (`sctlgpu_panel_near_weights`, double-float and FP64 forms)
    against the CPU oracle.  With the oracle's acceptance ratio (alpha = 2) node by node to
    1e-11; with the default alpha = 1 the weights applied to the torus density (what a potential
    sees) to 1e-9 -- single weights of the far neighbours differ up to ~1e-7 there, as the
    8-point rule at one diameter resolves the weights' sum far better than each weight."""
    torch, T, S = setup
    from sctl_gb300 import capi
    from sctl_gb300.learned import panel_weights
    xt, pt, pp, refs = oracle_pairs
    ref = refs[kernel]
    lib = capi.load()
    prev = lib.sctlgpu_panel_arithmetic(capi.MIXED if arith == "mixed" else capi.F64)
    try:
        xd = torch.from_numpy(xt).cuda().reshape(-1).contiguous()
        W = panel_weights(kernel, torch.from_numpy(pt).cuda(), torch.from_numpy(pp).cuda(), xd, S.X,
                          alpha=alpha).cpu().numpy()
    finally:
        lib.sctlgpu_panel_arithmetic(prev)
    assert lib.sctlgpu_device_status(None) == capi.OK
    node = max(np.abs(W[k] - ref[k]).max() / np.abs(ref[k]).max() for k in range(len(pt)))
    pot = max(abs((W[k] - ref[k]) @ T.sigma[p]) / abs(ref[k] @ T.sigma[p]) for k, p in enumerate(pp))
    print(f"kernel {kernel} {arith} alpha {alpha}: node weights {node:.2e}, density-weighted {pot:.2e}")
    if alpha == 2.0:
        assert node < 1e-11, node
    else:
        assert pot < 1e-9 and node < 1e-6, (pot, node)


def test_refinement_overflow_is_flagged_not_dropped(setup, oracle_pairs):
    """A per-level box queue too small for the refinement (alpha = 4 next to the panel) integrates
    the remaining boxes unrefined instead of dropping them -- the weights stay finite -- and sets
    bit 2 of the status word; an ordinary call leaves the word clear."""
    import ctypes
    torch, T, S = setup
    from sctl_gb300 import capi
    from sctl_gb300.learned import panel_weights
    xt, pt, pp, refs = oracle_pairs
    lib = capi.load()
    word = ctypes.c_uint(0)
    assert lib.sctlgpu_device_status_word(None, ctypes.byref(word)) == capi.OK
    xd = torch.from_numpy(xt).cuda().reshape(-1).contiguous()
    sel = torch.tensor([0]).cuda()  # 1e-4 panel sizes off its own panel
    W = panel_weights(1, torch.from_numpy(pt).cuda()[sel], torch.from_numpy(pp).cuda()[sel], xd, S.X, alpha=4.0)
    assert lib.sctlgpu_device_status_word(None, ctypes.byref(word)) == capi.OK
    assert word.value & 2, word.value
    w = W.cpu().numpy()[0]
    assert np.all(np.isfinite(w))
    panel_weights(1, torch.from_numpy(pt).cuda()[sel], torch.from_numpy(pp).cuda()[sel], xd, S.X, alpha=1.0)
    assert lib.sctlgpu_device_status_word(None, ctypes.byref(word)) == capi.OK
    assert word.value == 0


def test_matches_the_reference_legacy_quadrature(setup):
    """The GPU near-singular evaluation (far field + smooth-rule subtraction + adaptive panel
    corrections) against SCTL's own legacy boundary quadrature on the same torus, density and
    targets (tests/golden/legacy_torus_dl.npz, orders 32/48), in both panel arithmetics.  The
    golden also holds the legacy values with a 64-point direct rule: where the two agree to 1e-11
    the legacy value is exact to its rounding and the GPU must match it to 1e-9; elsewhere (targets
    next to a panel edge, whose neighbour the legacy rule integrates with its plain direct rule)
    twice the two values' difference bounds the legacy's own error (the denser rule at least
    halves it), and the GPU must lie within that."""
    import json
    import os
    torch, T, S = setup
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    meta = json.load(open(os.path.join(here, "legacy_torus_dl.json")))
    g = np.load(os.path.join(here, "legacy_torus_dl.npz"))
    U, U64 = g["U"], g["U_direct64"]
    est = np.abs(U - U64)
    trusted = est <= 1e-11
    assert meta["torus_seed"] == 0 and trusted.sum() >= 180  # 193 of 256 in the golden
    tg = T.targets(meta["n_trg"], seed=meta["target_seed"], hmin=meta["hmin"], hmax=meta["hmax"])
    xt = torch.from_numpy(tg["r_trg"]).cuda()
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    from sctl_gb300 import capi
    lib = capi.load()
    for arith in ("mixed", "f64"):  # double-float and FP64 panel kernels
        prev = lib.sctlgpu_panel_arithmetic(capi.MIXED if arith == "mixed" else capi.F64)
        try:
            v = S.evaluate(xt, sig, kernel=1, mode="mixed", digits=10).cpu().numpy()
        finally:
            lib.sctlgpu_panel_arithmetic(prev)
        err = np.abs(v - U)
        print(f"{arith}: {int(trusted.sum())} trusted targets, max abs {err[trusted].max():.3e}; others: "
              f"max abs {err[~trusted].max() if (~trusted).any() else 0:.3e} (legacy error estimate up to "
              f"{est.max():.3e})")
        # the potentials are O(1): 1e-9 absolute
        assert err[trusted].max() < 1e-9, (arith, err[trusted].max())
        # elsewhere the denser rule at least halves the legacy's error, so |U - exact| <= 2 |U - U64|
        assert np.all(err <= 2 * est + 1e-9), (arith, np.max(err - 2 * est))
