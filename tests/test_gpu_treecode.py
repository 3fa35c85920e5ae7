"""The GPU treecode (sctlgpu_treecode_*, the fast path of ParticleFMM::Eval) against the direct
sum: the FP64 oracle (the reference's Eval restated, pinned to the reference's own outputs) on
a target sample, and the GPU direct sum on whole target sets.

Tolerance: relative l2 of the potentials within 10^-digits (the accuracy `digits` asks of
ParticleFMM, SetAccuracy fmm-wrapper.txx:270-281) for digits 6 and 10, on the sphere/ball
workload, clustered sources and the torus far field; plus the accumulate flag, an all-direct
tree (one leaf) that must agree with the direct sum to rounding, the fallback to the direct sum
where the traversal saves too little, and repeated evaluations with new densities.
"""
import numpy as np
import pytest

import sctl_gb300 as S
from oracle import oracle as O
from sctl_gb300 import capi, workloads as W
from sctl_gb300 import treecode as TC

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64).reshape(-1)).cuda()


def nrm(k, d):
    return d["n_src"] if k in (1, 3) else None


@pytest.mark.parametrize("k", [0, 1, 2, 3])
@pytest.mark.parametrize("digits", [6, 10])
def test_treecode_vs_oracle_sphere_ball(cuda, k, digits):
    torch = cuda
    nt = 1 << 16
    d = W.sphere_ball(1 << 18, nt, k, seed=40 + k)
    tc = TC.Treecode(k, d["r_src"], d["r_trg"], n_src=nrm(k, d), digits=digits)
    info = tc.info()
    assert info["proxy_interactions"] > 0
    u = tc.eval(dev(torch, d["v_src"])).cpu().numpy()
    assert tc.status() == capi.OK
    sub = np.arange(0, nt, 128)
    ref = O.eval(k, d["r_trg"][sub], d["r_src"], d["n_src"], d["v_src"])
    got = u.reshape(nt, -1)[sub].reshape(-1)
    err = O.rel_l2(got, ref)
    saved = 1 - (info["direct_interactions"] + info["proxy_interactions"]) / info["direct_sum_interactions"]
    print(f"k{k} digits {digits}: rel_l2 {err:.2e}, order {info['order']} theta {info['theta']}, "
          f"interactions saved {saved:.2f}")
    assert err < 10.0 ** -digits


@pytest.mark.parametrize("digits", [6, 10])
def test_treecode_clusters_f64_and_mixed(cuda, digits):
    torch = cuda
    k = 1
    d = W.clusters(1 << 17, 1 << 14, k, seed=3, n_clusters=16, sigma=3e-2)
    ref = None
    for mode in ("f64", "mixed"):
        tc = TC.Treecode(k, d["r_src"], d["r_trg"], n_src=d["n_src"], digits=digits, mode=mode)
        assert tc.info()["proxy_interactions"] > 0
        u = tc.eval(dev(torch, d["v_src"])).cpu().numpy()
        sub = np.arange(0, 1 << 14, 64)
        if ref is None:
            ref = O.eval(k, d["r_trg"][sub], d["r_src"], d["n_src"], d["v_src"])
        assert O.rel_l2(u[sub], ref) < 10.0 ** -digits, mode


def test_treecode_accumulate_and_new_densities(cuda):
    torch = cuda
    k = 2
    d = W.sphere_ball(1 << 18, 1 << 14, k, seed=9)
    tc = TC.Treecode(k, d["r_src"], d["r_trg"], digits=6)
    assert tc.info()["direct_fallback"] == 0
    v1 = dev(torch, d["v_src"])
    v2 = dev(torch, np.random.default_rng(1).standard_normal(d["v_src"].size))
    u1 = tc.eval(v1).clone()
    u2 = tc.eval(v2).clone()
    out = u1.clone()
    tc.eval(v2, out=out, accumulate=True)
    assert torch.allclose(out, u1 + u2, rtol=0, atol=1e-13 * float(out.abs().max()))
    # host arrays (ParticleFMM's Eval on SCTL vectors): the same potentials, and accumulation
    uh = tc.eval_host(d["v_src"])
    assert np.abs(uh - u1.cpu().numpy()).max() <= 1e-14 * np.abs(uh).max()
    tc.eval_host(np.asarray(v2.cpu()), out=uh, accumulate=True)
    assert np.abs(uh - (u1 + u2).cpu().numpy()).max() <= 1e-13 * np.abs(uh).max()
    # linearity of the whole pipeline (moments, proxies, direct blocks)
    u3 = tc.eval(2.0 * v1 - v2)  # to the arithmetic's rounding (FP32 at digits 6)
    assert float((u3 - (2 * u1 - u2)).norm() / u3.norm()) < 1e-6


def test_treecode_coincident_targets_and_particle_cluster_form(cuda):
    """3000 coincident targets (one leaf above batch_max: the downward pass works in pieces),
    with the dual traversal and with the particle-cluster form."""
    torch = cuda
    k = 1
    d = W.sphere_ball(1 << 18, 1 << 13, k, seed=21)
    xt = d["r_trg"].copy()
    xt[:3000] = xt[0]
    sub = np.r_[0:5, 2990:3010, np.arange(3010, 1 << 13, 64)]
    ref = O.eval(k, xt[sub], d["r_src"], d["n_src"], d["v_src"])
    for dual in (True, False):
        tc = TC.Treecode(k, d["r_src"], xt, n_src=d["n_src"], digits=10, dual=dual)
        assert tc.info()["proxy_interactions"] > 0 and tc.info()["direct_fallback"] == 0
        u = tc.eval(dev(torch, d["v_src"])).cpu().numpy()
        assert O.rel_l2(u[sub], ref) < 1e-10, dual
        assert np.abs(u[:3000] - u[0]).max() <= 1e-12 * abs(u[0])


def test_treecode_sources_as_targets_and_flat_sources(cuda):
    """Targets = sources (self-interaction pairs contribute nothing, as in the direct sum), and a
    flat sheet of sources (zero extent in z: every cluster box is degenerate in one dimension)."""
    torch = cuda
    rng = np.random.default_rng(5)
    k = 2
    d = W.sphere_ball(1 << 17, 16, k, seed=30)
    xs = d["r_src"]
    tc = TC.Treecode(k, xs, xs, digits=10)
    assert tc.info()["proxy_interactions"] > 0 and tc.info()["target_clusters"] > 0
    u = tc.eval(dev(torch, d["v_src"])).cpu().numpy()
    sub = np.arange(0, 1 << 17, 97)
    ref = O.eval(k, xs[sub], xs, None, d["v_src"])
    assert O.rel_l2(u.reshape(-1, 3)[sub].reshape(-1), ref) < 1e-10
    k = 1
    ns, nt = 1 << 17, 1 << 14
    xs = np.c_[rng.uniform(-1, 1, (ns, 2)), np.zeros(ns)]
    xn = np.tile([0.0, 0.0, 1.0], (ns, 1))
    xt = np.c_[rng.uniform(-1, 1, (nt, 2)), rng.uniform(-0.5, 0.5, nt)]
    f = rng.standard_normal(ns)
    tc = TC.Treecode(k, xs, xt, n_src=xn, digits=10)
    assert tc.info()["proxy_interactions"] > 0
    u = tc.eval(dev(torch, f)).cpu().numpy()
    sub = np.arange(0, nt, 31)
    assert O.rel_l2(u[sub], O.eval(k, xt[sub], xs, xn, f)) < 1e-10


def test_treecode_moments_in_passes_are_identical(cuda):
    """A partial-moment scratch of 2 MB forces many moment passes; the per-cluster sums keep their
    order, so the moments are those of the single pass (the potentials then agree to the order of
    the plan's atomic additions)."""
    torch = cuda
    k = 3
    d = W.sphere_ball(1 << 18, 1 << 14, k, seed=44)
    v = dev(torch, d["v_src"])
    a = TC.Treecode(k, d["r_src"], d["r_trg"], n_src=d["n_src"], digits=6).eval(v).cpu().numpy()
    tc = TC.Treecode(k, d["r_src"], d["r_trg"], n_src=d["n_src"], digits=6, moment_bytes=2e6)
    assert tc.info()["direct_fallback"] == 0 and tc.info()["clusters"] > 0
    b = tc.eval(v).cpu().numpy()
    assert O.rel_l2(b, a) < 1e-15


def test_stokes_double_layer_symmetric_proxies(cuda):
    """The Stokes double layer's proxies carry the symmetric part of their moment, one per grid
    point (a second plan evaluating r . S r): double-float and FP64 plans against the FP64 oracle
    on clustered points and on a flat sheet (every cluster box degenerate in z), and the
    symmetric moments built in passes equal the single pass."""
    torch = cuda
    k = 3
    rng = np.random.default_rng(8)
    ns, nt = 1 << 17, 1 << 13
    d = W.clusters(ns, nt, k, seed=4, n_clusters=16, sigma=3e-2)
    xn = rng.standard_normal((ns, 3))
    xn /= np.linalg.norm(xn, axis=1, keepdims=True)
    flat = (np.c_[rng.uniform(-1, 1, (ns, 2)), np.zeros(ns)], xn,
            np.c_[rng.uniform(-1, 1, (nt, 2)), rng.uniform(-0.5, 0.5, nt)], rng.standard_normal(3 * ns))
    sub = np.arange(0, nt, 32)
    for xs, ns_, xt, f in ((d["r_src"], d["n_src"], d["r_trg"], d["v_src"]), flat):
        ref = O.eval(k, xt[sub], xs, ns_, f)
        for mode in ("mixed", "f64"):
            tc = TC.Treecode(k, xs, xt, n_src=ns_, digits=10, mode=mode)
            assert tc.info()["proxy_interactions"] > 0 and tc.info()["direct_fallback"] == 0, mode
            u = tc.eval(dev(torch, f)).cpu().numpy().reshape(-1, 3)[sub].reshape(-1)
            assert O.rel_l2(u, ref) < 1e-10, mode
            tc.close()
    v = dev(torch, d["v_src"])
    a = TC.Treecode(k, d["r_src"], d["r_trg"], n_src=d["n_src"], digits=10).eval(v).cpu().numpy()
    b = TC.Treecode(k, d["r_src"], d["r_trg"], n_src=d["n_src"], digits=10, moment_bytes=2e6).eval(v).cpu().numpy()
    assert O.rel_l2(b, a) < 1e-15


def test_treecode_coincident_sources(cuda):
    """Half the sources on one point outside the target ball: their leaf has a one-point grid
    (zero extent in every dimension), whose single proxy carries the leaf's whole moment exactly."""
    torch = cuda
    rng = np.random.default_rng(12)
    for k in (1, 3):
        d = W.sphere_ball(1 << 17, 1 << 13, k, seed=60 + k)
        xs, xn = d["r_src"].copy(), d["n_src"].copy()
        xs[: 1 << 16] = [2.5, 0.5, 0.25]
        xn[: 1 << 16] = rng.standard_normal((1 << 16, 3))
        xn /= np.linalg.norm(xn, axis=1, keepdims=True)
        lay = TC.layout(k, xs, d["r_trg"], digits=10)
        assert np.any(lay[4][:, 4:7].prod(1) == 1), "a one-point source cluster"
        tc = TC.Treecode(k, xs, d["r_trg"], n_src=xn, digits=10)
        assert tc.info()["direct_fallback"] == 0
        u = tc.eval(dev(torch, d["v_src"])).cpu().numpy()
        td = 3 if k == 3 else 1
        sub = np.arange(0, 1 << 13, 16)
        ref = O.eval(k, d["r_trg"][sub], xs, xn, d["v_src"])
        assert O.rel_l2(u.reshape(-1, td)[sub].reshape(-1), ref) < 1e-10, k


def test_treecode_falls_back_to_the_direct_sum(cuda):
    """A geometry where the traversal would keep over three quarters of Ns * Nt: evaluations run
    the direct sum, identical to sctlgpu_eval on the same arrays."""
    torch = cuda
    k = 2
    d = W.sphere_ball(1 << 16, 1 << 13, k, seed=9)
    tc = TC.Treecode(k, d["r_src"], d["r_trg"], digits=8)
    assert tc.info()["direct_fallback"] == 1
    u = tc.eval(dev(torch, d["v_src"])).cpu().numpy()
    ref = S.Stokes3D_FxU.Eval(None, d["r_trg"], d["r_src"], None, d["v_src"], digits=8, mode="mixed")
    np.testing.assert_array_equal(u, ref)
    out = torch.from_numpy(u.copy()).cuda()
    tc.eval(dev(torch, d["v_src"]), out=out, accumulate=True)
    np.testing.assert_allclose(out.cpu().numpy(), 2 * u, rtol=1e-15, atol=0)
    assert tc.status() == capi.OK


def test_treecode_single_leaf_is_the_direct_sum(cuda):
    """One leaf, FP64 arithmetic: the treecode is the direct sum up to summation order."""
    torch = cuda
    k = 3
    d = W.sphere_ball(3001, 1531, k, seed=7)
    tc = TC.Treecode(k, d["r_src"], d["r_trg"], n_src=d["n_src"], digits=-1, mode="f64", leaf_max=4096)
    assert tc.info()["proxy_interactions"] == 0
    u = tc.eval(dev(torch, d["v_src"])).cpu().numpy()
    ref = O.eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    assert O.rel_l2(u, ref) < 1e-14


def test_treecode_torus_far_field(cuda):
    """C5's far field (204,800 panel nodes, densities sigma * Q) at 65,536 near-surface targets,
    Laplace double layer, digits 10: against the GPU direct sum (mixed, digits 10)."""
    torch = cuda
    from sctl_gb300.torus import Torus
    T = Torus(seed=0)
    X, N, Q, sig = T.nodes()
    xt = T.targets(1 << 16, seed=7)["r_trg"]
    f = sig * Q
    ref = S.Laplace3D_DxU.Eval(None, xt, X, N, f, digits=10, mode="mixed")
    for digits in (6, 10):
        tc = TC.Treecode(1, X, xt, n_src=N, digits=digits)
        u = tc.eval(dev(torch, f)).cpu().numpy()
        err = O.rel_l2(u, ref)
        info = tc.info()
        print(f"torus digits {digits}: rel_l2 {err:.2e}, interactions "
              f"{(info['direct_interactions'] + info['proxy_interactions']) / info['direct_sum_interactions']:.3f}"
              " of the direct sum")
        assert err < 10.0 ** -digits


@pytest.mark.parametrize("mode,digits,tol", [("f64", -1, 1e-12), ("mixed", 10, 1e-10)])
@pytest.mark.parametrize("k", [1, 3])
def test_treecode_equals_its_numpy_restatement(cuda, k, mode, digits, tol):
    """The treecode against its numpy restatement from the host layout (moments, every block,
    the downward pass; tests/treecode_numpy.py) at degree 4, where the approximation error
    (~1e-6) is far above both evaluations' rounding: agreement to 1e-12 (FP64) or 1e-10
    (double-float moments, interactions and downward pass) pins the device implementation to
    the algorithm the layout describes."""
    import treecode_numpy as TN
    torch = cuda
    d = W.sphere_ball(1 << 14, 1 << 13, k, seed=80 + k)
    kw = dict(order=4, theta=0.45, leaf_max=128, batch_max=64)
    want, s = TN.evaluate(k, d["r_src"], d["n_src"], d["v_src"], d["r_trg"], digits=-1, **kw)
    assert s["target_clusters"] > 0 and s["clusters"] > 0 and s["direct_fallback"] == 0
    tc = TC.Treecode(k, d["r_src"], d["r_trg"], n_src=d["n_src"], digits=digits, mode=mode, **kw)
    got = tc.eval(dev(torch, d["v_src"])).cpu().numpy()
    assert O.rel_l2(got, want) < tol
    ref = O.eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    assert 1e-8 < O.rel_l2(got, ref) < 1e-4  # the approximation itself is far from exact
