"""The CPU panel-quadrature oracle (oracle/panel_oracle.py) pinned by a closed form: on a flat
square panel the double-layer weights of any target sum to the square's solid angle over 4 pi
(the bases sum to one), from 1e-4 to 1 panel sizes off the surface, above the panel, beside it
and beyond its corner."""
import time

import numpy as np
import pytest

from oracle import panel_oracle as PO


def flat_square(L=0.1, p=10):
    x = PO.cheb_nodes(p) * L
    S, T = np.meshgrid(x, x, indexing="ij")
    return np.stack([S.reshape(-1), T.reshape(-1), np.zeros(p * p)], 1)


@pytest.mark.parametrize("s0,t0", [(0.3, 0.6), (0.5, 0.5), (0.97, 0.02), (1.3, 0.4), (-0.2, -0.1)])
@pytest.mark.parametrize("h", [1e-4, -1e-3, 1e-2, -0.1, 1.0])
def test_flat_square_solid_angle(s0, t0, h):
    L = 0.1
    X = flat_square(L)
    xt = np.array([s0 * L, t0 * L, h * L])
    W = PO.panel_weights(X, xt, kernel=1)
    want = PO.square_solid_angle(L, s0, t0, h * L)
    assert abs(W.sum() - want) < 1e-13, (W.sum(), want)


@pytest.mark.parametrize("s0,t0", [(0.3, 0.6), (0.97, 0.02), (1.3, 0.4)])
@pytest.mark.parametrize("h", [1e-4, 1e-2, -1.0])
def test_flat_square_single_layer(s0, t0, h):
    """The single layer's weights of a flat square sum to the square's 1/r potential / 4 pi."""
    L = 0.1
    X = flat_square(L)
    xt = np.array([s0 * L, t0 * L, h * L])
    W = PO.panel_weights(X, xt, kernel=0)
    want = PO.square_single_layer(L, s0, t0, h * L)
    assert abs(W.sum() - want) < 1e-13 * max(1.0, abs(want)), (W.sum(), want)


def test_oracle_cost_is_small():
    X = flat_square()
    t0 = time.perf_counter()
    PO.panel_weights(X, np.array([0.05, 0.05, 1e-5]), kernel=1)
    assert time.perf_counter() - t0 < 5.0


def dense_rule_weights(X, xt, q=48):
    """Every node's weight by one q x q Gauss-Legendre rule over the whole panel (converged to
    rounding for targets a few panel sizes away)."""
    p = int(round(np.sqrt(X.shape[0])))
    F = X.reshape(p, p, 3)
    xn, bw = PO.cheb_nodes(p), PO.bary_weights(p)
    g, gw = PO.gauss_legendre01(q)
    Ls, Ds = PO.lagrange(xn, bw, g)
    P = np.einsum("ia,jb,abk->ijk", Ls, Ls, F)
    nrm = np.cross(np.einsum("ia,jb,abk->ijk", Ds, Ls, F), np.einsum("ia,jb,abk->ijk", Ls, Ds, F))
    r = xt[None, None] - P
    K = (r * nrm).sum(-1) / ((r * r).sum(-1)) ** 1.5 * np.outer(gw, gw)
    return PO.SCALE[1] * np.einsum("ij,ia,jb->ab", K, Ls, Ls).reshape(-1)


@pytest.mark.parametrize("panel", ["flat", "torus"])
def test_adaptive_weights_equal_a_dense_rule_away_from_the_panel(panel):
    """Node by node, the adaptive rule equals one dense Gauss rule over the whole panel for
    targets 2 to 50 panel sizes away (flat square, and a curved panel of the test torus)."""
    if panel == "flat":
        X, L = flat_square(0.1), 0.1
        c, nrm = np.array([0.05, 0.05, 0.0]), np.array([0.0, 0.0, 1.0])
    else:
        from sctl_gb300.torus import Torus
        T = Torus(seed=0)
        X, L = T.X[777], T.size[777]
        c, nrm = X.mean(0), T.N[777][44]
    for dist in (2.0, 5.0, 50.0):
        xt = c + dist * L * nrm + 0.3 * L * np.array([1.0, -0.5, 0.2])
        W = PO.panel_weights(X, xt, kernel=1)
        D = dense_rule_weights(X, xt)
        assert np.abs(W - D).max() <= 1e-13 * np.abs(D).max(), (dist, np.abs(W - D).max() / np.abs(D).max())


def test_oracle_matches_the_reference_legacy_quadrature():
    """Pinned to the reference itself: the near-singular double-layer potential of the torus
    workload from SCTL's legacy boundary quadrature (boundary_quadrature.hpp, orders 32/48,
    tests/golden/legacy_torus_dl.npz from make_legacy_golden.py) for targets 1e-4..1 panel sizes
    off the surface, against the full panel-by-panel sum of the oracle's weights."""
    import json
    import os

    from sctl_gb300.torus import Torus
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    meta = json.load(open(os.path.join(here, "legacy_torus_dl.json")))
    g = np.load(os.path.join(here, "legacy_torus_dl.npz"))
    U = g["U"]
    trusted = np.abs(U - g["U_direct64"]) <= 1e-11  # the legacy value does not move with a denser direct rule
    T = Torus(seed=meta["torus_seed"])
    tg = T.targets(meta["n_trg"], seed=meta["target_seed"], hmin=meta["hmin"], hmax=meta["hmax"])
    order = [int(i) for i in np.argsort(tg["h"]) if trusted[i]]
    picks = [order[int(q * (len(order) - 1))] for q in (0.0, 0.15, 0.35, 0.55, 0.8, 1.0)]  # 1e-4 .. 1 panel sizes
    for t in picks:
        v = sum(PO.panel_weights(T.X[p], tg["r_trg"][t], kernel=1) @ T.sigma[p] for p in range(T.np))
        assert abs(v - U[t]) <= 1e-10 + 1e-9 * abs(U[t]), (t, tg["h"][t], v, U[t])
