"""Near-singular panel weights on the CPU -- TEST INFRASTRUCTURE ONLY.

Only tests/ may import this module.  It restates, in numpy FP64, the
quadrature behind the NearInterac contract (boundary_integral.hpp:164-239):
for a target x and a p x p Chebyshev panel with nodes X_ab,

    W_ab = scale * int_[0,1]^2 K(x - X(s,t), Xs x Xt) l_a(s) l_b(t) ds dt,

with the geometry X(s,t) interpolated from the nodes by barycentric Lagrange
(as LagrangeInterp, lagrange-interp.hpp:28), the panel's parameter square
refined towards the target level by level (the legacy quadrature's dyadic
refinement, boundary_quadrature.hpp:364-478, as the method description) and
every accepted box integrated with a q x q Gauss-Legendre rule.  It is written
for accuracy, not speed: boxes are accepted at distance >= alpha * diameter
with alpha = 2 and q = 14 (the nearest singularity of a box's integrand lies
>= 5.6 half-sides away, so each box is exact to rounding), against alpha = 1
and 8 points on the GPU.

Pinned to the reference: the reference's current element list cannot run
this path (the QuadElemList NearInterac stubs assert, quad_element.cpp:278-286),
but its legacy boundary quadrature (boundary_quadrature.hpp, built by
oracle/legacy_quad.cpp with three interface gaps bridged) computes the same
integrals; tests/golden/legacy_torus_dl.npz holds its near-singular potentials
on the torus workload and tests/test_panel_oracle.py checks this restatement
against them (<= 1e-10 + 1e-9 |U|).  Closed forms pin it further: on a flat
square panel sum_ab W_ab is, for any target, the solid angle of the square
over 4 pi (double layer) or the square's 1/r potential over 4 pi (single
layer), and far from a panel every node's weight equals one dense Gauss rule.
"""
from __future__ import annotations

import numpy as np

SCALE = {0: 1.0 / (4.0 * np.pi), 1: 1.0 / (4.0 * np.pi)}  # Laplace3D_FxU, Laplace3D_DxU


def cheb_nodes(p: int):
    i = np.arange(p)
    return (1.0 - np.cos((2 * i + 1) * np.pi / (2 * p))) / 2.0


def bary_weights(p: int):
    i = np.arange(p)
    return (-1.0) ** i * np.sin((2 * i + 1) * np.pi / (2 * p))


def lagrange(xn, bw, s):
    """Basis values L (n, p) and derivatives D (n, p) at points s (no point on a node).

    D_a = l_a * sum_{b != a} w_b (x_b - x_a) / (T d_a d_b^2) with T d_a = sum_c w_c d_a / d_c and
    d = s - x: the textbook l_a (U/T - 1/d_a) cancels catastrophically next to a node."""
    d = s[:, None] - xn[None, :]
    t = bw[None, :] / d
    T = t.sum(1, keepdims=True)
    L = t / T
    Td = (bw[None, None, :] * d[:, :, None] / d[:, None, :]).sum(2)       # (n, p): T d_a
    dx = xn[None, :] - xn[:, None]                                        # (a, b): x_b - x_a
    terms = bw[None, None, :] * dx[None] / (d[:, None, :] ** 2)           # (n, a, b)
    p = len(xn)
    terms[:, np.arange(p), np.arange(p)] = 0.0
    D = L * terms.sum(2) / Td
    return L, D


def gauss_legendre01(q: int):
    x, w = np.polynomial.legendre.leggauss(q)
    return 0.5 * (x + 1.0), 0.5 * w


def panel_weights(X, xt, kernel=1, alpha=2.0, q=14, max_depth=40):
    """W (p*p,) of one (target, panel) pair; X (p*p, 3) node coordinates (node a*p + b, a along
    s), xt (3,).  kernel 1 = Laplace double layer (r.n)/r^3 with r = x - y, 0 = single layer 1/r
    (the area element |Xs x Xt|)."""
    X = np.asarray(X, np.float64)
    p = int(round(np.sqrt(X.shape[0])))
    F = X.reshape(p, p, 3)
    xn, bw = cheb_nodes(p), bary_weights(p)
    g, gw = gauss_legendre01(q)
    W = np.zeros((p, p))
    boxes = np.zeros((1, 2))
    for depth in range(max_depth + 1):
        if not len(boxes):
            break
        size = 2.0 ** -depth
        # box test at the centres (geometry and tangents interpolated there)
        c = boxes + 0.5 * size
        Ls, Ds = lagrange(xn, bw, c[:, 0])
        Lt, Dt = lagrange(xn, bw, c[:, 1])
        Xc = np.einsum("na,nb,abk->nk", Ls, Lt, F)
        Xs = np.einsum("na,nb,abk->nk", Ds, Lt, F)
        Xt = np.einsum("na,nb,abk->nk", Ls, Dt, F)
        diam = size * np.sqrt((Xs ** 2).sum(1) + (Xt ** 2).sum(1))
        dist = np.linalg.norm(Xc - xt[None], axis=1)
        acc = (dist >= alpha * diam) | (depth == max_depth)
        leaf = boxes[acc]
        if len(leaf):
            s = leaf[:, 0:1] + size * g[None]          # (m, q)
            t = leaf[:, 1:2] + size * g[None]
            m = len(leaf)
            Ls, Ds = lagrange(xn, bw, s.reshape(-1))
            Lt, Dt = lagrange(xn, bw, t.reshape(-1))
            Ls, Ds, Lt, Dt = (a.reshape(m, q, p) for a in (Ls, Ds, Lt, Dt))
            P = np.einsum("mia,mjb,abk->mijk", Ls, Lt, F)
            Ps = np.einsum("mia,mjb,abk->mijk", Ds, Lt, F)
            Pt = np.einsum("mia,mjb,abk->mijk", Ls, Dt, F)
            nrm = np.cross(Ps, Pt)
            r = xt[None, None, None, :] - P
            r2 = (r * r).sum(-1)
            if kernel == 1:
                K = (r * nrm).sum(-1) / r2 ** 1.5
            else:
                K = np.linalg.norm(nrm, axis=-1) / np.sqrt(r2)
            K = K * (gw[:, None] * gw[None, :])[None] * size * size
            W += np.einsum("mij,mia,mjb->ab", K, Ls, Lt)
        split = boxes[~acc]
        h = 0.5 * size
        boxes = np.concatenate([split + np.array([dx, dy]) * h for dx in (0, 1) for dy in (0, 1)]) \
            if len(split) else np.zeros((0, 2))
    return SCALE[kernel] * W.reshape(-1)


def square_solid_angle(L, s0, t0, h):
    """Solid angle over 4 pi of the square [0, L]^2 (z = 0) seen from (s0 L, t0 L, h), signed
    like the double layer with normal +z and r = x - y."""
    x1, x2, y1, y2 = -s0 * L, (1 - s0) * L, -t0 * L, (1 - t0) * L
    z = abs(h)

    def f(x, y):
        return np.arctan(x * y / (z * np.sqrt(x * x + y * y + z * z)))

    om = f(x2, y2) - f(x1, y2) - f(x2, y1) + f(x1, y1)
    return np.sign(h) * om / (4.0 * np.pi)


def square_single_layer(L, s0, t0, h):
    """int over the square [0, L]^2 (z = 0) of 1 / (4 pi |x - y|) dA, x = (s0 L, t0 L, h)."""
    x1, x2, y1, y2 = -s0 * L, (1 - s0) * L, -t0 * L, (1 - t0) * L
    z = abs(h)

    def F(x, y):
        r = np.sqrt(x * x + y * y + z * z)
        v = x * np.log(y + r) + y * np.log(x + r)
        if z > 0:
            v -= z * np.arctan(x * y / (z * r))
        return v

    return (F(x2, y2) - F(x1, y2) - F(x2, y1) + F(x1, y1)) / (4.0 * np.pi)

