"""Torus test surface for the near-singular double-layer quadrature.

Torus (R = 1, r = 0.3) split into 64 x 32 panels in (theta, phi); each panel
carries 10 x 10 nodes on the reference's Chebyshev rule (ChebQuadRule,
quadrule.txx:71-101: nodes (1 - cos((2i+1) pi / 2N)) / 2 on [0, 1], weights
from the integrals of the Chebyshev polynomials) -- 204,800 nodes in FP64.
The Laplace double-layer density is a sum of 8 random low-order Fourier
modes a cos(m theta + n phi + psi), |m|, |n| <= 3.  Targets sit at off-surface
distances log-uniform in [1e-4, 1] panel sizes on either side of a random
panel point.
"""
from __future__ import annotations

import numpy as np

R_MAJOR, R_MINOR = 1.0, 0.3


def cheb_rule(n: int):
    """ChebQuadRule<Real>::ComputeNdsWts: nodes and weights on [0, 1]."""
    i = np.arange(n)
    nds = (1.0 - np.cos((2 * i + 1) * np.pi / (2 * n))) / 2.0
    theta = (2 * i + 1) * np.pi / (2 * n)
    Minv = np.cos(np.outer(theta, np.arange(n))) / n
    Minv[:, 1:] *= 2.0
    b = np.array([0.0 if k % 2 else -1.0 / (k * k - 1.0) for k in range(n)])
    return nds, Minv @ b


def cheb_bary_weights(n: int):
    """Barycentric weights of the first-kind Chebyshev points (up to a common factor)."""
    i = np.arange(n)
    return (-1.0) ** i * np.sin((2 * i + 1) * np.pi / (2 * n))


def lagrange_matrix(x_nodes, bw, x):
    """L[k, a] = l_a(x_k): barycentric Lagrange basis at points x (exact at nodes)."""
    x = np.asarray(x, np.float64)
    d = x[:, None] - x_nodes[None, :]
    hit = np.isclose(d, 0.0, atol=0.0, rtol=0.0)
    d = np.where(hit, 1.0, d)
    t = bw[None, :] / d
    L = t / t.sum(1, keepdims=True)
    rows = hit.any(1)
    L[rows] = hit[rows].astype(np.float64)
    return L


def surface(theta, phi):
    c, s = np.cos(phi), np.sin(phi)
    rho = R_MAJOR + R_MINOR * c
    X = np.stack([rho * np.cos(theta), rho * np.sin(theta), R_MINOR * s], -1)
    n = np.stack([c * np.cos(theta), c * np.sin(theta), s], -1)  # outward unit normal
    jac = R_MINOR * rho  # |X_theta x X_phi|
    return X, n, jac


class Torus:
    """Panels, nodes, normals, smooth-quadrature weights and density."""

    def __init__(self, n_theta=64, n_phi=32, order=10, seed=0):
        self.n_theta, self.n_phi, self.p = n_theta, n_phi, order
        self.np = n_theta * n_phi
        self.dth, self.dph = 2 * np.pi / n_theta, 2 * np.pi / n_phi
        x, w = cheb_rule(order)
        self.x1d, self.w1d = x, w
        self.bw = cheb_bary_weights(order)
        # panel p = i * n_phi + j ; node q = a * order + b  (a along theta, b along phi)
        i, j = np.divmod(np.arange(self.np), n_phi)
        th = (i[:, None, None] + x[None, :, None]) * self.dth + 0 * x[None, None, :]
        ph = (j[:, None, None] + x[None, None, :]) * self.dph + 0 * x[None, :, None]
        X, n, jac = surface(th, ph)
        self.X = X.reshape(self.np, order * order, 3)
        self.N = n.reshape(self.np, order * order, 3)
        self.Q = (np.outer(w, w)[None] * jac * self.dth * self.dph).reshape(self.np, order * order)
        self.theta0, self.phi0 = i * self.dth, j * self.dph
        self.area = self.Q.sum(1)
        self.size = np.sqrt(self.area)  # panel size used for target distances
        rng = np.random.default_rng(seed)
        self.modes = [(int(rng.integers(-3, 4)), int(rng.integers(-3, 4)), float(rng.standard_normal()),
                       float(rng.uniform(0, 2 * np.pi))) for _ in range(8)]
        self.sigma = self.density(th, ph).reshape(self.np, order * order)

    def density(self, theta, phi):
        s = np.zeros(np.broadcast(theta, phi).shape)
        for m, n, a, psi in self.modes:
            s = s + a * np.cos(m * theta + n * phi + psi)
        return s

    def nodes(self):
        """Flat arrays of all nodes: coordinates, normals, weights, density."""
        return (self.X.reshape(-1, 3), self.N.reshape(-1, 3), self.Q.reshape(-1), self.sigma.reshape(-1))

    def targets(self, n: int, seed=1, hmin=1e-4, hmax=1.0, panels=None):
        """n targets: random panel, random (s, t), distance h = size * 10^U(log10 hmin, log10 hmax),
        random side.  Returns coordinates, owning panel, (s, t), h / size."""
        rng = np.random.default_rng(seed)
        p = rng.integers(0, self.np, n) if panels is None else np.asarray(panels)
        st = rng.uniform(0, 1, (n, 2))
        i, j = np.divmod(p, self.n_phi)
        X, nrm, _ = surface((i + st[:, 0]) * self.dth, (j + st[:, 1]) * self.dph)
        hr = 10.0 ** rng.uniform(np.log10(hmin), np.log10(hmax), n)
        side = np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0)
        xt = X + (side * hr * self.size[p])[:, None] * nrm
        return dict(r_trg=xt, panel=p, st=st, h=hr, side=side)

    def near_pairs(self, xt, factor=1.0):
        """(target, panel) pairs with the target within factor * panel size of the panel's
        node set (the smooth rule is not trusted there).  Returns int64 arrays."""
        cen = self.X.mean(1)
        rad = np.linalg.norm(self.X - cen[:, None, :], axis=2).max(1)
        pairs_t, pairs_p = [], []
        chunk = 4096
        for a in range(0, xt.shape[0], chunk):
            d = np.linalg.norm(xt[a:a + chunk, None, :] - cen[None], axis=2)
            tt, pp = np.nonzero(d < rad[None] + factor * self.size[None])
            pairs_t.append(tt + a)
            pairs_p.append(pp)
        return np.concatenate(pairs_t).astype(np.int64), np.concatenate(pairs_p).astype(np.int64)

    def singular_weights(self, f):
        return singular_weights(self, f)

    def singular_dot(self, f, sig, pp):
        return singular_dot(self, f, sig, pp)

    def basis_features(self, f):
        return basis_features(self, f)

    def upsample_matrix(self, k: int):
        """Interpolation matrix (k*k*p*p, p*p) from a panel's nodes to k x k sub-panels with
        p x p Chebyshev nodes each, the sub-panel weights (fraction of the panel rule), and the
        local coordinates (s, t) of the new nodes."""
        p = self.p
        sub = (np.arange(k)[:, None] + self.x1d[None, :]).reshape(-1) / k  # k*p points in [0,1]
        L = lagrange_matrix(self.x1d, self.bw, sub)                        # (k*p, p)
        Lu = np.einsum("ia,jb->ijab", L, L).reshape(k * p * k * p, p * p)
        w = np.outer(np.tile(self.w1d, k) / k, np.tile(self.w1d, k) / k).reshape(-1)
        s, t = np.meshgrid(sub, sub, indexing="ij")
        return Lu, w, np.stack([s.reshape(-1), t.reshape(-1)], 1)


def foot_point(xt):
    """Closest point on the torus of each target: angles (theta, phi) and signed distance (+ outside)."""
    x, y, z = xt[..., 0], xt[..., 1], xt[..., 2]
    th = np.arctan2(y, x)
    rho = np.hypot(x, y)
    ph = np.arctan2(z, rho - R_MAJOR)
    d = np.hypot(rho - R_MAJOR, z) - R_MINOR
    return th, ph, d


def pair_features(T: "Torus", xt, pt, pp):
    """15 features of (target, panel) pairs: local coordinates (s, t) of the target's foot point in
    the panel's parameter square (outside [0,1] for neighbouring panels), the signed log distance
    in panel sizes, and 12 panel-geometry features (metric, curvatures, size; constant per ring)."""
    th, ph, d = foot_point(xt[pt])
    th0, ph0 = T.theta0[pp], T.phi0[pp]
    s = np.remainder(th - th0 + np.pi, 2 * np.pi) - np.pi
    t = np.remainder(ph - ph0 + np.pi, 2 * np.pi) - np.pi
    s, t = s / T.dth, t / T.dph
    size = T.size[pp]
    hr = np.abs(d) / size
    hf = np.sign(d) * (np.log10(np.maximum(hr, 1e-6)) + 6.0) / 6.0
    phc = ph0 + 0.5 * T.dph
    rho = R_MAJOR + R_MINOR * np.cos(phc)
    lth, lph = rho * T.dth / size, R_MINOR * T.dph / size
    k1, k2 = np.cos(phc) / rho * size, size / R_MINOR
    geo = np.stack([np.cos(phc), np.sin(phc), rho, lth, lph, k1, k2, size * 10.0, T.area[pp] / size ** 2,
                    lth / lph, k1 * k2, 0.5 * (k1 + k2)], 1)
    return np.concatenate([np.stack([s, t, hf], 1), geo], 1)


def pair_features_device(T: "Torus", xt, pt, pp):
    """`pair_features` on torch tensors (any device, FP64): xt (n, 3) or flat target coordinates,
    pt / pp int64 pair indices.  Same formulas, evaluated where the pairs live."""
    import torch
    dev = xt.device
    key = ("_feat_tables", str(dev))
    tab = T.__dict__.get(key)
    if tab is None:
        phc = T.phi0 + 0.5 * T.dph
        rho = R_MAJOR + R_MINOR * np.cos(phc)
        lth, lph = rho * T.dth / T.size, R_MINOR * T.dph / T.size
        k1, k2 = np.cos(phc) / rho * T.size, T.size / R_MINOR
        geo = np.stack([np.cos(phc), np.sin(phc), rho, lth, lph, k1, k2, T.size * 10.0, T.area / T.size ** 2,
                        lth / lph, k1 * k2, 0.5 * (k1 + k2)], 1)
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)  # noqa: E731
        tab = (t(T.theta0), t(T.phi0), t(T.size), t(geo))
        T.__dict__[key] = tab
    th0, ph0, size, geo = tab
    x = xt.reshape(-1, 3)[pt]
    th = torch.atan2(x[:, 1], x[:, 0])
    rho = torch.hypot(x[:, 0], x[:, 1])
    ph = torch.atan2(x[:, 2], rho - R_MAJOR)
    d = torch.hypot(rho - R_MAJOR, x[:, 2]) - R_MINOR
    s = (torch.remainder(th - th0[pp] + np.pi, 2 * np.pi) - np.pi) / T.dth
    t = (torch.remainder(ph - ph0[pp] + np.pi, 2 * np.pi) - np.pi) / T.dph
    hr = d.abs() / size[pp]
    hf = torch.sign(d) * (torch.log10(hr.clamp_min(1e-6)) + 6.0) / 6.0
    return torch.cat([torch.stack([s, t, hf], 1), geo[pp]], 1).contiguous()


def _basis_device(T: "Torus", x):
    """Barycentric Lagrange basis of the panel's 1-D Chebyshev nodes at points x (n,), clamped to
    [0, 1]: (n, p), exact (one-hot) at the nodes."""
    import torch
    nodes = torch.as_tensor(T.x1d, dtype=torch.float64, device=x.device)
    bw = torch.as_tensor(T.bw, dtype=torch.float64, device=x.device)
    d = x.clamp(0.0, 1.0)[:, None] - nodes[None]
    hit = d == 0
    q = bw[None] / torch.where(hit, torch.ones_like(d), d)
    L = q / q.sum(1, keepdim=True)
    rows = hit.any(1)
    return torch.where(rows[:, None], hit.to(L.dtype), L)


SINGULAR_H0 = 0.05  # distance (panel sizes) over which the singular part is switched off


def singular_part(T: "Torus", f, h0=SINGULAR_H0):
    """Leading near-singular behaviour of the Laplace double-layer weights of (target, panel) pairs
    from their features: the density frozen at the (clamped) foot point times the solid angle of
    the panel's flat parameter rectangle, sign(d) * Omega / (4 pi), faded out as 1 / (1 + (h/h0)^2)
    with the distance h in panel sizes (farther away the weights are smooth and the frozen-density
    term would only add structure).  Returns the factor (n,) and the 1-D bases (n, p) along s and t;
    the weight of node (a, b) is factor * Ls[a] * Lt[b].  As d -> 0 inside the panel the factor
    tends to +-1/2, the double layer's jump."""
    import torch
    s, t, hf = f[:, 0], f[:, 1], f[:, 2]
    lth, lph = f[:, 6], f[:, 7]
    z = torch.pow(10.0, 6.0 * hf.abs() - 6.0)
    x1, x2 = -s * lth, (1.0 - s) * lth
    y1, y2 = -t * lph, (1.0 - t) * lph

    def corner(x, y):
        return torch.atan(x * y / (z * torch.sqrt(x * x + y * y + z * z)))

    omega = corner(x2, y2) - corner(x1, y2) - corner(x2, y1) + corner(x1, y1)
    fac = torch.sign(hf) * omega / (4.0 * np.pi) / (1.0 + (z / h0) ** 2)
    return fac, _basis_device(T, s), _basis_device(T, t)


def basis_features(T: "Torus", f):
    """The panel's 1-D Lagrange bases at the pair's clamped foot-point coordinates (s, t),
    (n, 2p): the functions the weights are built from, as extra network inputs."""
    import torch
    return torch.cat([_basis_device(T, f[:, 0]), _basis_device(T, f[:, 1])], 1)


def singular_weights(T: "Torus", f):
    """`singular_part` as (n, p*p) node weights, node q = a * p + b."""
    fac, Ls, Lt = singular_part(T, f)
    return (fac[:, None, None] * Ls[:, :, None] * Lt[:, None, :]).reshape(f.shape[0], -1)


def singular_dot(T: "Torus", f, sig, pp):
    """sum_q singular_weights[n, q] * sig[pp[n], q] without forming the weights; sig (np, p*p)."""
    import torch
    fac, Ls, Lt = singular_part(T, f)
    S = sig.reshape(sig.shape[0], T.p, T.p)[pp]
    return fac * torch.einsum("na,nab,nb->n", Ls, S, Lt)
