"""FP64 numpy restatement of the treecode's evaluation from its host layout
(`sctlgpu_treecode_layout`) -- test infrastructure: it computes the source proxies' moments, every
interaction block and the downward pass exactly as the library describes them, so that the CPU
suite can check the algorithm against the direct-sum oracle and the GPU suite can pin the device
implementation to it.

Conventions restated from sctl_gb300/csrc/treecode.cu: a cluster's interpolation box is the tight
box of its points; its grid has g_d Chebyshev points of the second kind along dimension d (one
point, at the box's upper end, along a side of zero extent), grid point k = (i g_1 + j) g_2 + l;
the Stokes double layer's proxies carry the symmetric part S of sum_s L_k(y_s) n_s (x) f_s, one
proxy per grid point.
"""
import numpy as np

from sctl_gb300 import treecode as TC

SCALE = {0: 1 / (4 * np.pi), 1: 1 / (4 * np.pi), 2: 1 / (8 * np.pi), 3: 3 / (4 * np.pi)}


def cheb(g):
    """The g Chebyshev points of the second kind (degree g - 1) and barycentric weights."""
    p = g - 1
    if p == 0:
        return np.array([1.0]), np.array([1.0])
    m = np.arange(p + 1)
    return np.cos(np.pi * m / p), (-1.0) ** m * np.where((m == 0) | (m == p), 0.5, 1.0)


def cheb_coord(lo, hi, x):
    return np.where(x >= 0, hi - 0.5 * (1.0 - x) * (hi - lo), lo + 0.5 * (1.0 + x) * (hi - lo))


def lagrange(t, x, w):
    """Barycentric Lagrange basis at the points t (n,) for nodes x: (n, len(x))."""
    d = t[:, None] - x[None, :]
    hit = d == 0
    q = np.where(hit, 0.0, w[None, :] / np.where(hit, 1.0, d))
    L = q / np.where(hit.any(1), 1.0, q.sum(1))[:, None]
    rows = hit.any(1)
    L[rows] = hit[rows].astype(float)
    return L


def grid_basis(pts, g):
    """Tensor-product basis of the tight box of pts with g = (g0, g1, g2) points: (n, g0 g1 g2),
    and the grid's coordinates (g0 g1 g2, 3)."""
    lo, hi = pts.min(0), pts.max(0)
    ext = hi - lo
    inv = np.where(ext > 0, 2.0 / np.where(ext > 0, ext, 1.0), 0.0)
    Ls, xs = [], []
    for d in range(3):
        x, w = cheb(int(g[d]))
        t = np.clip((pts[:, d] - lo[d]) * inv[d] - 1.0, -1.0, 1.0)
        Ls.append(lagrange(t, x, w))
        xs.append(cheb_coord(lo[d], hi[d], x))
    B = np.einsum("si,sj,sl->sijl", *Ls).reshape(len(pts), -1)
    G = np.stack(np.meshgrid(*xs, indexing="ij"), -1).reshape(-1, 3)
    return B, G


def kernel_sum(k, xt, xs, n, f, sym=False):
    """sum over sources of the (unscaled) kernel; r = x_t - y_s, coincident pairs contribute 0."""
    r = xt[:, None, :] - xs[None, :, :]
    r2 = (r * r).sum(2)
    y = np.where(r2 > 0, 1.0 / np.sqrt(np.where(r2 > 0, r2, 1.0)), 0.0)
    if k == 0:
        return (f[None, :] * y).sum(1)[:, None]
    if k == 1:
        return ((r * n[None]).sum(2) * f[None, :] * y ** 3).sum(1)[:, None]
    if k == 2:
        fd = (r * f[None]).sum(2) * y ** 3
        return (f[None] * y[..., None] + r * fd[..., None]).sum(1)
    if sym:  # n = diag(S), f = (2 S01, 2 S02, 2 S12)
        q = (n[None] * r * r).sum(2) + f[None, :, 0] * r[..., 0] * r[..., 1] + \
            f[None, :, 1] * r[..., 0] * r[..., 2] + f[None, :, 2] * r[..., 1] * r[..., 2]
    else:
        q = (r * n[None]).sum(2) * (r * f[None]).sum(2)
    return (r * (q * y ** 5)[..., None]).sum(1)


def evaluate(k, xs, xn, f, xt, **layout_kw):
    """Potentials at xt (nt * TrgDim) by the treecode of `TC.layout(k, xs, xt, **layout_kw)`."""
    s, blocks, slot_src, trg_order, clusters, tclusters = TC.layout(k, xs, xt, **layout_kw)
    sd, td = (3, 3) if k >= 2 else (1, 1)
    ns, nt = len(xs), len(xt)
    F = np.asarray(f, np.float64).reshape(ns, sd)
    Nrm = np.zeros((ns, 3)) if xn is None else np.asarray(xn, np.float64)
    n_src, n_slots = s["source_slots"], s["slots"]
    # slot arrays: sources (padding: zero density), then the source proxies
    X, N, D = np.zeros((n_slots, 3)), np.zeros((n_slots, 3)), np.zeros((n_slots, sd))
    sym = np.zeros(n_slots, bool)
    idx = slot_src[:n_src]
    real = idx >= 0
    X[:n_src][real], N[:n_src][real], D[:n_src][real] = xs[idx[real]], Nrm[idx[real]], F[idx[real]]
    for c in clusters:
        sb, se, p0, p1 = (int(v) for v in c[:4])
        ids = slot_src[sb:se]
        ids = ids[ids >= 0]
        B, G = grid_basis(xs[ids], c[4:7])
        npts = len(G)
        X[p0:p0 + npts] = G
        if k == 0:
            D[p0:p0 + npts, 0] = B.T @ F[ids, 0]
        elif k == 1:
            N[p0:p0 + npts] = B.T @ (F[ids] * Nrm[ids])
            D[p0:p0 + npts, 0] = 1.0
        elif k == 2:
            D[p0:p0 + npts] = B.T @ F[ids]
        else:
            M = (B.T @ (Nrm[ids][:, :, None] * F[ids][:, None, :]).reshape(len(ids), 9)).reshape(npts, 3, 3)
            N[p0:p0 + npts] = M[:, [0, 1, 2], [0, 1, 2]]
            D[p0:p0 + npts] = np.stack([M[:, 0, 1] + M[:, 1, 0], M[:, 0, 2] + M[:, 2, 0], M[:, 1, 2] + M[:, 2, 1]], 1)
            sym[p0:p0 + npts] = True
    # target list: sorted targets, then the target clusters' proxies
    T = np.zeros((s["target_list"], 3))
    T[:nt] = xt[trg_order]
    tgrid = []
    for c in tclusters:
        b, e, p0, p1 = (int(v) for v in c[:4])
        B, G = grid_basis(T[b:e], c[4:7])
        T[p0:p1] = G
        tgrid.append((b, e, p0, p1, B))
    U = np.zeros((s["target_list"], td))
    for s0, sn, t0, tn in blocks:
        sl = slice(s0, s0 + sn)
        for a in range(t0, t0 + tn, 512):
            ts = slice(a, min(t0 + tn, a + 512))
            if k == 3 and sym[s0]:
                U[ts] += kernel_sum(k, T[ts], X[sl], N[sl], D[sl], sym=True)
            else:
                U[ts] += kernel_sum(k, T[ts], X[sl], N[sl], D[sl] if sd == 3 else D[sl, 0])
    out_sorted = U[:nt].copy()
    for b, e, p0, p1, B in tgrid:  # the downward pass: every target cluster adds to its targets
        out_sorted[b:e] += B @ U[p0:p1]
    out = np.zeros((nt, td))
    out[trg_order] = out_sorted * SCALE[k]
    return out.reshape(-1), s
