"""Seeded synthetic inputs with the shapes and distributions of the direct-sum
workloads (no public dataset exists for this path).

* ``cube``      -- sources and targets uniform in [0,1]^3, densities N(0,1)
                  (8192 x 8192 Laplace FxU FP64 at digits 14 on the CPU);
* ``sphere_ball`` -- sources uniform on the unit sphere with outward unit
                  normals, targets uniform in the ball of radius 2, densities
                  N(0,1) (2^20 x 2^20 Laplace DxU / Stokes FxU, DxU);
* ``clusters``  -- 64 Gaussian clusters (centres uniform in [0,1]^3, sigma
                  1e-3), equal numbers of sources and targets per cluster
                  (2^20 x 2^20 precision stress, Laplace FxU / Stokes FxU).

All generators use numpy's PCG64 with an explicit seed, so the same inputs
are produced on every machine.
"""
from __future__ import annotations

import numpy as np

SRC_DIM = {0: 1, 1: 1, 2: 3, 3: 3}
NORMAL_DIM = {0: 0, 1: 3, 2: 0, 3: 3}


def _density(rng, n, kernel):
    return rng.standard_normal((n, SRC_DIM[kernel]))


def cube(n_src=8192, n_trg=8192, kernel=0, seed=0):
    rng = np.random.default_rng(seed)
    xs = rng.uniform(0.0, 1.0, (n_src, 3))
    xt = rng.uniform(0.0, 1.0, (n_trg, 3))
    f = _density(rng, n_src, kernel)
    xn = _unit(rng.standard_normal((n_src, 3))) if NORMAL_DIM[kernel] else np.zeros((0, 3))
    return dict(r_trg=xt, r_src=xs, n_src=xn, v_src=f)


def _unit(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def sphere_ball(n_src=1 << 20, n_trg=1 << 20, kernel=1, seed=0):
    rng = np.random.default_rng(seed)
    xs = _unit(rng.standard_normal((n_src, 3)))
    xn = xs.copy()  # outward unit normal of the unit sphere
    d = _unit(rng.standard_normal((n_trg, 3)))
    rad = 2.0 * rng.uniform(0.0, 1.0, n_trg) ** (1.0 / 3.0)
    xt = d * rad[:, None]
    f = _density(rng, n_src, kernel)
    return dict(r_trg=xt, r_src=xs, n_src=xn if NORMAL_DIM[kernel] else np.zeros((0, 3)), v_src=f)


def clusters(n_src=1 << 20, n_trg=1 << 20, kernel=0, seed=0, n_clusters=64, sigma=1e-3):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 1.0, (n_clusters, 3))
    ps, pt = n_src // n_clusters, n_trg // n_clusters
    xs = (c[:, None, :] + sigma * rng.standard_normal((n_clusters, ps, 3))).reshape(-1, 3)
    xt = (c[:, None, :] + sigma * rng.standard_normal((n_clusters, pt, 3))).reshape(-1, 3)
    f = _density(rng, xs.shape[0], kernel)
    xn = _unit(rng.standard_normal((xs.shape[0], 3))) if NORMAL_DIM[kernel] else np.zeros((0, 3))
    return dict(r_trg=xt, r_src=xs, n_src=xn, v_src=f)


GENERATORS = {"cube": cube, "sphere_ball": sphere_ball, "clusters": clusters}


def near_blocks(n_blocks=4096, kernel=1, seed=0, panel=False, diameter=0.1):
    """Uneven near-field blocks: block b has Ns = round(100*64^u) sources
    (or 100*k^2, k = 1..8, with panel=True: 10x10 panels upsampled k x per
    side) on a random smooth patch of the given diameter, unit random normals,
    and Nt = round(16*128^v) targets within one patch diameter off the patch;
    u, v ~ U(0,1).  Blocks sit at random places in [0, 10]^3.

    Returns concatenated arrays and an (n_blocks, 4) int64 block table of
    (src_begin, src_count, trg_begin, trg_count)."""
    rng = np.random.default_rng(seed)
    sd = SRC_DIM[kernel]
    if panel:
        ns = 100 * rng.integers(1, 9, n_blocks) ** 2
    else:
        ns = np.rint(100.0 * 64.0 ** rng.uniform(0, 1, n_blocks)).astype(np.int64)
    nt = np.rint(16.0 * 128.0 ** rng.uniform(0, 1, n_blocks)).astype(np.int64)
    xs, xn, f, xt = [], [], [], []
    for b in range(n_blocks):
        c = rng.uniform(0.0, 10.0, 3)
        q, _ = np.linalg.qr(rng.standard_normal((3, 3)))  # random orientation
        kap = rng.uniform(-3.0, 3.0, 2)

        def surf(m):
            uv = rng.uniform(-0.5, 0.5, (m, 2)) * diameter
            z = 0.5 * (kap[0] * uv[:, 0] ** 2 + kap[1] * uv[:, 1] ** 2)
            p = np.stack([uv[:, 0], uv[:, 1], z], 1)
            nrm = np.stack([-kap[0] * uv[:, 0], -kap[1] * uv[:, 1], np.ones(m)], 1)
            return p, _unit(nrm)

        p, _ = surf(int(ns[b]))
        xs.append(c + p @ q.T)
        xn.append(_unit(rng.standard_normal((int(ns[b]), 3))))
        f.append(rng.standard_normal((int(ns[b]), sd)))
        pt, nt_ = surf(int(nt[b]))
        h = diameter * rng.uniform(0.01, 1.0, int(nt[b]))
        xt.append(c + (pt + nt_ * h[:, None]) @ q.T)
    sb = np.concatenate([[0], np.cumsum(ns)[:-1]])
    tb = np.concatenate([[0], np.cumsum(nt)[:-1]])
    blocks = np.stack([sb, ns, tb, nt], 1).astype(np.int64)
    return dict(r_trg=np.concatenate(xt), r_src=np.concatenate(xs),
                n_src=np.concatenate(xn) if NORMAL_DIM[kernel] else np.zeros((0, 3)),
                v_src=np.concatenate(f), blocks=blocks)


def near_list_case(kind: str, seed: int = 0):
    """Inputs of a near-list build (BuildNearList's Xtrg, Xsrc, src_radius, elem_nds_cnt/dsp):

    * "clusters": 300 elements of 0..11 nodes scattered (sigma 0.02) around uniform centres in
      the unit cube, node radii U(0.01, 0.06), 4000 uniform targets (some elements empty);
    * "torus": the 64 x 32-panel torus (10 x 10 Chebyshev nodes per panel), node radius = its
      panel's size, 1500 targets at 1e-4..1 panel sizes off the surface;
    * "many": 70,000 single-node elements in the unit cube, radii U(0, 0.01), 20,000 targets
      (element ids need three 8-bit radix passes)."""
    rng = np.random.default_rng(seed)
    if kind == "clusters":
        ne = 300
        cnt = rng.integers(0, 12, ne)
        cnt[[5, 17, 299]] = 0
        cen = rng.uniform(0, 1, (ne, 3))
        xs = np.repeat(cen, cnt, 0) + rng.normal(0, 0.02, (int(cnt.sum()), 3))
        rad = rng.uniform(0.01, 0.06, int(cnt.sum()))
        xt = rng.uniform(0, 1, (4000, 3))
    elif kind == "torus":
        from .torus import Torus
        T = Torus(seed=seed)
        cnt = np.full(T.np, T.p * T.p)
        xs = T.X.reshape(-1, 3)
        rad = np.repeat(T.size, T.p * T.p)
        xt = T.targets(1500, seed=seed + 1)["r_trg"]
    elif kind == "many":
        ne = 70000
        cnt = np.ones(ne, np.int64)
        xs = rng.uniform(0, 1, (ne, 3))
        rad = rng.uniform(0, 0.01, ne)
        xt = rng.uniform(0, 1, (20000, 3))
    else:
        raise ValueError(kind)
    cnt = cnt.astype(np.int64)
    dsp = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int64)
    return dict(r_trg=np.ascontiguousarray(xt, np.float64), r_src=np.ascontiguousarray(xs, np.float64),
                src_radius=np.ascontiguousarray(rad, np.float64), elem_nds_cnt=cnt, elem_nds_dsp=dsp)
