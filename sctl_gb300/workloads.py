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
