"""Plan creation rejects malformed block tables before touching a device."""
import ctypes

import numpy as np

from sctl_gb300 import capi
from sctl_gb300 import workloads as W


def create(blocks, ns, nt, kernel=1, mode=capi.MIXED, tmap=None, n_out=-1):
    h = ctypes.c_void_p()
    b = np.ascontiguousarray(blocks, np.int64).reshape(-1, 4)
    tm = None if tmap is None else np.ascontiguousarray(tmap, np.int64)
    return capi.load().sctlgpu_near_plan_create(ctypes.byref(h), kernel, mode, -1, b.shape[0], b.ctypes.data, ns, nt,
                                               None if tm is None else tm.ctypes.data, n_out)


def test_invalid_blocks_rejected():
    assert create([[0, 5, 0, 3]], 4, 3) == capi.ERR_INVALID_SIZE          # sources past the end
    assert create([[0, 4, 2, 3]], 4, 3) == capi.ERR_INVALID_SIZE          # targets past the end
    assert create([[0, -1, 0, 3]], 4, 3) == capi.ERR_INVALID_SIZE
    assert create([[0, 4, 0, 3]], 4, 3, kernel=9) == capi.ERR_INVALID_KERNEL
    assert create([[0, 4, 0, 3]], 4, 3, mode=7) == capi.ERR_INVALID_MODE
    assert create([[0, 4, 0, 3]], 4, 3, tmap=[0, 1, 5], n_out=3) == capi.ERR_INVALID_ARGUMENT
    assert create([[0, 4, 0, 3]], 4, 3, mode=capi.F32, tmap=[0, 1, 2], n_out=3) == capi.ERR_INVALID_ARGUMENT


def test_near_blocks_generator_shapes():
    d = W.near_blocks(64, 1, seed=0)
    b = d["blocks"]
    assert b.shape == (64, 4)
    assert b[:, 1].min() >= 100 and b[:, 1].max() <= 6400 and b[:, 3].min() >= 16 and b[:, 3].max() <= 2048
    assert d["r_src"].shape[0] == b[:, 1].sum() and d["r_trg"].shape[0] == b[:, 3].sum()
    assert np.all(b[1:, 0] == np.cumsum(b[:, 1])[:-1])
    p = W.near_blocks(16, 0, seed=1, panel=True)
    assert set(np.unique(p["blocks"][:, 1])) <= {100 * k * k for k in range(1, 9)}


def test_torus_pair_features_device_form_matches_numpy():
    """The torch form of the learned path's pair features (run where the pairs live) equals the
    numpy form used to define them."""
    import torch
    from sctl_gb300.torus import Torus, pair_features, pair_features_device
    T = Torus(seed=0)
    tg = T.targets(1500, seed=5)
    pt, pp = T.near_pairs(tg["r_trg"], 1.0)
    a = pair_features(T, tg["r_trg"], pt, pp)
    b = pair_features_device(T, torch.from_numpy(tg["r_trg"]).reshape(-1), torch.from_numpy(pt),
                             torch.from_numpy(pp)).numpy()
    assert a.shape == b.shape == (pt.size, 15)
    assert np.abs(a - b).max() < 1e-12
