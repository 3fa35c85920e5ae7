"""The treecode's host side (sctlgpu_treecode_layout, no device): trees, slot layout and
interaction blocks.  Properties checked on clustered and surface point sets:

* every target batch sees every source exactly once -- directly (a leaf's slots) or through
  the proxies of exactly one approximated cluster containing it;
* batches partition the targets, and the target order is a permutation;
* approximated clusters satisfy the acceptance test against their batches and hold more
  sources than proxy slots;
* every block starts and ends on a pair boundary (one pairing of the slot list serves all
  blocks), padding slots are the only sources missing from the slot list.
"""
import numpy as np
import pytest

from sctl_gb300 import capi, workloads as W
from sctl_gb300 import treecode as TC


def _points(kind, ns, nt, seed):
    rng = np.random.default_rng(seed)
    if kind == "sphere_ball":
        d = W.sphere_ball(ns, nt, 1, seed)
        return d["r_src"], d["r_trg"]
    if kind == "clusters":
        c = rng.standard_normal((5, 3))
        xs = c[rng.integers(0, 5, ns)] + 1e-2 * rng.standard_normal((ns, 3))
        xt = c[rng.integers(0, 5, nt)] + 3e-2 * rng.standard_normal((nt, 3))
        return xs, xt
    # flat sheet (z = 0) with targets above it
    xs = np.c_[rng.uniform(-1, 1, (ns, 2)), np.zeros(ns)]
    xt = np.c_[rng.uniform(-1, 1, (nt, 2)), rng.uniform(0.01, 1, nt)]
    return xs, xt


def _box(p):
    lo, hi = p.min(0), p.max(0)
    return 0.5 * (lo + hi), 0.5 * np.linalg.norm(hi - lo)


@pytest.mark.parametrize("kind", ["sphere_ball", "clusters", "sheet"])
@pytest.mark.parametrize("kernel", [0, 3])
def test_layout_covers_every_source_once(kind, kernel):
    ns, nt = 12000, 3000
    xs, xt = _points(kind, ns, nt, 3)
    order, theta = 3, 0.6
    s, blocks, slot_src, trg_order, clusters = TC.layout(kernel, xs, xt, order=order, theta=theta, leaf_max=96,
                                                         batch_max=64)
    npts = (order + 1) ** 3
    per_point = 3 if kernel == 3 else 1
    assert s["order"] == order and s["theta"] == theta
    assert s["clusters"] > 0 and s["proxy_interactions"] > 0, "the test geometry must exercise the proxies"
    nsrc = s["source_slots"]
    real = slot_src[:nsrc]
    assert np.array_equal(np.sort(real[real >= 0]), np.arange(ns))
    assert np.all(slot_src[nsrc:] == -2)
    assert np.array_equal(np.sort(trg_order), np.arange(nt))
    assert np.all(blocks[:, 0] % 2 == 0) and np.all(blocks[:, 1] % 2 == 0)
    pstart = {int(c[2]): c for c in clusters}
    assert np.all(clusters[:, 3] - clusters[:, 2] == (npts * per_point + 1) // 2 * 2)
    batches = {}
    for b in blocks:
        batches.setdefault((int(b[2]), int(b[3])), []).append(b)
    t_ranges = sorted(batches)
    assert t_ranges[0][0] == 0 and sum(n for _, n in t_ranges) == nt
    for (a, n), (a2, _) in zip(t_ranges, t_ranges[1:]):
        assert a + n == a2
    pp = pc = 0
    for (t0, tn), bl in batches.items():
        cnt = np.zeros(ns, np.int64)
        cb, rb = _box(xt[trg_order[t0:t0 + tn]])
        for b in bl:
            s0, sn = int(b[0]), int(b[1])
            if s0 < nsrc:
                assert s0 + sn <= nsrc
                src = slot_src[s0:s0 + sn]
                np.add.at(cnt, src[src >= 0], 1)
                pp += sn * tn
            else:
                pos = s0
                while pos < s0 + sn:  # merged proxy ranges of adjacent clusters
                    c = pstart[pos]
                    src = slot_src[c[0]:c[1]]
                    src = src[src >= 0]
                    assert src.size > npts * per_point
                    np.add.at(cnt, src, 1)
                    cc, rc = _box(xs[src])
                    assert rb + rc < theta * np.linalg.norm(cb - cc) * (1 + 1e-12)
                    pos = int(c[3])
                assert pos == s0 + sn
                pc += sn * tn
        assert np.all(cnt == 1), (kind, np.unique(cnt))
    assert pp == s["direct_interactions"] and pc == s["proxy_interactions"]


def test_layout_defaults_follow_digits():
    xs, xt = _points("sphere_ball", 4000, 1000, 1)
    orders = [TC.layout(1, xs, xt, digits=d)[0]["order"] for d in (3, 6, 10, 14)]
    assert orders == sorted(orders) and orders[0] < orders[-1]


def test_layout_and_create_reject_bad_arguments():
    xs, xt = _points("clusters", 500, 100, 2)
    for kw in ({"order": 16}, {"theta": 1.0}):
        with pytest.raises(capi.SctlGpuError) as e:
            TC.layout(1, xs, xt, **kw)
        assert e.value.status == capi.ERR_INVALID_ARGUMENT
    bad = xs.copy()
    bad[7, 1] = np.nan
    with pytest.raises(capi.SctlGpuError) as e:
        TC.layout(1, bad, xt)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    with pytest.raises(capi.SctlGpuError) as e:
        TC.layout(17, xs, xt)
    assert e.value.status == capi.ERR_INVALID_KERNEL
    # FP32 results are not offered (scattered FP64 outputs); checked before any device use
    with pytest.raises(capi.SctlGpuError) as e:
        TC.Treecode(1, xs, xt, n_src=np.ones_like(xs), mode="f32")
    assert e.value.status == capi.ERR_INVALID_MODE


def test_layout_empty_and_single_leaf():
    xs, xt = _points("clusters", 50, 20, 4)
    s, blocks, slot_src, trg_order, clusters = TC.layout(0, xs, xt, order=4, leaf_max=64)
    assert s["clusters"] == 0 and s["proxy_interactions"] == 0
    assert s["direct_interactions"] == 20 * s["source_slots"]
    s, blocks, *_ = TC.layout(0, np.zeros((0, 3)), xt)
    assert s["blocks"] == 0 and s["slots"] == 0
    s, blocks, *_ = TC.layout(0, xs, np.zeros((0, 3)))
    assert s["blocks"] == 0
