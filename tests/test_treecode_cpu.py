"""The treecode's host side (sctlgpu_treecode_layout, no device): trees, slot layout and
interaction blocks.  Properties checked on clustered and surface point sets:

* every (target, source) pair is covered exactly once -- directly, through the proxies of a
  source cluster, through the proxies of a target cluster (later interpolated to its
  targets), or both -- with and without target-side proxies;
* the target order is a permutation and the target list is the targets then the target
  clusters' proxies;
* approximated pairs of clusters satisfy the acceptance test, and clusters with proxies hold
  more points than proxies;
* a cluster's grid has order + 1 points along its longest side, no more along any other, and
  one point along a side of zero extent (a flat sheet);
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
    if kind == "coincident":  # half the sources on one point: a cluster with a one-point grid
        c = rng.standard_normal((5, 3))
        xs = c[rng.integers(0, 5, ns)] + 1e-2 * rng.standard_normal((ns, 3))
        xs[: ns // 2] = c[0] + 0.5
        xt = c[rng.integers(0, 5, nt)] + 3e-2 * rng.standard_normal((nt, 3))
        return xs, xt
    # flat sheet (z = 0) with targets above it
    xs = np.c_[rng.uniform(-1, 1, (ns, 2)), np.zeros(ns)]
    xt = np.c_[rng.uniform(-1, 1, (nt, 2)), rng.uniform(0.01, 1, nt)]
    return xs, xt


def _box(p):
    lo, hi = p.min(0), p.max(0)
    return 0.5 * (lo + hi), 0.5 * np.linalg.norm(hi - lo)


@pytest.mark.parametrize("kind", ["sphere_ball", "clusters", "sheet", "coincident"])
@pytest.mark.parametrize("kernel", [0, 3])
@pytest.mark.parametrize("dual", [True, False])
def test_layout_covers_every_pair_once(kind, kernel, dual):
    ns, nt = 12000, 3000
    xs, xt = _points(kind, ns, nt, 3)
    order, theta = 3, 0.6
    s, blocks, slot_src, trg_order, clusters, tclusters = TC.layout(kernel, xs, xt, order=order, theta=theta,
                                                                    leaf_max=96, batch_max=64, dual=dual)
    per_point = 1  # the Stokes double layer too: one proxy per grid point with a symmetric density
    assert s["order"] == order and s["theta"] == theta
    assert s["clusters"] > 0 and s["proxy_interactions"] > 0, "the test geometry must exercise the proxies"
    if not dual:
        assert s["target_clusters"] == 0
    nsrc = s["source_slots"]
    real = slot_src[:nsrc]
    assert np.array_equal(np.sort(real[real >= 0]), np.arange(ns))
    assert np.all(slot_src[nsrc:] == -2)
    assert np.array_equal(np.sort(trg_order), np.arange(nt))
    sgrid, tgrid = clusters[:, 4:7].prod(1), tclusters[:, 4:7].prod(1)
    assert s["target_list"] == nt + tgrid.sum()
    assert np.all(blocks[:, 0] % 2 == 0) and np.all(blocks[:, 1] % 2 == 0)
    assert np.all(clusters[:, 3] - clusters[:, 2] == (sgrid * per_point + 1) // 2 * 2)
    assert np.all(tclusters[:, 3] - tclusters[:, 2] == tgrid) and np.all(tclusters[:, 1] - tclusters[:, 0] > tgrid)
    for c in (clusters, tclusters):
        assert np.all(c[:, 4:7] >= 1) and np.all(c[:, 4:7] <= order + 1)
    for c in clusters:  # the longest side has the full order; a flat side one point
        src = slot_src[c[0]:c[1]]
        p = xs[src[src >= 0]]
        ext = p.max(0) - p.min(0)
        if ext.max() > 0:
            assert c[4 + int(np.argmax(ext))] == order + 1
        assert np.all(c[4:7][ext == 0] == 1)
        if kind == "sheet":
            assert c[6] == 1
    if kind == "coincident":  # the coincident sources' leaf is approximated by a single proxy
        assert np.any(clusters[:, 4:7].prod(1) == 1)
    sprox = {int(c[2]): c for c in clusters}
    tprox = {int(c[2]): c for c in tclusters}
    cnt = np.zeros((nt, ns), np.uint8)  # (sorted target, source) coverage
    direct = approx = 0
    for b in blocks:
        s0, sn, t0, tn = (int(v) for v in b)
        if t0 < nt:  # sorted targets (adjacent batches merged)
            assert t0 + tn <= nt
            tgroups = [np.arange(t0, t0 + tn)]
        else:  # target clusters' proxies (adjacent clusters merged)
            tgroups, pos = [], t0
            while pos < t0 + tn:
                c = tprox[pos]
                tgroups.append(np.arange(c[0], c[1]))
                pos = int(c[3])
            assert pos == t0 + tn
        if s0 < nsrc:
            assert s0 + sn <= nsrc
            src = slot_src[s0:s0 + sn]
            groups = [src[src >= 0]]
        else:
            groups, pos = [], s0
            while pos < s0 + sn:  # merged proxy ranges of adjacent clusters
                c = sprox[pos]
                src = slot_src[c[0]:c[1]]
                groups.append(src[src >= 0])
                assert groups[-1].size > c[4:7].prod() * per_point
                pos = int(c[3])
            assert pos == s0 + sn
        for tset in tgroups:
            cb, rb = _box(xt[trg_order[tset]])
            for g in groups:
                cnt[np.ix_(tset, g)] += 1
                if s0 >= nsrc:
                    cc, rc = _box(xs[g])
                    if t0 >= nt:  # cluster-cluster: the two boxes are separated
                        assert rb + rc < theta * np.linalg.norm(cb - cc) * (1 + 1e-12)
                    else:  # merged batches against a source cluster: every target beyond r_s / theta
                        assert rc < theta * np.linalg.norm(xt[trg_order[tset]] - cc, axis=1).min() * (1 + 1e-12)
                elif t0 >= nt:  # target proxies against sources (adjacent source nodes merged): every
                    # source is beyond r_t / theta of the target cluster's centre
                    assert rb < theta * np.linalg.norm(xs[g] - cb, axis=1).min() * (1 + 1e-12)
        if t0 < nt and s0 < nsrc:
            direct += sn * tn
        else:
            approx += sn * tn
    assert cnt.min() == 1 and cnt.max() == 1, (kind, dual)
    assert direct == s["direct_interactions"] and approx == s["proxy_interactions"]


def test_dual_layout_uses_target_proxies_and_saves_work():
    xs, xt = _points("clusters", 20000, 20000, 5)
    a = TC.layout(1, xs, xt, order=3, theta=0.6, leaf_max=96, batch_max=64, dual=True)[0]
    b = TC.layout(1, xs, xt, order=3, theta=0.6, leaf_max=96, batch_max=64, dual=False)[0]
    assert a["target_clusters"] > 0
    assert a["direct_interactions"] + a["proxy_interactions"] < b["direct_interactions"] + b["proxy_interactions"]


def test_layout_defaults_follow_digits():
    xs, xt = _points("sphere_ball", 4000, 1000, 1)
    orders = [TC.layout(1, xs, xt, digits=d)[0]["order"] for d in (3, 6, 10, 14)]
    assert orders == sorted(orders) and orders[0] < orders[-1]


def test_layout_and_create_reject_bad_arguments():
    xs, xt = _points("clusters", 500, 100, 2)
    for kw in ({"order": 16}, {"theta": 1.0}, {"batch_max": 4096}):
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
    s, blocks, slot_src, trg_order, clusters, tclusters = TC.layout(0, xs, xt, order=4, leaf_max=64)
    assert s["clusters"] == 0 and s["target_clusters"] == 0 and s["proxy_interactions"] == 0
    assert s["direct_interactions"] == 20 * s["source_slots"]
    s, blocks, *_ = TC.layout(0, np.zeros((0, 3)), xt)
    assert s["blocks"] == 0 and s["slots"] == 0
    s, blocks, *_ = TC.layout(0, xs, np.zeros((0, 3)))
    assert s["blocks"] == 0


@pytest.mark.parametrize("kernel", [0, 1, 2, 3])
def test_numpy_restatement_matches_the_direct_sum(kernel):
    """The treecode restated in numpy from its host layout (moments, every block, the downward
    pass; tests/treecode_numpy.py) against the direct-sum oracle: the algorithm the layout
    describes is accurate to its interpolation degree."""
    import treecode_numpy as TN
    from oracle import oracle as O
    d = W.sphere_ball(1 << 13, 1 << 13, kernel, seed=70 + kernel)
    xn = d["n_src"] if kernel in (1, 3) else None
    u, s = TN.evaluate(kernel, d["r_src"], xn, d["v_src"], d["r_trg"], order=4, theta=0.5, leaf_max=128,
                       batch_max=64, digits=10)
    assert s["proxy_interactions"] > 0 and s["target_clusters"] > 0
    ref = O.eval(kernel, d["r_trg"], d["r_src"], xn, d["v_src"])
    assert O.rel_l2(u, ref) < 1e-3  # degree 4
