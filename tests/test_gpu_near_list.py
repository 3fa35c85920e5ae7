"""GPU near lists (sctlgpu_near_list_build) against the reference's own
BuildNearList outputs (golden) and the brute-force oracle: exact arrays
(the target-major order of one target's entries compared as a set, as the
reference's order there comes from an unstable sort), host and device
inputs, edge cases, determinism, and the torus evaluation on GPU-built pairs."""
import numpy as np
import pytest

from oracle import oracle as O
from sctl_gb300 import capi
from sctl_gb300 import workloads as W
from sctl_gb300.nearlist import NearList

from test_near_list_cpu import CASES, check_against, golden

pytestmark = pytest.mark.gpu


def build(d, device=False):
    if device:
        import torch
        t = {k: torch.from_numpy(v).cuda() for k, v in d.items()}
        return NearList(t["r_trg"], t["elem_nds_cnt"], t["elem_nds_dsp"], t["r_src"], t["src_radius"]).arrays(False)
    return NearList(d["r_trg"], d["elem_nds_cnt"], d["elem_nds_dsp"], d["r_src"], d["src_radius"]).arrays()


def oracle_list(d):
    pe, pt = O.near_pairs(d["r_trg"], d["elem_nds_cnt"], d["elem_nds_dsp"], d["r_src"], d["src_radius"])
    return O.near_list_from_pairs(pe, pt, d["r_trg"].shape[0], d["elem_nds_cnt"].size), pe


@pytest.mark.parametrize("kind,seed", CASES)
@pytest.mark.parametrize("device", [False, True])
def test_near_list_matches_reference_golden(cuda, kind, seed, device):
    d = W.near_list_case(kind, seed)
    got = build(d, device)
    check_against(got, golden(kind, seed))
    # ties inside one target's target-major entries are in element order here (stable)
    e_of = np.repeat(np.arange(d["elem_nds_cnt"].size), got["near_elem_cnt"])
    tm = e_of[got["near_scatter_index"]]
    for t in np.nonzero(got["near_trg_cnt"] > 1)[0][:500]:
        seg = tm[got["near_trg_dsp"][t]:got["near_trg_dsp"][t] + got["near_trg_cnt"][t]]
        assert np.all(np.diff(seg) > 0)
    np.testing.assert_array_equal(got["near_trg_elem"], tm)
    assert capi.load().sctlgpu_device_status(None) == capi.OK


def test_near_list_edge_cases(cuda):
    rng = np.random.default_rng(5)
    base = W.near_list_case("clusters", 1)
    # duplicate targets, targets far outside, a radius of 0, targets exactly on nodes
    xt = np.concatenate([base["r_trg"][:500], np.repeat(base["r_trg"][:3], 4, 0), [[50.0, -3.0, 7.0]],
                         base["r_src"][:20]])
    d = dict(base, r_trg=np.ascontiguousarray(xt))
    d["src_radius"] = d["src_radius"].copy()
    d["src_radius"][:10] = 0.0
    want, _ = oracle_list(d)
    got = build(d)
    for k in ("near_elem_cnt", "near_elem_dsp", "near_trg_idx", "near_trg_cnt", "near_trg_dsp"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    # no targets; no elements; all elements without nodes; a single element (no radix pass)
    e0 = dict(d, r_trg=np.zeros((0, 3)))
    assert NearList(**{k: e0[k] for k in ("r_trg", "elem_nds_cnt", "elem_nds_dsp", "r_src", "src_radius")}).n_near == 0
    z = np.zeros(0, np.int64)
    L = NearList(d["r_trg"], z, z, d["r_src"], d["src_radius"])
    assert L.n_near == 0 and np.all(L.arrays()["near_trg_cnt"] == 0)
    cnt0 = np.zeros_like(d["elem_nds_cnt"])
    L = NearList(d["r_trg"], cnt0, d["elem_nds_dsp"] * 0, d["r_src"], d["src_radius"])
    assert L.n_near == 0
    one = dict(r_trg=rng.uniform(0, 1, (3000, 3)), elem_nds_cnt=np.array([40]), elem_nds_dsp=np.array([0]),
               r_src=rng.uniform(0.4, 0.6, (40, 3)), src_radius=np.full(40, 0.1))
    want, _ = oracle_list(one)
    got = build(one)
    np.testing.assert_array_equal(got["near_trg_idx"], want["near_trg_idx"])
    np.testing.assert_array_equal(got["near_scatter_index"], np.arange(got["near_trg_idx"].size))
    assert capi.load().sctlgpu_device_status(None) == capi.OK


def test_near_list_deterministic(cuda):
    d = W.near_list_case("torus", 2)
    a, b = build(d), build(d, device=True)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_torus_evaluation_on_gpu_near_list(cuda):
    """Near pairs from the GPU near list drive the same evaluation: with node radius 1.5 panel
    sizes (a node-based radius needs more than the centre-based 1 size + panel radius; at 1.0
    the smooth rule's error above a panel's centre reaches 1.5e-8) Gauss's law holds to 1e-8."""
    torch = cuda
    from sctl_gb300.nearquad import PanelSurface
    from sctl_gb300.torus import Torus
    T = Torus(seed=0)
    S = PanelSurface(T.X, T.N, T.Q, T.size)
    tg = T.targets(3000, seed=17, hmin=1e-4, hmax=1.0)
    xt = torch.from_numpy(tg["r_trg"]).cuda()
    pairs = S.near_pairs_grid(xt, 1.5)
    one = torch.ones(T.np * 100, dtype=torch.float64, device="cuda")
    v = S.evaluate(xt, one, pairs=pairs).cpu().numpy()
    assert np.abs(v - np.where(tg["side"] < 0, -1.0, 0.0)).max() < 1e-8
