"""Near lists (BuildNearList, boundary_integral.txx:50-522): the oracle's
brute-force restatement pinned against the reference's own outputs
(tests/golden/near_list.npz, made by tests/golden/make_near_golden.py from the
reference's BuildNearList), and the C ABI's argument checks (no GPU)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from sctl_gb300 import capi
from sctl_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "near_list.npz")
CASES = [("clusters", 0), ("torus", 0), ("many", 3)]


def segment_sorted(scatter, cnt, dsp):
    """The reference orders one target's entries by an unstable sort on the target index
    (SortPair compares the key only, comm.hpp:604): compare each target's entries as a set."""
    out = scatter.copy()
    for t in np.nonzero(cnt)[0]:
        out[dsp[t]:dsp[t] + cnt[t]] = np.sort(scatter[dsp[t]:dsp[t] + cnt[t]])
    return out


def check_against(got, want):
    for k in ("near_elem_cnt", "near_elem_dsp", "near_trg_idx", "near_trg_cnt", "near_trg_dsp"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    np.testing.assert_array_equal(segment_sorted(got["near_scatter_index"], got["near_trg_cnt"], got["near_trg_dsp"]),
                                  segment_sorted(want["near_scatter_index"], want["near_trg_cnt"],
                                                 want["near_trg_dsp"]))


def golden(kind, seed):
    g = np.load(GOLDEN)
    tag = f"{kind}_{seed}"
    return {k: g[f"{tag}/{k}"] for k in ("near_elem_cnt", "near_elem_dsp", "near_trg_idx", "near_scatter_index",
                                        "near_trg_cnt", "near_trg_dsp")}


@pytest.mark.parametrize("kind,seed", CASES)
def test_oracle_matches_reference_golden(kind, seed):
    d = W.near_list_case(kind, seed)
    pe, pt = O.near_pairs(d["r_trg"], d["elem_nds_cnt"], d["elem_nds_dsp"], d["r_src"], d["src_radius"])
    got = O.near_list_from_pairs(pe, pt, d["r_trg"].shape[0], d["elem_nds_cnt"].size)
    check_against(got, golden(kind, seed))


@pytest.mark.skipif(not O.ref_available(), reason="reference wrapper not built here")
def test_oracle_matches_reference_live():
    rng = np.random.default_rng(11)
    ne = 150
    cnt = rng.integers(1, 6, ne)
    dsp = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    xs = rng.uniform(0, 1, (int(cnt.sum()), 3))
    rad = rng.uniform(0, 0.1, int(cnt.sum()))
    xt = rng.uniform(-0.1, 1.1, (2000, 3))
    pe, pt = O.near_pairs(xt, cnt, dsp, xs, rad)
    got = O.near_list_from_pairs(pe, pt, 2000, ne)
    r = O.ref_near_list(xt, cnt, dsp, xs, rad)
    np.testing.assert_array_equal(xt[got["near_trg_idx"]], r["xtrg_near"])
    r["near_trg_idx"] = got["near_trg_idx"]
    check_against(got, r)


def test_near_list_argument_errors_without_gpu():
    import ctypes
    lib = capi.load()
    h = ctypes.c_void_p()
    x = np.zeros(6)
    c = np.zeros(2, np.int64)
    p, q = x.ctypes.data, c.ctypes.data
    assert lib.sctlgpu_near_list_build(None, 1, p, 1, q, q, 1, p, p, 0, None) == capi.ERR_NULL_POINTER
    assert lib.sctlgpu_near_list_build(ctypes.byref(h), -1, p, 1, q, q, 1, p, p, 0, None) == capi.ERR_INVALID_SIZE
    assert lib.sctlgpu_near_list_build(ctypes.byref(h), 1, None, 1, q, q, 1, p, p, 0, None) == capi.ERR_NULL_POINTER
    assert lib.sctlgpu_near_list_build(ctypes.byref(h), 1, p, 1, q, q, 1, p, None, 0, None) == capi.ERR_NULL_POINTER
    assert lib.sctlgpu_near_list_build(ctypes.byref(h), 1, p, 1, q, q, 1, p, p, 8, None) == \
        capi.ERR_INVALID_ARGUMENT
    assert lib.sctlgpu_near_list_sizes(None, None, None, None) == capi.ERR_NULL_POINTER
    assert lib.sctlgpu_near_list_destroy(None) == capi.OK
