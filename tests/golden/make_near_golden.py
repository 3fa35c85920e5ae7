"""Generates tests/golden/near_list.npz by running the REFERENCE's own
BuildNearList<double,3> (boundary_integral.txx:50-522, one rank) through
oracle/_ref/libsctlref.so (`make -C oracle ref REF=<checkout>`).

    python tests/golden/make_near_golden.py

Inputs are regenerated from sctl_gb300.workloads.near_list_case(kind, seed); the
reference's outputs are stored with Xtrg_near as target indices (targets are
distinct points, so the coordinates identify them).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from sctl_gb300 import workloads as W  # noqa: E402

CASES = [("clusters", 0), ("torus", 0), ("many", 3)]


def main():
    out = {}
    for kind, seed in CASES:
        d = W.near_list_case(kind, seed)
        r = O.ref_near_list(d["r_trg"], d["elem_nds_cnt"], d["elem_nds_dsp"], d["r_src"], d["src_radius"])
        index = {tuple(x): i for i, x in enumerate(d["r_trg"])}
        assert len(index) == d["r_trg"].shape[0]
        trg_idx = np.array([index[tuple(x)] for x in r["xtrg_near"]], np.int64)
        tag = f"{kind}_{seed}"
        out[f"{tag}/near_trg_idx"] = trg_idx
        for k in ("near_elem_cnt", "near_elem_dsp", "near_scatter_index", "near_trg_cnt", "near_trg_dsp"):
            out[f"{tag}/{k}"] = r[k]
        print(tag, "near entries", trg_idx.size)
    np.savez_compressed(os.path.join(HERE, "near_list.npz"), **out)


if __name__ == "__main__":
    main()
