"""Generates the golden fixtures in this directory by running the REFERENCE's own
GenericKernel::Eval / KernelMatrix (header-only SCTL, wrapped by
oracle/ref_driver.cpp and built with `make -C oracle ref REF=<checkout>`).

    python tests/golden/make_golden.py [--ref /path/to/sctl]

Inputs are regenerated from the seeds stored in each fixture, so only the
reference's outputs (and the small deterministic inputs) are committed.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from sctl_gb300 import workloads as W  # noqa: E402

NAMES = ["Laplace3D_FxU", "Laplace3D_DxU", "Stokes3D_FxU", "Stokes3D_DxU"]


def small_deterministic(k):
    """The 7-source x 5-target inputs of src/test-kernel_functions.cpp:491-499."""
    nd, sd, td = O.DIMS[k]
    Ns, Nt = 7, 5
    Xs = np.array([0.1 * (i + 1) - 0.35 for i in range(Ns * 3)])
    Vs = np.array([0.3 * (i % 5) - 0.4 for i in range(Ns * sd)])
    Xt = np.array([1.7 + 0.2 * i for i in range(Nt * 3)])
    Xn = np.tile([0.0, 1.0, 0.0], Ns) if nd else np.zeros(0)
    return Xt, Xs, Xn, Vs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("SCTL_REF", os.path.join(ROOT, "baseline", "_ref")),
                    help="installed reference (oracle/install_ref.sh fills baseline/_ref)")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.ref}"], check=True)
    meta = {"reference_veclen_f64": O.ref().ref_vec_len(1), "reference_veclen_f32": O.ref().ref_vec_len(0),
            "generator": "tests/golden/make_golden.py", "cases": {}}
    out = {}
    for k, name in enumerate(NAMES):
        nd, sd, td = O.DIMS[k]
        # 1) the reference test's deterministic 7x5 inputs: Eval and KernelMatrix
        Xt, Xs, Xn, Vs = small_deterministic(k)
        out[f"{name}/small/Xt"], out[f"{name}/small/Xs"], out[f"{name}/small/Xn"], out[f"{name}/small/Vs"] = Xt, Xs, Xn, Vs
        out[f"{name}/small/eval_f64"] = O.ref_eval(k, Xt, Xs, Xn, Vs, digits=-1)
        out[f"{name}/small/kmat_f64"] = O.ref_kernel_matrix(k, Xt, Xs, Xn)
        out[f"{name}/small/eval_f32"] = O.ref_eval(k, Xt, Xs, Xn, Vs, digits=-1, precision="f32")
        # 2) seeded sphere/ball inputs, ragged sizes (not multiples of any tile)
        for tag, (ns, nt, seed) in {"ragged": (1531, 997, 11), "one_target": (300, 1, 12)}.items():
            d = W.sphere_ball(ns, nt, k, seed)
            for digits in (-1, 6, 10):
                out[f"{name}/{tag}/eval_f64_d{digits}"] = O.ref_eval(k, d["r_trg"], d["r_src"], d["n_src"],
                                                                    d["v_src"], digits=digits)
            out[f"{name}/{tag}/eval_f32"] = O.ref_eval(k, d["r_trg"].astype(np.float32),
                                                        d["r_src"].astype(np.float32),
                                                        d["n_src"].astype(np.float32),
                                                        d["v_src"].astype(np.float32), digits=-1, precision="f32")
            meta["cases"][f"{name}/{tag}"] = {"generator": "sphere_ball", "n_src": ns, "n_trg": nt, "seed": seed}
        # 3) kernel matrix on seeded inputs
        d = W.sphere_ball(40, 50, k, 13)
        out[f"{name}/kmat40x50/kmat_f64"] = O.ref_kernel_matrix(k, d["r_trg"], d["r_src"], d["n_src"])
        meta["cases"][f"{name}/kmat40x50"] = {"generator": "sphere_ball", "n_src": 40, "n_trg": 50, "seed": 13}
    # 4) the 8192 x 8192 unit-cube Laplace FxU case, FP64 digits 14, seed 0
    d = W.cube(8192, 8192, 0, 0)
    out["Laplace3D_FxU/cube8192/eval_f64_d14"] = O.ref_eval(0, d["r_trg"], d["r_src"], d["n_src"], d["v_src"],
                                                            digits=14)
    meta["cases"]["Laplace3D_FxU/cube8192"] = {"generator": "cube", "n_src": 8192, "n_trg": 8192, "seed": 0}
    np.savez_compressed(os.path.join(HERE, "reference_eval.npz"), **out)
    with open(os.path.join(HERE, "reference_eval.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
