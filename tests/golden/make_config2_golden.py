"""Generates tests/golden/reference_config2.npz: the REFERENCE's own
GenericKernel::Eval<Real,true> (oracle/_ref/libsctlref_hot.so, built by
`make -C oracle hot` from the reference installed in baseline/_ref) on the
sphere/ball workload at full source count -- 2^20 sources on the unit sphere
(outward normals), a 256-target sample of the radius-2 ball -- for
Laplace3D_DxU, Stokes3D_FxU and Stokes3D_DxU, in FP64 and FP32, at digits
6, 10 and 14 (and FP64 at full digits, the oracle the errors are measured
against).  Also the reference's FP32 Eval at full digits on a source-count
sweep (2^10 .. 2^20 sources, the same 256 targets) to locate the N at which the
FP32 forms agree to 1e-6.

    python tests/golden/make_config2_golden.py

Inputs are regenerated from sctl_gb300.workloads.sphere_ball(n_src, 256,
kernel, seed) with the seeds stored below; only outputs are committed.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from sctl_gb300 import workloads as W  # noqa: E402

NAMES = {1: "Laplace3D_DxU", 2: "Stokes3D_FxU", 3: "Stokes3D_DxU"}
N_SRC = 1 << 20
N_TRG = 256
SEED = 200  # + kernel id
DIGITS = (6, 10, 14)
SWEEP = tuple(1 << e for e in range(10, 21, 2))


def f32(a):
    return np.asarray(a, np.float32)


def main():
    out, meta = {}, {"generator": "tests/golden/make_config2_golden.py", "n_src": N_SRC, "n_trg": N_TRG,
                     "seed_base": SEED, "digits": list(DIGITS), "sweep_n_src": list(SWEEP), "cases": {}}
    for k, name in NAMES.items():
        d = W.sphere_ball(N_SRC, N_TRG, k, SEED + k)
        args = (d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
        out[f"{name}/f64_d-1"] = O.ref_hot_eval(k, *args, digits=-1)
        for dg in DIGITS:
            out[f"{name}/f64_d{dg}"] = O.ref_hot_eval(k, *args, digits=dg)
            out[f"{name}/f32_d{dg}"] = O.ref_hot_eval(k, *map(f32, args), digits=dg, precision="f32")
        for ns in SWEEP:
            s = W.sphere_ball(ns, N_TRG, k, SEED + k)
            sa = (s["r_trg"], s["r_src"], s["n_src"], s["v_src"])
            out[f"{name}/sweep{ns}/f64_d-1"] = O.ref_hot_eval(k, *sa, digits=-1)
            out[f"{name}/sweep{ns}/f32_d-1"] = O.ref_hot_eval(k, *map(f32, sa), digits=-1, precision="f32")
            meta["cases"][f"{name}/sweep{ns}"] = {
                "ref_f32_vs_ref_f64_rel_l2": O.rel_l2(out[f"{name}/sweep{ns}/f32_d-1"],
                                                      out[f"{name}/sweep{ns}/f64_d-1"])}
        meta["cases"][name] = {dg: {"ref_f64_vs_oracle": O.rel_l2(out[f"{name}/f64_d{dg}"], out[f"{name}/f64_d-1"]),
                                    "ref_f32_vs_oracle": O.rel_l2(out[f"{name}/f32_d{dg}"], out[f"{name}/f64_d-1"])}
                               for dg in DIGITS}
        print(name, json.dumps(meta["cases"][name]))
    meta["reference_veclen_f64"] = O.ref().ref_vec_len(1) if O.ref_available() else None
    np.savez_compressed(os.path.join(HERE, "reference_config2.npz"), **out)
    with open(os.path.join(HERE, "reference_config2.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
