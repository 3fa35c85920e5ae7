"""Generates tests/golden/reference_ext.npz: the REFERENCE's own GenericKernel
Eval / KernelMatrix (oracle/_ref/libsctlref.so, `make -C oracle ref
REF=<checkout>`) for the twelve micro-kernels beyond the four hot-path ones
(kernel_functions.hpp:81-659), in FP64 and FP32.

    python tests/golden/make_ext_golden.py

Inputs are regenerated from `ext_case(kernel)` below (seeded); the Helmholtz
kernels use the wavenumber MU.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

MU = 2.5
KERNELS = range(4, 16)


def ext_case(k, nt=523, ns=411, seed=0):
    """Targets and sources uniform in [-1, 1]^3 (the first 3 targets on sources: masked pairs),
    random normals, N(0,1) densities."""
    rng = np.random.default_rng(1000 + k + seed)
    nd, sd, td = O.DIMS[k]
    xs = rng.uniform(-1, 1, (ns, 3))
    xt = rng.uniform(-1, 1, (nt, 3))
    xt[:3] = xs[:3]
    n = rng.normal(size=(ns, 3)) if nd else np.zeros((0, 3))
    f = rng.normal(size=ns * sd)
    return xt.reshape(-1), xs.reshape(-1), n.reshape(-1), f


def main():
    out = {"mu": np.array(MU)}
    for k in KERNELS:
        xt, xs, n, f = ext_case(k)
        nn = n if n.size else None
        for prec in ("f64", "f32"):
            out[f"{k}/eval_{prec}"] = O.ref_eval(k, xt, xs, nn, f, precision=prec, mu=MU)
        out[f"{k}/eval_f64_d6"] = O.ref_eval(k, xt, xs, nn, f, digits=6, precision="f64", mu=MU)
        xt2, xs2, n2, _ = ext_case(k, nt=20, ns=25, seed=1)
        out[f"{k}/kmat_f64"] = O.ref_kernel_matrix(k, xt2, xs2, n2 if n2.size else None, mu=MU)
        print(k, "ok")
    np.savez_compressed(os.path.join(HERE, "reference_ext.npz"), **out)


if __name__ == "__main__":
    main()
