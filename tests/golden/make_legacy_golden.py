"""Generates tests/golden/legacy_torus_dl.npz: the near-singular Laplace
double-layer potential of the torus workload computed by the REFERENCE's own
legacy boundary quadrature (sctl::Quadrature, boundary_quadrature.hpp:362-1827,
built from the installed reference by `make -C oracle legacy`, see
oracle/legacy_quad.cpp for the three interface gaps it bridges).

    python tests/golden/make_legacy_golden.py

Surface and density: sctl_gb300.torus.Torus(seed=0) -- 64 x 32 panels of
10 x 10 Chebyshev nodes, R = 1, r = 0.3, the Fourier-mode density.  Targets:
Torus.targets(256, seed=21, hmin=1e-4, hmax=1) (off-surface distances
log-uniform in [1e-4, 1] panel sizes, either side).  Quadrature orders
(order_singular, order_direct) = (32, 48): against the CPU restatement
(oracle/panel_oracle.py, exact to rounding) the legacy values then agree to
4.5e-11 at worst on 8 targets from 7e-4 to 0.3 panel sizes; with (24, 24) the
legacy's direct part is short of points at 0.1-0.3 panel sizes and errs by up
to 2.6e-6, with (24, 40) by 3e-10.  Only the potentials are stored; inputs are
regenerated.

The legacy rule integrates a panel adjacent to a near-edge target with its
plain direct rule once the target is outside its near-singular radius; there
48 points per direction are not enough (2.3e-5 at a target 0.063 panel sizes
off the surface and 0.033 of a panel from an edge; 4.8e-7 with 64).  The
golden therefore also holds the values with order_direct = 64: where the two
agree to 1e-11 the legacy value is exact to its rounding, elsewhere their
difference is its error estimate.
"""
from __future__ import annotations

import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from sctl_gb300.torus import Torus  # noqa: E402

N_TRG, SEED, ORDERS = 256, 21, (32, 48)


def legacy_potential(T, xt, orders=ORDERS, green=False):
    exe = os.path.join(ROOT, "oracle", "_ref", "legacy_quad")
    with tempfile.TemporaryDirectory() as tmp:
        fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("qqddqq", T.n_theta, T.n_phi, 1.0, 0.3, *orders))
            f.write(np.ascontiguousarray(T.sigma.reshape(-1), np.float64).tobytes())
            f.write(struct.pack("q", xt.shape[0]))
            f.write(np.ascontiguousarray(xt, np.float64).tobytes())
        subprocess.run([exe, fin, fout] + (["green"] if green else []), check=True)
        out = np.fromfile(fout)
    return out[:xt.shape[0]], out[xt.shape[0]]


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "legacy"], check=True)
    T = Torus(seed=0)
    tg = T.targets(N_TRG, seed=SEED, hmin=1e-4, hmax=1.0)
    U, _ = legacy_potential(T, tg["r_trg"])
    # the same with a denser rule for the parts it integrates directly: where the two agree the
    # legacy value is trusted to its rounding; where not, their difference bounds its own error
    U64, _ = legacy_potential(T, tg["r_trg"], orders=(ORDERS[0], 64))
    # the legacy test's Green's identity at cheaper orders (at the golden's orders it runs for hours)
    _, green = legacy_potential(T, tg["r_trg"][:1], orders=(16, 16), green=True)
    np.savez_compressed(os.path.join(HERE, "legacy_torus_dl.npz"), U=U, U_direct64=U64)
    meta = {"generator": "tests/golden/make_legacy_golden.py", "torus_seed": 0, "n_trg": N_TRG, "target_seed": SEED,
            "hmin": 1e-4, "hmax": 1.0, "orders": list(ORDERS),
            "legacy_greens_identity_max_err_orders_16_16": green,
            "targets_where_orders_48_and_64_agree_to_1e-11": int((abs(U - U64) <= 1e-11).sum())}
    with open(os.path.join(HERE, "legacy_torus_dl.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
