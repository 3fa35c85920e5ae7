"""The oracle's restatement of the twelve micro-kernels beyond the hot-path four
(kernel_functions.hpp:81-659) pinned against the reference's own Eval and
KernelMatrix outputs (tests/golden/reference_ext.npz, made by
tests/golden/make_ext_golden.py)."""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_ext_golden import KERNELS, MU, ext_case  # noqa: E402

GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_ext.npz"))


@pytest.mark.parametrize("k", KERNELS)
def test_oracle_ext_matches_reference(k):
    xt, xs, n, f = ext_case(k)
    nn = n if n.size else None
    assert O.rel_l2(O.eval(k, xt, xs, nn, f, mu=MU), GOLDEN[f"{k}/eval_f64"]) < 1e-13
    assert O.rel_l2(O.eval(k, xt, xs, nn, f, precision="ld", mu=MU), GOLDEN[f"{k}/eval_f64"]) < 1e-13
    assert O.rel_l2(O.eval(k, xt, xs, nn, f, precision="f32", mu=MU), GOLDEN[f"{k}/eval_f32"]) < 2e-6
    xt2, xs2, n2, _ = ext_case(k, nt=20, ns=25, seed=1)
    M = O.kernel_matrix(k, xt2, xs2, n2 if n2.size else None, mu=MU)
    want = GOLDEN[f"{k}/kmat_f64"]
    assert np.abs(M - want).max() <= 1e-13 * np.abs(want).max()
    # the masked pairs (targets 0-2 sit on sources 0-2) contribute nothing
    assert np.all(M[:O.DIMS[k][1], :O.DIMS[k][2]] == 0)
