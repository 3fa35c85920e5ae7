"""Boundary-integral evaluation on a panel surface: smooth far field plus
near-singular panel corrections -- BoundaryIntegralOp::ComputePotential
(boundary_integral.txx:716-722) with its two halves,

* far field: every node is a source with weight Q (ComputeFarField,
  :1248-1309: F_far = F * wts, then the direct sum), evaluated by
  `sctlgpu_eval`;
* near field: for every (target, panel) pair from the GPU near list (target
  within `near_factor` panel sizes of one of the panel's nodes, BuildNearList's
  test, :50-522), the panel's accurate contribution minus its smooth-rule part
  (SetupNear / ComputeNearInterac, :927-1381), evaluated by
  `sctlgpu_panel_near_correction` (adaptive refinement) or applied from stored
  near matrices.

All arrays are torch tensors on the GPU used as plain device buffers; every
kernel of an evaluation is one of libsctlgpu's.
"""
from __future__ import annotations

import numpy as np
import torch

from . import capi


class PanelSurface:
    def __init__(self, X, N, Q, size, device="cuda"):
        """X, N: (np, p*p, 3) node coordinates and unit normals; Q: (np, p*p) smooth weights;
        size: (np,) panel sizes (near-field radius unit).  Host arrays; everything derived from
        them is computed on the host and uploaded once."""
        X, N, Q, size = (np.ascontiguousarray(a, np.float64) for a in (X, N, Q, size))
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=device)  # noqa: E731
        self.X, self.N, self.Q, self.size = t(X), t(N), t(Q), t(size)
        self.np, self.nn = X.shape[0], X.shape[1]
        self.negQ = t(-Q.reshape(-1))  # smooth-rule weights of the subtraction plan
        # near list inputs (BuildNearList): every node of panel P carries the radius near_factor * size_P
        self._elem_cnt = torch.as_tensor(np.full(self.np, self.nn, np.int64), device=device)
        self._elem_dsp = torch.as_tensor(np.arange(self.np, dtype=np.int64) * self.nn, device=device)
        self._node_size = np.repeat(size, self.nn)
        self._node_rad = {}

    # ------------------------------------------------------------ near list
    def near_pairs(self, r_trg, near_factor=1.5):
        """(target, panel) pairs from the GPU near list (`NearList`, BuildNearList's test,
        boundary_integral.txx:50-522): a target is near a panel when it lies within
        near_factor * size_P of one of the panel's nodes (1.5 keeps the 10 x 10 smooth rule's error
        below 1e-8 for every other target; at 1.0 it reaches 1.5e-8 above a panel's centre).
        Sorted by panel, then target; both arrays int64 on the device."""
        import ctypes

        from .nearlist import NearList
        xt = r_trg.reshape(-1).contiguous()
        rad = self._node_rad.get(near_factor)
        if rad is None:
            rad = self._node_rad[near_factor] = torch.as_tensor(near_factor * self._node_size, device=xt.device)
        L = NearList(xt, self._elem_cnt, self._elem_dsp, self.X.reshape(-1), rad)
        n = L.n_near
        t = torch.empty(max(n, 1), dtype=torch.int64, device=xt.device)
        p = torch.empty(max(n, 1), dtype=torch.int64, device=xt.device)
        lib = capi.load()
        stream = torch.cuda.current_stream().cuda_stream
        capi.check(lib.sctlgpu_near_list_get(L._h, None, None, t.data_ptr(), None, None, None, None, stream),
                   "sctlgpu_near_list_get")
        capi.check(lib.sctlgpu_near_list_elem_index(L._h, ctypes.c_void_p(p.data_ptr()), stream),
                   "sctlgpu_near_list_elem_index")
        L.close()
        return t[:n], p[:n]

    # the name of the GPU near-list search before the brute-force form was retired
    near_pairs_grid = near_pairs

    # ------------------------------------------------------------ far field
    def far_field(self, r_trg, sigma, kernel=1, mode="mixed", digits=10, out=None, method="direct"):
        """ComputeFarField (boundary_integral.txx:1248-1309): F_far = sigma * Q on the device
        (`sctlgpu_far_densities`), then the sum over every node -- one direct sum
        (method="direct", ParticleFMM::EvalDirect) or the treecode (method="treecode", the fast
        path ParticleFMM::Eval takes for 40,000 targets or more; its trees are kept per target
        array); added into `out` when it is given, else written to a new array."""
        xt = r_trg.reshape(-1)
        nt = xt.numel() // 3
        src = self.X.reshape(-1)
        nrm = self.N.reshape(-1)
        lib = capi.load()
        stream = torch.cuda.current_stream().cuda_stream
        sig = sigma.reshape(-1).contiguous()
        f = torch.empty_like(sig)
        capi.check(lib.sctlgpu_far_densities(self.np * self.nn, sig.numel() // (self.np * self.nn), sig.data_ptr(),
                                             self.Q.data_ptr(), f.data_ptr(), stream), "far densities")
        accumulate = out is not None
        if out is None:
            out = torch.empty(nt * (3 if kernel >= 2 else 1), dtype=torch.float64, device=xt.device)
        if method == "treecode":
            return self.treecode(xt, kernel, mode, digits).eval(f, out=out, accumulate=accumulate)
        if method != "direct":
            raise ValueError(f"unknown far-field method {method!r}")
        flags = capi.DEVICE_PTRS | (capi.ACCUMULATE if accumulate else 0)
        capi.check(lib.sctlgpu_eval(kernel, capi.MODE_IDS[mode], digits, nt, xt.data_ptr(), src.numel() // 3,
                                    src.data_ptr(), nrm.data_ptr() if kernel in (1, 3) else None,
                                    f.data_ptr(), out.data_ptr(), flags, stream), "far field")
        return out

    def treecode(self, r_trg, kernel=1, mode="mixed", digits=10):
        """The far-field treecode of these nodes and targets (built on first use; the geometry
        calls of ParticleFMM, SetSrcCoord / SetTrgCoord, fmm-wrapper.txx:505-540)."""
        from .treecode import Treecode
        xt = r_trg.reshape(-1)
        # the cached trees hold a reference to their target array (its storage cannot be reused
        # while cached) and are rebuilt when the array is written in place (its version changes)
        key = (xt.data_ptr(), xt.numel(), xt._version, kernel, mode, digits)
        if getattr(self, "_tc_key", None) != key:
            self._tc = Treecode(kernel, self.X.reshape(-1), xt, n_src=self.N.reshape(-1) if kernel in (1, 3) else None,
                                digits=digits, mode=mode)
            self._tc_key, self._tc_trg = key, xt
        return self._tc

    # ------------------------------------------------------------ near field
    def near_correction(self, r_trg, sigma, pairs, kernel=1, alpha=1.0, max_depth=22, out=None,
                        subtract_smooth=True):
        """Adaptive near-singular integral of every (target, panel) pair, minus (optionally) the
        panel's smooth-rule part in FP64."""
        xt = r_trg.reshape(-1).contiguous()
        nt = xt.numel() // 3
        t, p = pairs
        sig = sigma.reshape(self.np, self.nn).contiguous()
        if out is None:
            out = torch.zeros(nt, dtype=torch.float64, device=xt.device)
        stream = torch.cuda.current_stream().cuda_stream
        capi.check(capi.load().sctlgpu_panel_near_correction(
            kernel, t.numel(), t.data_ptr(), p.data_ptr(), nt, xt.data_ptr(), self.np, self.X.data_ptr(),
            self.N.data_ptr(), self.Q.data_ptr(), sig.data_ptr(), None, -1, float(alpha), int(max_depth),
            1 if subtract_smooth else 0, out.data_ptr(), stream), "near correction")
        return out

    def smooth_subtraction_plan(self, nt, pairs, kernel=1, mode="mixed", digits=10):
        """Near plan that subtracts each near panel's smooth-rule part in the arithmetic and
        coordinate frame of the far field (blocks: panel nodes x that panel's near list)."""
        from .near import NearPlan
        t, p = (a.cpu().numpy() for a in pairs)
        counts = np.bincount(p, minlength=self.np)
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
        live = np.nonzero(counts)[0]
        blocks = np.stack([live * self.nn, np.full(live.size, self.nn), starts[live], counts[live]], 1)
        return NearPlan(kernel, blocks, self.np * self.nn, nt, mode=mode, digits=digits, trg_index=t)

    def near_matrix(self, r_trg, pairs, kernel=1, alpha=1.0, max_depth=22, float_pairs=True):
        """SetupNear's precomputation for repeated applications (e.g. every iteration of an
        iterative solver): the accurate weights of every (target, panel) pair, see NearMatrix."""
        return NearMatrix(self, r_trg, pairs, kernel, alpha, max_depth, float_pairs)

    def evaluate(self, r_trg, sigma, kernel=1, mode="mixed", digits=10, near_factor=1.5, alpha=1.0, pairs=None,
                 plan=None, matrix=None, far="direct"):
        """Far field (smooth rule over every node) + near corrections.  The smooth part of the near
        panels is subtracted with a near plan in the far field's arithmetic, so the large
        near-singular smooth terms cancel exactly as in the reference's FP64 flow.  With `matrix`
        (a NearMatrix of the same pairs) the accurate near part is applied from the stored
        weights instead of being integrated again.  `far` selects the far-field summation
        ("direct" or "treecode")."""
        xt = r_trg.reshape(-1).contiguous()
        out = self.far_field(xt, sigma, kernel, mode, digits, method=far)
        if pairs is None:
            pairs = self.near_pairs(xt, near_factor)
        if plan is None:
            plan = self.smooth_subtraction_plan(xt.numel() // 3, pairs, kernel, mode, digits)
        plan.execute(xt, self.X.reshape(-1), self.N.reshape(-1), sigma.reshape(-1).contiguous(), out,
                     w_src=self.negQ, accumulate=True)
        if matrix is not None:
            matrix.apply(sigma, out)
        else:
            self.near_correction(xt, sigma, pairs, kernel, alpha, out=out, subtract_smooth=False)
        return out


class NearMatrix:
    """Precomputed near interactions of a panel surface (SetupNear, boundary_integral.txx:927-1241,
    with the NearInterac weights of every pair) and their application (ComputeNearInterac,
    :1311-1381) by `sctlgpu_near_matrix_apply`.

    Blocks are stored element-major like the reference's K_near: pair j (panel p_j, target t_j)
    owns the 100 accurate weights W_j = scale * int K(x_t - y) l_a l_b dA (adaptive quadrature,
    `sctlgpu_panel_near_weights`).  The target-major order in which each target's pairs are
    summed (the reference's near_trg_dsp and scatter order) is a stable sort by target.  With
    `pairs` (default) the FP64 weights are converted in place to float pairs after the setup
    and applied in double-float by `sctlgpu_near_matrix_apply_pairs` (the HBM-bound form on
    GB300, whose FP64 pipe cannot keep up with the weights); otherwise in FP64."""

    def __init__(self, S: PanelSurface, r_trg, pairs, kernel=1, alpha=1.0, max_depth=22, float_pairs=True):
        xt = r_trg.reshape(-1).contiguous()
        self.nt = xt.numel() // 3
        t, p = pairs
        self.n_pairs, self.nn, self.np = int(t.numel()), S.nn, S.np
        dev = xt.device
        self.W = torch.empty(self.n_pairs, S.nn, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream().cuda_stream
        if self.n_pairs:
            capi.check(capi.load().sctlgpu_panel_near_weights(
                kernel, self.n_pairs, t.data_ptr(), p.data_ptr(), self.nt, xt.data_ptr(), S.np, S.X.data_ptr(),
                float(alpha), int(max_depth), self.W.data_ptr(), stream), "panel_near_weights")
        self.float_pairs = bool(float_pairs)
        if self.float_pairs and self.n_pairs:
            capi.check(capi.load().sctlgpu_to_float_pairs(self.W.numel(), self.W.data_ptr(), self.W.data_ptr(),
                                                          stream), "to_float_pairs")
        self.trg_pair = torch.argsort(t, stable=True).contiguous()
        counts = torch.bincount(t, minlength=self.nt)
        self.trg_dsp = torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), counts.cumsum(0)]).contiguous()
        self.pair_elem = p.contiguous()
        self.pair_kdsp = (torch.arange(self.n_pairs, dtype=torch.int64, device=dev) * S.nn).contiguous()
        self.elem_nds_dsp = (torch.arange(S.np, dtype=torch.int64, device=dev) * S.nn).contiguous()
        self.elem_nds_cnt = torch.full((S.np,), S.nn, dtype=torch.int64, device=dev)
        # the index chain (target-major entry -> pair -> element -> nodes) resolved once
        self.resolved = torch.empty(2 * max(self.n_pairs, 1), dtype=torch.int64, device=dev)
        capi.check(capi.load().sctlgpu_near_matrix_resolve(
            1, 1, self.n_pairs, self.trg_pair.data_ptr(), self.n_pairs, self.pair_elem.data_ptr(),
            self.pair_kdsp.data_ptr(), self.np, self.elem_nds_dsp.data_ptr(), self.elem_nds_cnt.data_ptr(),
            self.W.numel(), S.np * S.nn, self.resolved.data_ptr(), stream), "near_matrix_resolve")

    @property
    def nbytes(self):
        """Bytes one application reads from the stored blocks (the HBM-bound part)."""
        return self.W.numel() * 8

    def apply(self, sigma, out):
        """out[t] += sum over t's near pairs of W_j . sigma[panel_j] (from the resolved entries)."""
        f = sigma.reshape(-1).contiguous()
        w = self.W.data_ptr()
        capi.check(capi.load().sctlgpu_near_matrix_apply_resolved(
            1, 1, self.nt, self.trg_dsp.data_ptr(), self.n_pairs, self.resolved.data_ptr(), self.W.numel(),
            None if self.float_pairs else w, w if self.float_pairs else None, f.numel(), f.data_ptr(),
            out.data_ptr(), torch.cuda.current_stream().cuda_stream), "near_matrix_apply")
        return out

    def apply_unresolved(self, sigma, out):
        """The same through the index chain (sctlgpu_near_matrix_apply[_pairs], the reference's arrays)."""
        f = sigma.reshape(-1).contiguous()
        fn = capi.load().sctlgpu_near_matrix_apply_pairs if self.float_pairs else capi.load().sctlgpu_near_matrix_apply
        capi.check(fn(
            1, 1, self.nt, self.trg_dsp.data_ptr(), self.n_pairs, self.trg_pair.data_ptr(), self.n_pairs,
            self.pair_elem.data_ptr(), self.pair_kdsp.data_ptr(), self.np, self.elem_nds_dsp.data_ptr(),
            self.elem_nds_cnt.data_ptr(), self.W.numel(), self.W.data_ptr(), f.numel(), f.data_ptr(),
            out.data_ptr(), torch.cuda.current_stream().cuda_stream), "near_matrix_apply")
        return out
