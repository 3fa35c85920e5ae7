"""Learned near-singular quadrature: a small MLP predicts the 100 accurate
weights W_ab(t) = int_P K(x_t - y) l_a(s) l_b(t) dA(y) of a (target, panel)
pair from the target's local coordinates (s, t, h) and 12 panel-geometry
features; the pair's correction is then sum_ab (W_ab - W^smooth_ab) sigma_ab.

* Labels come from the adaptive quadrature (`sctlgpu_panel_near_weights`).
* Training and inference run on the tcgen05 kernels of libsctlgpu
  (`sctlgpu_mlp_*`): BF16 weights and activations, FP32 accumulation.
* The networks may learn the weights minus a known near-singular part (solid
  angle x density frozen at the foot point, `torus.singular_part`).
* Two networks trained from different seeds and a calibrated error model form
  the a-posteriori check: a pair is accepted only when it is inside the trained
  range, the networks' predicted corrections agree to the tolerance, and the
  calibrated bound on its error (held-out weight errors at its distance times
  the panel density, see `LearnedCorrection.error_bound`) is below the
  tolerance; every other pair takes the plain adaptive path.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi

IN_DIM, OUT_DIM = 15, 100


class MLP:
    """in -> 256 -> 256 -> 256 -> out network living on the GPU (libsctlgpu)."""

    def __init__(self, in_dim=IN_DIM, out_dim=OUT_DIM, max_batch=1 << 14, seed=0):
        self.in_dim, self.out_dim, self.max_batch = in_dim, out_dim, max_batch
        h = ctypes.c_void_p()
        capi.check(capi.load().sctlgpu_mlp_create(ctypes.byref(h), in_dim, out_dim, max_batch, seed), "mlp_create")
        self._h = h
        self.n_params = int(capi.load().sctlgpu_mlp_num_params(h))

    def close(self):
        if getattr(self, "_h", None):
            capi.load().sctlgpu_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        capi.check(capi.load().sctlgpu_mlp_get_params(self._h, out.ctypes.data), "mlp_get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        capi.check(capi.load().sctlgpu_mlp_set_params(self._h, p.ctypes.data), "mlp_set_params")

    def layers(self, p=None):
        """Split the flat parameters into [(W, b)] with W (N x K) as stored."""
        p = self.get_params() if p is None else p
        dims = [(256, 64), (256, 256), (256, 256), (128, 256)]
        out, o = [], 0
        for n, k in dims:
            W = p[o:o + n * k].reshape(n, k)
            o += n * k
            b = p[o:o + n]
            o += n
            out.append((W, b))
        return out

    def _pad(self, x):
        B = x.shape[0]
        Bp = (B + 127) // 128 * 128
        if Bp != B:
            x = torch.cat([x, torch.zeros(Bp - B, x.shape[1], dtype=x.dtype, device=x.device)])
        return x.contiguous(), B, Bp

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        """x: (B, in_dim) FP32 CUDA -> (B, out_dim) FP32."""
        outs = []
        for a in range(0, x.shape[0], self.max_batch):
            xb, B, Bp = self._pad(x[a:a + self.max_batch].float())
            y = torch.empty(Bp, self.out_dim, dtype=torch.float32, device=x.device)
            capi.check(capi.load().sctlgpu_mlp_forward(self._h, Bp, xb.data_ptr(), y.data_ptr(),
                                                       torch.cuda.current_stream().cuda_stream), "mlp_forward")
            outs.append(y[:B])
        return torch.cat(outs)

    def forward_dot(self, x: torch.Tensor, dens: torch.Tensor, index: torch.Tensor, out: torch.Tensor):
        """out[b] += sum_j y[b, j] * dens[index[b], j] (fused into the last GEMM's epilogue)."""
        for a in range(0, x.shape[0], self.max_batch):
            xb, B, Bp = self._pad(x[a:a + self.max_batch].float())
            idx = torch.full((Bp,), -1, dtype=torch.int64, device=x.device)
            idx[:B] = index[a:a + B]
            o = torch.zeros(Bp, dtype=torch.float64, device=x.device)
            capi.check(capi.load().sctlgpu_mlp_forward_dot(self._h, Bp, xb.data_ptr(), dens.data_ptr(), idx.data_ptr(),
                                                           o.data_ptr(), torch.cuda.current_stream().cuda_stream),
                       "mlp_forward_dot")
            out[a:a + B] += o[:B]
        return out

    def train_step(self, x: torch.Tensor, t: torch.Tensor, lr: float, want_loss=False):
        loss = ctypes.c_float(0.0)
        capi.check(capi.load().sctlgpu_mlp_train_step(self._h, x.shape[0], x.data_ptr(), t.data_ptr(), float(lr),
                                                      ctypes.byref(loss) if want_loss else None,
                                                      torch.cuda.current_stream().cuda_stream), "mlp_train_step")
        return loss.value if want_loss else None

    def gradients(self, x: torch.Tensor, t: torch.Tensor):
        g = np.empty(self.n_params, np.float32)
        loss = ctypes.c_float(0.0)
        capi.check(capi.load().sctlgpu_mlp_gradients(self._h, x.shape[0], x.data_ptr(), t.data_ptr(), g.ctypes.data,
                                                     ctypes.byref(loss)), "mlp_gradients")
        return g, loss.value


def panel_weights(kernel, pairs_t, pairs_p, r_trg, X, alpha=1.0, max_depth=22):
    """Accurate weights (n_pairs, 100) of (target, panel) pairs by adaptive quadrature."""
    n = pairs_t.numel()
    w = torch.empty(n, 100, dtype=torch.float64, device=r_trg.device)
    if n:
        capi.check(capi.load().sctlgpu_panel_near_weights(
            kernel, n, pairs_t.data_ptr(), pairs_p.data_ptr(), r_trg.numel() // 3, r_trg.data_ptr(), X.shape[0],
            X.data_ptr(), float(alpha), int(max_depth), w.data_ptr(), torch.cuda.current_stream().cuda_stream),
            "panel_near_weights")
    return w


def smooth_weights(kernel, pairs_t, pairs_p, r_trg, X, N, Q):
    """Smooth-rule weights (n_pairs, 100): scale * K(x_t - X_ab, N_ab) * Q_ab."""
    xt = r_trg.reshape(-1, 3)[pairs_t]                       # (n, 3)
    Xp, Np, Qp = X[pairs_p], N[pairs_p], Q[pairs_p]          # (n, 100, 3), (n, 100)
    r = xt[:, None, :] - Xp
    r2 = (r * r).sum(-1)
    ri = torch.where(r2 > 0, r2.rsqrt(), torch.zeros_like(r2))
    k = ri if kernel == 0 else (r * Np).sum(-1) * ri ** 3
    return k * Qp * capi.load().sctlgpu_scale_factor(kernel)


class Standardizer:
    """Per-column affine map to zero mean and unit deviation (deviations floored at 1e-12)."""

    def __init__(self, x: torch.Tensor):
        self.mu = x.mean(0)
        self.sd = x.std(0).clamp_min(1e-12)

    @classmethod
    def from_arrays(cls, mu: torch.Tensor, sd: torch.Tensor) -> "Standardizer":
        st = cls.__new__(cls)
        st.mu, st.sd = mu, sd
        return st

    def fwd(self, x):
        return ((x - self.mu) / self.sd).float()

    def inv(self, y):
        return y.double() * self.sd + self.mu


class LearnedCorrection:
    """Ensemble of correction networks with range gating, a disagreement check and an error model
    calibrated on held-out labels.

    With `singular` (a surface with `singular_weights(f)` and `singular_dot(f, sig, pp)`, e.g. the
    torus) the networks learn only the weights minus their known near-singular part (the jump and
    the solid angle of the flat panel), a smoother function of the features; predictions add the
    part back."""

    CALIB_BINS = 16  # bins of |signed log distance feature| in [0, 1]
    CALIB_SAFETY = 2.0

    def __init__(self, n_models=2, max_batch=1 << 14, seeds=(1, 2), singular=None, basis_inputs=False):
        self.singular = singular
        # with basis_inputs the networks also see the panel's Lagrange bases at the foot point
        # (from `singular.basis_features`, 2p more inputs)
        self.basis_inputs = bool(basis_inputs) and singular is not None
        in_dim = IN_DIM + (20 if self.basis_inputs else 0)
        self.models = [MLP(in_dim=in_dim, max_batch=max_batch, seed=s) for s in seeds[:n_models]]
        self.fx = self.fy = None
        self.range = None
        self.calib = self.calib_sum = None

    def fit(self, feats: torch.Tensor, w: torch.Tensor, steps=2000, batch=1 << 14, lr=2e-3, seed=0, log=None,
            val_frac=0.1):
        """Train every model on (features, accurate weights), holding out `val_frac` of the pairs to
        calibrate the error model; returns the final losses."""
        g = torch.Generator(device=feats.device).manual_seed(seed)
        perm = torch.randperm(feats.shape[0], device=feats.device, generator=g)
        n_val = int(feats.shape[0] * val_frac)
        val, trn = perm[:n_val], perm[n_val:]
        fv, wv = feats[val], w[val]
        feats, w = feats[trn], w[trn]
        if self.singular is not None:
            w = w - self.singular.singular_weights(feats)
        self.range = (feats.min(0).values, feats.max(0).values)
        inp = self.inputs(feats)
        self.fx, self.fy = Standardizer(inp), Standardizer(w)
        X, Y = self.fx.fwd(inp).contiguous(), self.fy.fwd(w).contiguous()
        del inp
        del w
        n = X.shape[0]
        losses = []
        for mi, m in enumerate(self.models):
            last = None
            for it in range(steps):
                idx = torch.randint(0, n, (batch,), device=X.device, generator=g)
                lr_t = lr * 0.5 * (1 + np.cos(np.pi * it / steps))
                want = it == steps - 1 or (log and it % 500 == 0)
                loss = m.train_step(X[idx].contiguous(), Y[idx].contiguous(), lr_t, want_loss=want)
                if want:
                    last = loss
                    if log:
                        log(f"model {mi} step {it} loss {loss:.4e}")
            losses.append(last)
        self._calibrate(fv, wv)
        return losses

    def _bin(self, feats):
        return (feats[:, 2].abs().clamp(0, 1) * self.CALIB_BINS).long().clamp(max=self.CALIB_BINS - 1)

    def _calibrate(self, fv, wv):
        """Per distance bin, on held-out pairs: the largest weight error of the ensemble mean
        (max over nodes) and the largest error of its weight sum (bins without held-out pairs get
        the overall largest), times the safety factor."""
        pred = self.predict_weights(fv).mean(0)
        e = pred - wv
        b = self._bin(fv)
        out = []
        for err in (e.abs().max(1).values, e.sum(1).abs()):
            top = err.max() if err.numel() else torch.tensor(float("inf"), device=fv.device, dtype=torch.float64)
            c = torch.full((self.CALIB_BINS,), float(top), dtype=torch.float64, device=fv.device)
            for i in range(self.CALIB_BINS):
                m = b == i
                if m.any():
                    c[i] = err[m].max()
            out.append(c * self.CALIB_SAFETY)
        self.calib, self.calib_sum = out

    def error_bound(self, feats, sig):
        """Calibrated bound on |predicted - accurate correction| of pairs with features `feats` and
        panel densities `sig` (n, 100): with e the weight errors and m the panel's mean density,
        |e . sig| <= |sum e| |m| + max|e| sum|sig - m|, each factor from the calibration."""
        b = self._bin(feats)
        m = sig.mean(1)
        return self.calib_sum[b] * m.abs() + self.calib[b] * (sig - m[:, None]).abs().sum(1)

    def inputs(self, feats):
        """Network inputs of pairs with features `feats`."""
        if not self.basis_inputs:
            return feats
        return torch.cat([feats, self.singular.basis_features(feats)], 1)

    def in_range(self, feats):
        lo, hi = self.range
        return ((feats >= lo) & (feats <= hi)).all(1)

    def save(self, path: str):
        """Checkpoint (`sctl_gb300.checkpoint` container): every network's parameters, the feature
        and weight standardizers, the trained feature range and the calibration tables -- all a
        trained correction needs to be used again or trained further (Adam restarts)."""
        from . import checkpoint
        arrays = {f"model{i}": m.get_params() for i, m in enumerate(self.models)}
        for tag, st in (("fx", self.fx), ("fy", self.fy)):
            arrays[f"{tag}_mu"] = st.mu.double().cpu().numpy()
            arrays[f"{tag}_sd"] = st.sd.double().cpu().numpy()
        arrays["range_lo"], arrays["range_hi"] = (r.double().cpu().numpy() for r in self.range)
        arrays["calib"], arrays["calib_sum"] = self.calib.cpu().numpy(), self.calib_sum.cpu().numpy()
        meta = {"n_models": len(self.models), "in_dim": self.models[0].in_dim, "out_dim": self.models[0].out_dim,
                "basis_inputs": self.basis_inputs, "singular": self.singular is not None,
                "calib_bins": self.CALIB_BINS, "calib_safety": self.CALIB_SAFETY}
        checkpoint.save(path, arrays, meta)

    def load(self, path: str, device="cuda"):
        """Restores a checkpoint written by `save` into this object (same network shape, the same
        singular-part and basis-input settings)."""
        from . import checkpoint
        arrays, meta = checkpoint.load(path)
        if (meta.get("n_models") != len(self.models) or meta.get("in_dim") != self.models[0].in_dim or
                meta.get("out_dim") != self.models[0].out_dim or
                bool(meta.get("basis_inputs")) != self.basis_inputs or
                bool(meta.get("singular")) != (self.singular is not None) or
                meta.get("calib_bins") != self.CALIB_BINS):
            raise checkpoint.CheckpointError(f"checkpoint {path!r} was written for another configuration: {meta}")
        for i, m in enumerate(self.models):
            m.set_params(arrays[f"model{i}"])
        t = lambda a: torch.from_numpy(a).to(device)  # noqa: E731
        self.fx = Standardizer.from_arrays(t(arrays["fx_mu"]), t(arrays["fx_sd"]))
        self.fy = Standardizer.from_arrays(t(arrays["fy_mu"]), t(arrays["fy_sd"]))
        self.range = (t(arrays["range_lo"]), t(arrays["range_hi"]))
        self.calib, self.calib_sum = t(arrays["calib"]), t(arrays["calib_sum"])
        return self

    def predict(self, feats: torch.Tensor):
        """Per-model network outputs in weight units, (n_models, n, 100) FP64: the accurate weights,
        or with `singular` the accurate weights minus their singular part."""
        x = self.fx.fwd(self.inputs(feats)).contiguous()
        return torch.stack([self.fy.inv(m.forward(x)) for m in self.models])

    def predict_weights(self, feats: torch.Tensor):
        """Per-model predicted accurate weights, (n_models, n, 100) FP64."""
        p = self.predict(feats)
        if self.singular is not None:
            p = p + self.singular.singular_weights(feats)[None]
        return p


def learned_near_field(S, T, L: LearnedCorrection, r_trg: torch.Tensor, sigma: torch.Tensor, tol: float,
                       kernel=1, mode="mixed", digits=10, near_factor=1.5, alpha=1.0, pairs=None, plan=None,
                       stats=None, h_cut=0.1):
    """Potential with learned near corrections where the pair is near-singular (the target's foot point
    inside the panel and its distance below h_cut panel sizes -- elsewhere the smooth rule is already
    accurate and the network would only add its own error), inside the trained feature range, its
    calibrated error bound is within `tol` and the two networks agree to `tol`; the plain adaptive path
    for every other near pair.  The bound needs only the features and the density, so it is checked
    before the networks run: pairs it rules out cost no inference."""
    from .torus import pair_features_device
    xt = r_trg.reshape(-1).contiguous()
    nt = xt.numel() // 3
    out = S.far_field(xt, sigma, kernel, mode, digits)
    if pairs is None:
        pairs = S.near_pairs(xt, near_factor)
    if plan is None:
        plan = S.smooth_subtraction_plan(nt, pairs, kernel, mode, digits)
    plan.execute(xt, S.X.reshape(-1), S.N.reshape(-1), sigma.reshape(-1).contiguous(), out, w_src=S.negQ,
                 accumulate=True)
    pt, pp = pairs
    f = pair_features_device(T, xt, pt, pp)
    hfeat_cut = (np.log10(h_cut) + 6.0) / 6.0
    in_panel = (f[:, 0] >= 0) & (f[:, 0] <= 1) & (f[:, 1] >= 0) & (f[:, 1] <= 1) & (f[:, 2].abs() < hfeat_cut)
    ok = L.in_range(f) & in_panel
    sig = sigma.reshape(S.np, S.nn)
    dens = (sig * L.fy.sd[None]).contiguous()
    const = (sig * L.fy.mu[None]).sum(1)
    idx = torch.nonzero(ok, as_tuple=True)[0]
    idx = idx[L.error_bound(f[idx], sig[pp[idx]]) <= tol]
    if idx.numel():
        x = L.fx.fwd(L.inputs(f[idx])).contiguous()
        preds = []
        for m in L.models:
            o = torch.zeros(idx.numel(), dtype=torch.float64, device=xt.device)
            m.forward_dot(x, dens, pp[idx].contiguous(), o)
            preds.append(o + const[pp[idx]])
        if L.singular is not None:
            base = L.singular.singular_dot(f[idx], sig, pp[idx])
            preds = [p + base for p in preds]
        agree = (preds[0] - preds[1]).abs() <= tol
        acc_idx = idx[agree]
        out.index_add_(0, pt[acc_idx], 0.5 * (preds[0][agree] + preds[1][agree]))
    else:
        acc_idx = idx
    if acc_idx.numel():
        rej = torch.ones(pt.numel(), dtype=torch.bool, device=xt.device)
        rej[acc_idx] = False
        rt, rp = pt[rej].contiguous(), pp[rej].contiguous()
    else:
        rt, rp = pt, pp
    if rt.numel():
        S.near_correction(xt, sigma, (rt, rp), kernel, alpha, out=out, subtract_smooth=False)
    if stats is not None:
        stats.update(pairs=int(pt.numel()), candidates=int(ok.sum()), inferred=int(idx.numel()),
                     accepted=int(acc_idx.numel()), fallback=int(rt.numel()),
                     accepted_per_target=torch.bincount(pt[acc_idx], minlength=nt))
    return out
