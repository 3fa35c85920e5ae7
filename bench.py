"""Benchmark of the particle-kernel direct sums on GB300.

Workload (one "step"): the mixed-precision (digits = 10) direct sums of
Laplace3D_DxU, Stokes3D_FxU and Stokes3D_DxU over 2^20 sources uniform on the
unit sphere (outward normals) and 2^20 targets uniform in the radius-2 ball,
densities N(0,1) -- 3 * 2^40 interactions.  Inputs are seeded synthetic data
(no dataset exists for this path).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` = whole-job Ginteractions/s with inputs
resident in HBM; `e2e` = the same through the public host-array API with the
host<->device copies inside the timed region; `roofline` = the dominant
kernel's interactions/s against the FP32-issue roofline; `cpu_baseline` = the
reference's own CPU Eval (built from its installed headers) on this host's cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

KERNELS = [1, 2, 3]  # Laplace3D_DxU, Stokes3D_FxU, Stokes3D_DxU
NAMES = {0: "Laplace3D_FxU", 1: "Laplace3D_DxU", 2: "Stokes3D_FxU", 3: "Stokes3D_DxU"}
# Algorithmic FP32-pipe ops + MUFU ops per interaction (formulas of kernel_functions.hpp,
# excluding Newton refinement and masking) and the reference's own FLOPS() counters.
ALG_OPS = {0: (7, 1), 1: (13, 1), 2: (18, 1), 3: (20, 1)}
REF_FLOPS = {0: 6, 1: 14, 2: 23, 3: 26}
N_SRC = N_TRG = 1 << 20
DIGITS = 10
SMS = 152
FP32_LANES = 128
FP64_PER_SM = 2  # FP64 FMA per SM per clock on GB300 (measured 1.9 at the 2070 MHz nominal clock)
MUFU_PER_SM = 16


def peaks():
    p = {}
    try:
        p = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    return p


def roofline_peak_int_s(kernel, sm_mhz, fp64=False):
    """Interactions/s at the issue roofline: the algorithmic ops of one interaction on the FP32
    pipe (128 lanes per SM) or, for the FP64 form, the FP64 pipe (FP64_PER_SM per clock), and one
    reciprocal square root on the MUFU unit (16 per SM per clock)."""
    ops, mufu = ALG_OPS[kernel]
    per_clk = min((FP64_PER_SM if fp64 else FP32_LANES) / ops, MUFU_PER_SM / mufu)
    return SMS * sm_mhz * 1e6 * per_clk


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_baseline(threads=0, n_trg=4096, kernels=KERNELS, digits=DIGITS):
    """The reference's CPU Eval on this host, FP64, all host cores, on a bounded sample (n_trg
    targets x all 2^20 sources per kernel; cost is exactly Ns*Nt, so interactions/s compare).

    kind "reference": the reference's own GenericKernel::Eval<double,true> (its SIMD code, built
    from baseline/_ref by `make -C oracle hot`, OpenMP over all cores), at the same digits as the
    GPU step.  kind "port" (only where the reference is not installed): the plain-C restatement
    (oracle/sctl_oracle.c, exact 1/sqrt), which is slower than the reference's SIMD code."""
    from oracle import oracle as O
    from sctl_gb300 import workloads as W
    use_ref = O.ref_hot_available()
    pairs, secs = 0, 0.0
    for k in kernels:
        d = W.sphere_ball(N_SRC, n_trg, k, seed=100 + k)
        t0 = time.perf_counter()
        if use_ref:
            O.ref_hot_eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"], digits=digits)
        else:
            O.eval(k, d["r_trg"], d["r_src"], d["n_src"], d["v_src"], nthreads=threads)
        secs += time.perf_counter() - t0
        pairs += N_SRC * n_trg
    names = [NAMES[k] for k in kernels]
    if use_ref:
        return {"value": pairs / secs / 1e9, "unit": "Ginteractions/s", "cores": O.ref_hot_threads(),
                "kind": "reference",
                "sample": f"{n_trg} targets x 2^{N_SRC.bit_length() - 1} sources per kernel, kernels {names}, FP64, "
                          f"digits {digits}: the reference's GenericKernel::Eval<double,true> (static digits "
                          f"dispatcher, OpenMP; built from baseline/_ref with -O3 -mcpu/-march=native), "
                          f"{secs:.1f} s"}
    cores = threads if threads > 0 else O.max_threads()
    return {"value": pairs / secs / 1e9, "unit": "Ginteractions/s", "cores": cores, "kind": "port",
            "sample": f"{n_trg} targets x 2^{N_SRC.bit_length() - 1} sources per kernel, kernels {names}, FP64 "
                      f"(fallback: the reference is not installed in baseline/_ref; oracle/sctl_oracle.c restating "
                      f"generic-kernel.txx Eval, exact 1/sqrt), {secs:.1f} s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n_trg = 4096
    samples = []
    for _ in range(args.warmup):
        cpu_baseline(n_trg=n_trg // 8)
    for _ in range(args.steps):
        samples.append(cpu_baseline(n_trg=n_trg))
    val = statistics.median(s["value"] for s in samples)
    cb = dict(samples[-1])
    cb["value"] = val
    line = {"impl": "reference", "metric": "Laplace/Stokes Ginteractions/s mixed vs FP64 @1e-10", "value": val,
            "unit": "Ginteractions/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "sphere_ball 2^20 src x 2^20 trg, Laplace3D_DxU + Stokes3D_FxU + Stokes3D_DxU, "
                                   "digits 10", "sample_per_step": f"{n_trg} targets x 2^20 sources per kernel"},
            "cpu_baseline": cb,
            "e2e": {"value": val, "unit": "Ginteractions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ref_full_section(kernel=1, digits=DIGITS):
    """Confirms that the bounded CPU sample extrapolates: the reference's own Eval<double,true> for
    one kernel over the full 2^20 x 2^20 sphere/ball problem (one call), against the 4096-target
    sample the CPU legs time.  Cost is exactly Ns*Nt, so the two interaction rates should agree."""
    from oracle import oracle as O
    from sctl_gb300 import workloads as W
    if not O.ref_hot_available():
        return {"unavailable": "the reference is not installed in baseline/_ref"}
    d = W.sphere_ball(N_SRC, N_TRG, kernel, seed=100 + kernel)
    res = {"kernel": NAMES[kernel], "digits": digits, "threads": O.ref_hot_threads()}
    sub = {a: (v[:4096] if a == "r_trg" else v) for a, v in d.items()}
    t0 = time.perf_counter()
    O.ref_hot_eval(kernel, sub["r_trg"], sub["r_src"], sub["n_src"], sub["v_src"], digits=digits)
    s = time.perf_counter() - t0
    res["sample_4096_targets"] = {"s": s, "gint_s": 4096 * N_SRC / s / 1e9}
    t0 = time.perf_counter()
    O.ref_hot_eval(kernel, d["r_trg"], d["r_src"], d["n_src"], d["v_src"], digits=digits)
    s = time.perf_counter() - t0
    res["full_2p20_x_2p20"] = {"s": s, "gint_s": N_TRG * N_SRC / s / 1e9}
    res["full_over_sample"] = res["full_2p20_x_2p20"]["gint_s"] / res["sample_4096_targets"]["gint_s"]
    return res


def _ev_ms(torch, fn, reps=3):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e30
    for _ in range(reps):
        torch.cuda.synchronize()
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def near_field_section(torch, stream, panel=False):
    """4096 uneven Laplace3D_DxU near blocks (100..6400 sources, 16..2048 targets), one persistent
    launch per plan execution (CUDA-graph replay), FP64 vs mixed digits 10.  With panel=True the
    sources per block are 10 x 10 panels upsampled k x per side (Ns = 100 k^2, k = 1..8)."""
    from oracle import oracle as O
    from sctl_gb300 import workloads as W
    from sctl_gb300.near import NearPlan
    k = 1
    d = W.near_blocks(4096, k, seed=0, panel=panel)
    blocks = d["blocks"]
    ns, nt = d["r_src"].shape[0], d["r_trg"].shape[0]
    pairs = int((blocks[:, 1] * blocks[:, 3]).sum())
    dd = {a: torch.from_numpy(np.ascontiguousarray(v)).cuda() for a, v in d.items() if a != "blocks"}
    # algorithmic bytes of one execution (FP64 inputs): sources x, n, f; targets x in, potential out
    alg_bytes = ns * (3 + 3 + 1) * 8 + nt * (3 * 8 + 8)
    res = {"workload": "4096 blocks, Ns=" + ("100*k^2, k=1..8" if panel else "round(100*64^u)") +
                       ", Nt=round(16*128^v), Laplace3D_DxU, seed 0",
           "interactions": pairs, "algorithmic_bytes": alg_bytes}
    outs = {}
    for mode, dg in (("mixed", 10), ("f64", -1)):
        plan = NearPlan(k, blocks, ns, nt, mode=mode, digits=dg)
        out = torch.zeros(nt, dtype=torch.float64, device="cuda")
        run = lambda: plan.execute(dd["r_trg"], dd["r_src"], dd["n_src"], dd["v_src"], out)  # noqa: E731
        run()
        ms = _ev_ms(torch, run)
        outs[mode] = out.cpu().numpy()
        res[f"{mode}_d{dg}"] = {"ms": ms, "gint_s": pairs / (ms * 1e-3) / 1e9, "hbm_gb_s": alg_bytes / (ms * 1e-3) / 1e9,
                               **plan.info()}
    res["mixed_vs_f64_speedup"] = res["f64_d-1"]["ms"] / res["mixed_d10"]["ms"]
    sel = blocks[:200]
    ref = np.concatenate([O.eval(k, d["r_trg"][t0:t0 + m], d["r_src"][s0:s0 + n], d["n_src"][s0:s0 + n],
                                 d["v_src"][s0:s0 + n]) for s0, n, t0, m in sel])
    end = int(sel[-1, 2] + sel[-1, 3])
    res["mixed_rel_l2_vs_fp64_oracle_200_blocks"] = O.rel_l2(outs["mixed"][:end], ref)
    res["f64_rel_l2_vs_fp64_oracle_200_blocks"] = O.rel_l2(outs["f64"][:end], ref)
    return res


def cluster_section(torch, stream):
    """64 Gaussian clusters (sigma 1e-3), 2^20 sources, Laplace FxU / Stokes FxU, error vs the FP64
    oracle on 128 targets for digits 6, 8, 10, 12 (mixed) and the FP64 form."""
    import sctl_gb300 as S
    from oracle import oracle as O
    from sctl_gb300 import workloads as W
    res = {}
    for k in (0, 2):
        d = W.clusters(1 << 20, 1 << 10, k, seed=0)
        sub = {a: (v[::8][:128] if a == "r_trg" else v) for a, v in d.items()}
        ref = O.eval(k, sub["r_trg"], sub["r_src"], sub["n_src"], sub["v_src"])
        dd = {a: torch.from_numpy(np.ascontiguousarray(v)).cuda() for a, v in sub.items()}
        kern = [S.Laplace3D_FxU, S.Laplace3D_DxU, S.Stokes3D_FxU, S.Stokes3D_DxU][k]
        row = {}
        for mode, dg in (("mixed", 6), ("mixed", 8), ("mixed", 10), ("mixed", 12), ("f64", -1)):
            out = kern.Eval(None, dd["r_trg"], dd["r_src"], dd["n_src"], dd["v_src"], digits=dg, mode=mode)
            torch.cuda.synchronize()
            row[f"{mode}_d{dg}_rel_l2"] = O.rel_l2(out.cpu().numpy(), ref)
        res[NAMES[k]] = row
    return res


def cube_section(torch, stream):
    """8192 x 8192 unit-cube Laplace FxU, FP64 digits 14: GPU vs the CPU port on all host cores."""
    import sctl_gb300 as S
    from oracle import oracle as O
    from sctl_gb300 import workloads as W
    d = W.cube(8192, 8192, 0, 0)
    dd = {a: torch.from_numpy(np.ascontiguousarray(v)).cuda() for a, v in d.items()}
    out = torch.zeros(8192, dtype=torch.float64, device="cuda")
    run = lambda: S.Laplace3D_FxU.Eval(out, dd["r_trg"], dd["r_src"], dd["n_src"], dd["v_src"], digits=14,  # noqa
                                       mode="f64")
    run()
    out.zero_()
    run()
    torch.cuda.synchronize()
    gpu = out.cpu().numpy()
    ms = _ev_ms(torch, run)
    t0 = time.perf_counter()
    ref = O.eval(0, d["r_trg"], d["r_src"], d["n_src"], d["v_src"])
    cpu_s = time.perf_counter() - t0
    return {"gpu_ms": ms, "gpu_gint_s": 8192 * 8192 / (ms * 1e-3) / 1e9, "cpu_port_s": cpu_s,
            "cpu_port_gint_s": 8192 * 8192 / cpu_s / 1e9, "cpu_cores": O.max_threads(),
            "rel_l2_vs_cpu": O.rel_l2(gpu, ref)}


def kmat_section(torch, stream):
    """KernelMatrix (SetupNear's per-block matrices) for a large near block: 2048 targets x 6400
    sources, Stokes3D_FxU and Laplace3D_DxU, FP64 / mixed (double-float entries) / FP32; written
    bytes per second against the measured HBM bandwidth, and the mixed entries against FP64."""
    import sctl_gb300 as S
    from sctl_gb300 import workloads as W
    hbm = peaks().get("hbm_gbs", 6800.0)
    res = {"workload": "2048 targets x 6400 sources (sphere/ball points), matrices written to HBM"}
    for k, kern in ((2, S.Stokes3D_FxU), (1, S.Laplace3D_DxU)):
        d = W.sphere_ball(6400, 2048, k, seed=11)
        row = {}
        ref = None
        for mode in ("f64", "mixed", "f32"):
            dt = torch.float32 if mode == "f32" else torch.float64
            dd = [torch.from_numpy(np.ascontiguousarray(d[a])).to(dt).cuda() for a in ("r_trg", "r_src", "n_src")]
            run = lambda: kern.KernelMatrix(dd[0], dd[1], dd[2], digits=-1 if mode != "mixed" else 10,  # noqa: E731
                                            mode=mode)
            M = run()
            ms = _ev_ms(torch, run, reps=3)
            nbytes = M.numel() * M.element_size()
            row[mode] = {"ms": ms, "gb_s": nbytes / (ms * 1e-3) / 1e9,
                         "frac_of_measured_hbm": nbytes / (ms * 1e-3) / 1e9 / hbm}
            if mode == "f64":
                ref = M
            elif mode == "mixed":
                row[mode]["max_rel_vs_f64"] = ((M - ref).abs().max() / ref.abs().max()).item()
            del M
        res[NAMES[k]] = row
    return res


def ext_section(torch, stream, nt=1 << 16, ns=1 << 18):
    """The twelve micro-kernels beyond the hot-path four: FP64 and FP32 direct sums of 2^16 targets x
    2^18 sources (uniform in [-1,1]^3, N(0,1) densities, wavenumber 2.5), Ginteractions/s, and the
    FP64 result against the oracle on 64 targets."""
    import sctl_gb300 as S
    from oracle import oracle as O
    from sctl_gb300 import capi
    rng = np.random.default_rng(0)
    res = {"workload": f"{nt} targets x {ns} sources in [-1,1]^3, digits -1"}
    names = {v: k for k, v in capi.KERNEL_IDS.items()}
    for k in range(4, 16):
        nd, sd, td = O.DIMS[k]
        xs, xt = rng.uniform(-1, 1, (ns, 3)), rng.uniform(-1, 1, (nt, 3))
        n = rng.normal(size=(ns, 3)) if nd else np.zeros((0, 3))
        f = rng.normal(size=ns * sd)
        K = S.GenericKernel(names[k], ctx=2.5 if k in capi.HELMHOLTZ_IDS else None)
        row = {}
        for mode, dt in (("f64", torch.float64), ("f32", torch.float32)):
            d = [torch.from_numpy(np.ascontiguousarray(a)).to(dt).cuda() for a in (xt, xs, n, f)]
            out = torch.zeros(nt * td, dtype=dt, device="cuda")
            run = lambda: K.Eval(out, d[0], d[1], d[2], d[3], digits=-1, mode=mode)  # noqa: E731
            run()
            ms = _ev_ms(torch, run, reps=2)
            row[f"{mode}_gint_s"] = nt * ns / (ms * 1e-3) / 1e9
            if mode == "f64":
                out.zero_()
                run()
                ref = O.eval(k, xt[:64], xs, n if nd else None, f, mu=2.5)
                row["f64_rel_l2_vs_oracle_64_targets"] = O.rel_l2(out.cpu().numpy()[:64 * td], ref)
        res[names[k]] = row
    return res


def mlp_section(torch, stream):
    """tcgen05 BF16 tensor-core path: one large GEMM (65536 x 256 x 4096) and the correction network
    (15 -> 256 -> 256 -> 256 -> 100, GELU) forward on 2^17 pairs and training steps on 2^14 pairs,
    against the measured cuBLAS bf16 peak."""
    import math

    from sctl_gb300 import capi
    from sctl_gb300.learned import MLP
    pk = peaks()
    peak_tf = pk.get("bf16_tflops", 1900.0)
    res = {}
    M, N, K = 65536, 256, 4096
    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    Bt = (torch.randn(N, K, device="cuda", generator=g) / math.sqrt(K)).to(torch.bfloat16)
    C = torch.empty(M, N, device="cuda")
    lib = capi.load()
    gemm = lambda: capi.check(lib.sctlgpu_tc_gemm_bf16(M, N, K, A.data_ptr(), Bt.data_ptr(), None, 0,  # noqa: E731
                                                       C.data_ptr(), None, None, 0, stream.cuda_stream), "tc_gemm")
    gemm()
    ms = _ev_ms(torch, gemm, reps=5)
    ref = A[:256].float() @ Bt.float().T
    flops = 2.0 * M * N * K
    res["gemm_65536x256x4096"] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12,
                                  "frac_of_measured_bf16": flops / (ms * 1e-3) / 1e12 / peak_tf,
                                  "rel_err_vs_fp32": ((C[:256] - ref).abs().max() / ref.abs().max()).item()}
    del A, Bt, C
    net = MLP(max_batch=1 << 17, seed=3)
    alg = 2.0 * (15 * 256 + 2 * 256 * 256 + 256 * 100)  # algorithmic flops per pair (unpadded layers)
    padded = 2.0 * (64 * 256 + 2 * 256 * 256 + 256 * 128)
    B = 1 << 17
    x = torch.randn(B, 15, device="cuda", generator=g)
    fwd = lambda: net.forward(x)  # noqa: E731
    fwd()
    ms = _ev_ms(torch, fwd, reps=5)
    res["forward_2p17"] = {"ms": ms, "pairs_per_s": B / (ms * 1e-3), "tflops_alg": alg * B / (ms * 1e-3) / 1e12,
                           "tflops_padded": padded * B / (ms * 1e-3) / 1e12,
                           "frac_of_measured_bf16": padded * B / (ms * 1e-3) / 1e12 / peak_tf}
    Bt_ = 1 << 14
    xt, yt = torch.randn(Bt_, 15, device="cuda", generator=g), torch.randn(Bt_, 100, device="cuda", generator=g)
    train = lambda: net.train_step(xt, yt, 1e-4)  # noqa: E731
    train()
    ms = _ev_ms(torch, train, reps=5)
    res["train_step_2p14"] = {"ms": ms, "tflops_padded": 3 * padded * Bt_ / (ms * 1e-3) / 1e12,
                              "frac_of_measured_bf16": 3 * padded * Bt_ / (ms * 1e-3) / 1e12 / peak_tf}
    net.close()
    res["peak_basis"] = f"bf16_tflops {peak_tf} of MEASURED_PEAKS.json (cuBLAS 8192^3 burst)"
    return res


def torus_section(torch, n_eval=1 << 20, n_train=440000, steps=4000, learned=True):
    """Near-singular Laplace double layer on the 64 x 32-panel torus (204,800 nodes): plain path
    (far field + smooth subtraction + adaptive panel corrections) vs the learned path (two
    tcgen05 networks, gated, plain-path fallback) at n_eval targets; labels from the near pairs
    of n_train other targets (440,000 targets give about 2^22 weight sets)."""
    from sctl_gb300.learned import LearnedCorrection, learned_near_field, panel_weights
    from sctl_gb300.nearquad import PanelSurface
    from sctl_gb300.torus import Torus, pair_features_device
    T = Torus(seed=0)
    S = PanelSurface(T.X, T.N, T.Q, T.size)
    res = {"workload": f"torus R=1 r=0.3, 64x32 panels x 10x10 Chebyshev nodes, {n_eval} targets at h in "
                       f"[1e-4,1] panel sizes (log-uniform), Laplace3D_DxU, far field mixed digits 10"}
    tg = T.targets(n_eval, seed=7)
    xt = torch.from_numpy(tg["r_trg"]).cuda().reshape(-1).contiguous()
    one = torch.ones(T.np * 100, dtype=torch.float64, device="cuda")
    sig = torch.from_numpy(T.sigma.reshape(-1)).cuda()
    pairs = S.near_pairs(xt, 1.5)
    plan = S.smooth_subtraction_plan(n_eval, pairs)
    res["near_pairs"] = int(pairs[0].numel())
    # BuildNearList on the GPU (node radius 1.5 panel sizes), timed as a whole (it synchronises once)
    best = 1e30
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pg = S.near_pairs_grid(xt, 1.5)
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t0)
    res["near_list_gpu"] = {"ms": best * 1e3, "pairs": int(pg[0].numel()), "node_radius_panel_sizes": 1.5,
                            "nodes": T.np * 100}
    del pg
    v1 = S.evaluate(xt, one, pairs=pairs, plan=plan).cpu().numpy()
    exact = np.where(tg["side"] < 0, -1.0, 0.0)
    res["plain_gauss_law_max_abs_err"] = float(np.abs(v1 - exact).max())
    t_plain = _ev_ms(torch, lambda: S.evaluate(xt, sig, pairs=pairs, plan=plan), reps=2)
    plain = S.evaluate(xt, sig, pairs=pairs, plan=plan)
    res["plain_ms"] = t_plain
    res["plain_far_field_ms"] = _ev_ms(torch, lambda: S.far_field(xt, sig), reps=2)
    # the same evaluation with the far field by the treecode (trees built once per target set)
    t0 = time.perf_counter()
    S.treecode(xt)
    res["treecode_setup_s"] = time.perf_counter() - t0
    vt = S.evaluate(xt, one, pairs=pairs, plan=plan, far="treecode").cpu().numpy()
    res["plain_treecode_gauss_law_max_abs_err"] = float(np.abs(vt - exact).max())
    res["plain_treecode_ms"] = _ev_ms(torch, lambda: S.evaluate(xt, sig, pairs=pairs, plan=plan, far="treecode"),
                                      reps=2)
    res["plain_treecode_max_rel_diff_vs_direct"] = (
        (S.evaluate(xt, sig, pairs=pairs, plan=plan, far="treecode") - S.evaluate(xt, sig, pairs=pairs, plan=plan))
        .abs().max() / S.evaluate(xt, sig, pairs=pairs, plan=plan).abs().max()).item()
    # SetupNear once, ComputeNearInterac per application: stored accurate weights
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    M = S.near_matrix(xt, pairs)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    acc = torch.zeros(n_eval, dtype=torch.float64, device="cuda")
    apply_ms = _ev_ms(torch, lambda: M.apply(sig, acc), reps=5)
    apply_unresolved_ms = _ev_ms(torch, lambda: M.apply_unresolved(sig, acc), reps=5)
    hbm = peaks().get("hbm_gbs", 6800.0)
    # bytes per application: the stored blocks, plus per pair its resolved entry (K offset, F offset
    # and length), plus per target its offsets and the read-modify-write of the potential (densities
    # stay in L2)
    alg = M.nbytes + M.n_pairs * 16 + n_eval * (8 + 16)
    with_m = S.evaluate(xt, sig, pairs=pairs, plan=plan, matrix=M)
    res["near_matrix"] = {"setup_s": setup_s, "matrix_bytes": M.nbytes, "apply_ms": apply_ms,
                          "apply_through_index_chain_ms": apply_unresolved_ms,
                          "apply_gb_s": alg / (apply_ms * 1e-3) / 1e9,
                          "apply_frac_of_measured_hbm": alg / (apply_ms * 1e-3) / 1e9 / hbm,
                          "evaluate_ms": _ev_ms(torch, lambda: S.evaluate(xt, sig, pairs=pairs, plan=plan, matrix=M),
                                                reps=2),
                          "evaluate_treecode_far_ms": _ev_ms(
                              torch, lambda: S.evaluate(xt, sig, pairs=pairs, plan=plan, matrix=M, far="treecode"),
                              reps=2),
                          "max_rel_diff_vs_adaptive": ((with_m - plain).abs().max() / plain.abs().max()).item()}
    del M
    if not learned:
        return res
    # learned path
    tt = T.targets(n_train, seed=100)
    xtr = torch.from_numpy(tt["r_trg"]).cuda().reshape(-1).contiguous()
    pt, pp = S.near_pairs(xtr, 1.5)
    t0 = time.perf_counter()
    W = panel_weights(1, pt, pp, xtr, S.X)
    torch.cuda.synchronize()
    res["labels"] = int(pt.numel())
    res["label_s"] = time.perf_counter() - t0
    f = pair_features_device(T, xtr, pt, pp)
    L = LearnedCorrection(max_batch=1 << 14, singular=T, basis_inputs=True)
    t0 = time.perf_counter()
    res["train_losses"] = L.fit(f, W, steps=steps, batch=1 << 14, lr=3e-3)
    torch.cuda.synchronize()
    res["train_s"] = time.perf_counter() - t0
    del f, W
    # held-out calibration (ensemble mean, max over nodes and pairs, x2) per |log distance| bin;
    # bins are 1/16 of [1e-6, 1] panel sizes in log10, the labels cover bins 5-15
    res["held_out_max_weight_err_by_bin"] = [float(f"{x:.3g}") for x in L.calib.tolist()]
    res["held_out_max_weight_sum_err_by_bin"] = [float(f"{x:.3g}") for x in L.calib_sum.tolist()]
    for tol in (1e-8, 1e-3, 1e-1):
        st = {}
        out = learned_near_field(S, T, L, xt, sig, tol, pairs=pairs, plan=plan, stats=st)
        ms = _ev_ms(torch, lambda: learned_near_field(S, T, L, xt, sig, tol, pairs=pairs, plan=plan), reps=2)
        err = (out - plain).abs().max().item() / plain.abs().max().item()
        st.pop("accepted_per_target", None)
        res[f"learned_tol{tol:g}"] = {"ms": ms, "speedup_vs_plain": t_plain / ms, "max_rel_err_vs_plain": err,
                                      **st}
    return res


def treecode_section(torch, n=1 << 20):
    """ParticleFMM::Eval's fast path (the treecode, sctlgpu_treecode_*) against the direct sum:
    the sphere/ball workload at n x n (Laplace DxU, Stokes DxU) and the torus far field (204,800
    panel nodes, densities sigma * Q, n near-surface targets), mixed arithmetic at digits 6 and
    10.  Accuracy: relative l2 on a 512-target sample against the FP64 oracle."""
    import sctl_gb300 as S
    from oracle import oracle as O
    from sctl_gb300 import capi
    from sctl_gb300 import treecode as TC
    from sctl_gb300 import workloads as W
    from sctl_gb300.torus import Torus
    cases = []
    for k in (1, 3):
        d = W.sphere_ball(n, n, k, seed=500 + k)
        cases.append((f"sphere_ball_{NAMES[k]}", k, d["r_src"], d["n_src"], d["r_trg"], d["v_src"]))
    T = Torus(seed=0)
    X, N, Q, sig = T.nodes()
    cases.append(("torus_far_field_Laplace3D_DxU", 1, X, N, T.targets(n, seed=7)["r_trg"], sig * Q))
    res = {"workload": f"n = {n} targets; sphere/ball sources n on the unit sphere; torus 204,800 nodes"}
    stream = torch.cuda.current_stream().cuda_stream
    for name, k, xs, xn, xt, f in cases:
        td = 3 if k >= 2 else 1
        nt, ns = xt.shape[0], xs.shape[0]
        dv = {a: torch.from_numpy(np.ascontiguousarray(v, np.float64).reshape(-1)).cuda()
              for a, v in (("xs", xs), ("xn", xn), ("xt", xt), ("f", f))}
        out = torch.empty(nt * td, dtype=torch.float64, device="cuda")
        sub = np.arange(0, nt, max(1, nt // 512))
        ref = O.eval(k, xt[sub], xs, xn, f)
        r = {"n_src": ns, "n_trg": nt}
        for digits in (6, 10):
            direct = lambda: S.eval_device(k, capi.MIXED, digits, nt, dv["xt"].data_ptr(), ns, dv["xs"].data_ptr(),  # noqa: E731
                                           dv["xn"].data_ptr(), dv["f"].data_ptr(), out.data_ptr(), False, stream)
            t_direct = _ev_ms(torch, direct, reps=1)
            err_direct = O.rel_l2(out.cpu().numpy().reshape(nt, td)[sub].reshape(-1), ref)
            t0 = time.perf_counter()
            tc = TC.Treecode(k, xs, xt, n_src=xn, digits=digits)
            setup_s = time.perf_counter() - t0
            t_tc = _ev_ms(torch, lambda: tc.eval(dv["f"], out=out), reps=2)
            err = O.rel_l2(out.cpu().numpy().reshape(nt, td)[sub].reshape(-1), ref)
            # end to end from host arrays (densities in, potentials out, synchronous)
            fh, uh = np.ascontiguousarray(f, np.float64).reshape(-1), np.zeros(nt * td)
            t_host = 1e30
            for _ in range(2):
                t0 = time.perf_counter()
                tc.eval_host(fh, out=uh)
                t_host = min(t_host, (time.perf_counter() - t0) * 1e3)
            info = tc.info()
            tc.close()
            r[f"digits{digits}"] = {
                "direct_ms": t_direct, "direct_rel_l2": err_direct, "treecode_ms": t_tc, "treecode_rel_l2": err,
                "treecode_host_arrays_ms": t_host,
                "speedup": t_direct / t_tc, "setup_s": setup_s, "order": info["order"], "theta": info["theta"],
                "interactions_vs_direct": (info["direct_interactions"] + info["proxy_interactions"])
                / info["direct_sum_interactions"], "clusters": info["clusters"], "blocks": info["blocks"]}
        res[name] = r
    return res


def learning_curve_section(torch, n_train=220000, steps_list=(2000, 8000, 32000, 96000), batch=1 << 14):
    """Held-out accuracy of the correction network against training length: one network (the
    15 -> 256 -> 256 -> 256 -> 100 GELU MLP on the tcgen05 kernels, singular part subtracted, basis
    inputs) trained for each step count on the same labels (adaptive-quadrature weights of the near
    pairs of n_train torus targets), with the cosine learning-rate schedule stretched to the run.
    Reports the final training loss, the held-out max weight error per distance bin (the quantity
    the acceptance gate is calibrated on) and its worst bin."""
    from sctl_gb300.learned import LearnedCorrection, panel_weights
    from sctl_gb300.nearquad import PanelSurface
    from sctl_gb300.torus import Torus, pair_features_device
    T = Torus(seed=0)
    S = PanelSurface(T.X, T.N, T.Q, T.size)
    tt = T.targets(n_train, seed=100)
    xtr = torch.from_numpy(tt["r_trg"]).cuda().reshape(-1).contiguous()
    pt, pp = S.near_pairs(xtr, 1.5)
    W = panel_weights(1, pt, pp, xtr, S.X)
    f = pair_features_device(T, xtr, pt, pp)
    res = {"labels": int(pt.numel()), "batch": batch, "runs": []}
    for steps in steps_list:
        L = LearnedCorrection(n_models=1, max_batch=batch, singular=T, basis_inputs=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss = L.fit(f, W, steps=steps, batch=batch, lr=3e-3)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        per_bin = (L.calib / L.CALIB_SAFETY).tolist()  # measured held-out maxima (without the safety factor)
        res["runs"].append({"steps": steps, "train_s": secs, "final_loss": loss[0],
                            "epochs": steps * batch / (0.9 * pt.numel()),
                            "held_out_max_weight_err_by_bin": [float(f"{x:.3g}") for x in per_bin],
                            "held_out_max_weight_err_worst": float(max(per_bin))})
        for m in L.models:
            m.close()
    return res


def main():
    global KERNELS, N_SRC
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n", type=int, default=N_TRG, help="targets per rank")
    ap.add_argument("--ns", type=int, default=N_SRC, help="sources")
    ap.add_argument("--kernels", default="1,2,3", help="kernel ids of the step (default: the three sphere/ball kernels)")
    ap.add_argument("--quick", action="store_true", help="timed region only (for profiler runs)")
    ap.add_argument("--skip-torus", action="store_true", help="omit the near-singular torus section")
    ap.add_argument("--section", choices=["near", "near_panel", "clusters", "cube", "torus", "torus_plain", "mlp",
                                          "ext", "kmat", "ref_full", "learning_curve", "treecode"],
                    help="run only this secondary workload and print its JSON (profiling of one kernel family)")
    ap.add_argument("--torus-n", type=int, default=1 << 20, help="targets of the torus section")
    ap.add_argument("--tc-n", type=int, default=1 << 20, help="targets (and sphere sources) of the treecode section")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.section == "ref_full":
        print(json.dumps({"section": args.section, **ref_full_section()}), flush=True)
        return
    if args.section:
        import torch
        from sctl_gb300 import capi
        capi.load()
        stream = torch.cuda.current_stream()
        fn = {"near": lambda: near_field_section(torch, stream),
              "near_panel": lambda: near_field_section(torch, stream, panel=True),
              "clusters": lambda: cluster_section(torch, stream),
              "cube": lambda: cube_section(torch, stream), "mlp": lambda: mlp_section(torch, stream),
              "ext": lambda: ext_section(torch, stream), "kmat": lambda: kmat_section(torch, stream),
              "torus": lambda: torus_section(torch, n_eval=args.torus_n),
              "torus_plain": lambda: torus_section(torch, n_eval=args.torus_n, learned=False),
              "learning_curve": lambda: learning_curve_section(torch),
              "treecode": lambda: treecode_section(torch, n=args.tc_n)}[args.section]
        print(json.dumps({"section": args.section, **fn()}), flush=True)
        return

    import torch
    import torch.distributed as dist

    import sctl_gb300 as S
    from sctl_gb300 import capi
    from sctl_gb300 import workloads as W
    from sctl_gb300.parallel import max_over_ranks

    KERNELS = [int(x) for x in args.kernels.split(",")]
    N_SRC = args.ns
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    capi.load()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)

    # Resident inputs (each rank: its own 2^20 targets against the 2^20 sources).
    data = {}
    for k in KERNELS:
        d = W.sphere_ball(N_SRC, args.n, k, seed=rank * 16 + k)
        data[k] = {a: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for a, v in d.items()}
        data[k]["out"] = torch.empty(args.n * (3 if k >= 2 else 1), dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step(mode="mixed", digits=DIGITS, timing=None):
        for k in KERNELS:
            d = data[k]
            S.eval_device(k, capi.MODE_IDS[mode], digits, args.n, d["r_trg"].data_ptr(), N_SRC,
                          d["r_src"].data_ptr(), d["n_src"].data_ptr() if d["n_src"].numel() else 0,
                          d["v_src"].data_ptr(), d["out"].data_ptr(), False, stream.cuda_stream)
            if timing is not None:
                timing.setdefault(k, []).append(capi.last_kernel_ms())

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    capi.set_timing(True)
    kern_ms = {}
    n0 = capi.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            step(timing=kern_ms)
            ev[i][1].record(stream)
        barrier()
    launches = capi.launch_count() - n0
    capi.set_timing(False)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = sum(step_ms) / len(step_ms)
    ms = max_over_ranks(ms)
    pairs_step = len(KERNELS) * N_SRC * args.n
    value = pairs_step * world / (ms * 1e-3) / 1e9
    clocks = clk.summary()
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": "Laplace/Stokes Ginteractions/s mixed vs FP64 @1e-10", "value": value,
                              "unit": "Ginteractions/s", "ms_per_step": ms, "quick": True,
                              "gpu_launches": launches, "kernels": KERNELS, "n_trg": args.n, "n_src": N_SRC}),
                  flush=True)
        return

    # --- everything below is outside the timed region ---
    # The precision x digits grid on target slices against all 2^20 sources: FP64 and FP32 at digits
    # 6 / 10 / 14 (the reference's two real types) and the mixed form at the same digits; throughput,
    # roofline fraction (FP32 issue for FP32 and mixed, FP64 pipe for FP64) and rel-l2 against the
    # FP64 oracle on the slice's first 256 targets.
    from oracle import oracle as O
    detail = {}
    sm_mhz = peaks().get("sm_max_mhz", 2070.0)
    for k in KERNELS:
        d = data[k]
        row = {"mixed_ms_per_launch": statistics.median(kern_ms[k]),
               "mixed_gint_s": N_SRC * args.n / (statistics.median(kern_ms[k]) * 1e-3) / 1e9}
        host = {a: d[a].cpu().numpy() for a in ("r_trg", "r_src", "n_src", "v_src")}
        ref = O.eval(k, host["r_trg"].reshape(-1, 3)[:256], host["r_src"], host["n_src"], host["v_src"])
        for mode in ("f64", "f32", "mixed"):
            for dg in (6, 10, 14):
                sub = min(args.n, (1 << 13) if mode == "f64" else (1 << 16))
                r_trg = d["r_trg"][:sub * 3] if mode != "f32" else d["r_trg"][:sub * 3].float()
                args_ = [d[a] if mode != "f32" else d[a].float() for a in ("r_src", "n_src", "v_src")]
                out = torch.empty(sub * (3 if k >= 2 else 1), dtype=torch.float32 if mode == "f32" else torch.float64,
                                  device=dev)
                capi.set_timing(True)
                t = []
                for _ in range(2):
                    S.eval_device(k, capi.MODE_IDS[mode], dg, sub, r_trg.data_ptr(), N_SRC, args_[0].data_ptr(),
                                  args_[1].data_ptr() if args_[1].numel() else 0, args_[2].data_ptr(), out.data_ptr(),
                                  False, stream.cuda_stream)
                    t.append(capi.last_kernel_ms())
                capi.set_timing(False)
                gint = N_SRC * sub / (min(t) * 1e-3) / 1e9
                if mode == "f64":
                    frac = gint * 1e9 / roofline_peak_int_s(k, sm_mhz, fp64=True)
                else:
                    frac = gint * 1e9 / roofline_peak_int_s(k, sm_mhz)
                got = out.cpu().numpy().astype(np.float64).reshape(sub, -1)[:256].reshape(-1)
                row[f"{mode}_d{dg}"] = {"gint_s": gint, "targets": sub, "roofline_frac": frac,
                                        "roofline": "fp64_pipe" if mode == "f64" else "fp32_issue",
                                        "rel_l2_vs_fp64_oracle": O.rel_l2(got, ref)}
        row["mixed_d10_vs_f64_d10"] = row["mixed_d10"]["gint_s"] / row["f64_d10"]["gint_s"]
        row["roofline_frac_fp32_issue"] = row["mixed_gint_s"] * 1e9 / roofline_peak_int_s(k, sm_mhz)
        detail[NAMES[k]] = row

    # Accuracy vs the FP64 oracle on 256 targets per kernel.
    from oracle import oracle as O
    for k in KERNELS:
        d = data[k]
        idx = slice(0, 256)
        host = {a: d[a].cpu().numpy() for a in ("r_trg", "r_src", "n_src", "v_src")}
        ref = O.eval(k, host["r_trg"].reshape(-1, 3)[idx], host["r_src"], host["n_src"], host["v_src"])
        got = d["out"].cpu().numpy().reshape(args.n, -1)[idx].reshape(-1)
        detail[NAMES[k]]["rel_l2_vs_fp64_oracle"] = O.rel_l2(got, ref)
        detail[NAMES[k]]["max_rel_vs_fp64_oracle"] = O.max_rel(got, ref)

    # End to end through the public host-array API (pinned host buffers, copies inside the timed region).
    host_in = {}
    h2d = d2h = 0
    for k in KERNELS:
        hk = {}
        for a in ("r_trg", "r_src", "n_src", "v_src"):
            t = torch.empty(data[k][a].shape, dtype=torch.float64, pin_memory=True)
            t.copy_(data[k][a].cpu())
            hk[a] = t.numpy()
            h2d += t.numel() * 8
        hk["out"] = torch.empty(data[k]["out"].shape, dtype=torch.float64, pin_memory=True).numpy()
        d2h += hk["out"].size * 8
        host_in[k] = hk
    kern_objs = {1: S.Laplace3D_DxU, 2: S.Stokes3D_FxU, 3: S.Stokes3D_DxU}
    e2e_steps = max(1, args.steps)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for k in KERNELS:
            h = host_in[k]
            h["out"][:] = 0
            kern_objs[k].Eval(h["out"], h["r_trg"], h["r_src"], h["n_src"], h["v_src"], digits=DIGITS, mode="mixed")
    barrier()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s = max_over_ranks(e2e_s)
    e2e = {"value": pairs_step * world / e2e_s / 1e9, "unit": "Ginteractions/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}

    dom = max(KERNELS, key=lambda k: statistics.median(kern_ms[k]))
    dom_ms = statistics.median(kern_ms[dom])
    pk = peaks()
    sm_max = pk.get("sm_max_mhz", 2070.0)
    peak_int = roofline_peak_int_s(dom, sm_max)
    achieved = N_SRC * args.n / (dom_ms * 1e-3)
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get(NAMES[dom])
        except Exception:
            traffic = None
    roofline = {"bound": "fp32_issue", "kernel": f"direct_sum_pk_kernel<{NAMES[dom]}> (mixed, double-float on packed FP32)",
                "achieved": achieved / 1e9, "peak": peak_int / 1e9, "unit": "Ginteractions/s",
                "frac": achieved / peak_int, "traffic": traffic,
                "peak_basis": f"{SMS} SMs x {sm_max:.0f} MHz (sm_max_mhz of MEASURED_PEAKS.json) x "
                              f"min({FP32_LANES} FP32 lanes / {ALG_OPS[dom][0]} ops, {MUFU_PER_SM} MUFU / "
                              f"{ALG_OPS[dom][1]}) per interaction (of measured clock; lanes and MUFU rate nominal)",
                "achieved_fp32_tflops_equiv": achieved * (ALG_OPS[dom][0]) / 1e12,
                "launch_ms": dom_ms}

    extras = {}
    if rank == 0:
        # secondary workloads: a failure is recorded in its entry and does not cost the headline line
        sections = [("near_field_blocks", lambda: near_field_section(torch, stream)),
                    ("near_field_blocks_panel_variant", lambda: near_field_section(torch, stream, panel=True)),
                    ("precision_stress_clusters", lambda: cluster_section(torch, stream)),
                    ("cube8192_fp64_d14", lambda: cube_section(torch, stream)),
                    ("tensor_core_mlp", lambda: mlp_section(torch, stream)),
                    ("other_micro_kernels", lambda: ext_section(torch, stream)),
                    ("kernel_matrix", lambda: kmat_section(torch, stream)),
                    ("far_field_treecode", lambda: treecode_section(torch))]
        if not args.skip_torus:
            sections.append(("torus_near_singular", lambda: torus_section(torch)))
        for name, fn in sections:
            try:
                extras[name] = fn()
            except Exception as exc:  # noqa: BLE001
                extras[name] = {"error": f"{type(exc).__name__}: {exc}"}
                print(f"section {name} failed: {exc}", file=sys.stderr, flush=True)

    line = {"metric": "Laplace/Stokes Ginteractions/s mixed vs FP64 @1e-10", "value": value,
            "unit": "Ginteractions/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+df (double-float) from f64 inputs", "data": "synthetic (seeded PCG64)",
            "config": {"workload": f"sphere_ball: 2^20 sources on the unit sphere x {args.n} targets in the "
                                   f"radius-2 ball per GPU; Laplace3D_DxU + Stokes3D_FxU + Stokes3D_DxU; mixed "
                                   f"precision, digits {DIGITS}",
                       "interactions_per_step_per_gpu": pairs_step, "parallelism": f"replicas x{world}",
                       "l2": "256 MB buffer written between timed steps; per-step inputs 0.4 GB > 129 MB L2"},
            "gpu_launches": launches, "clocks": clocks, "e2e": e2e, "roofline": roofline,
            "per_kernel": detail, **extras}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
