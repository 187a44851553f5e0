#!/usr/bin/env python
"""Benchmark of the fused flowMC sampling path on one GB300 (per rank).

Workload (default ``rosenbrock128``): the RQSpline bundle with an HMC local
kernel on the 128-D Rosenbrock chain log p = -sum_i [(1-x_i)^2/20 +
5 (x_{i+1}-x_i^2)^2], 16384 chains, HMC n_leapfrog=16 step 0.01 (identity
mass), 40 local + 40 global NFProposal steps per loop, MaskedCouplingRQSpline
12 layers x [512, 512] x 12 bins with BF16 conditioners, AdamW lr 5e-4,
batch 65536, 5 epochs per training loop, n_max_examples 65536, x0 ~ N(0, I)
(seed 4). ``mixture64`` is the 64-D 4-mode mixture bundle with MALA.

A step is one loop of the bundle's schedule (local phase + global phase,
plus flow training in training loops). The schedule has (W+K)//2 training
loops then the rest production loops; the first W training loops are the
untimed warm-up, the K timed loops follow. Defaults W=3, K=37 give the
workload's 20 + 20 loops. value = chain-steps/s = n_chains * (n_local +
n_global) * K / timed seconds (summed over ranks, which run independent
replicas). The working set (chain buffers of several GB, flow weights) is
far larger than L2, so L2 is not flushed between steps.

By default the K timed loops are captured as one CUDA graph before the timed
region (``graph_capture_ms``, the one-time capture, is reported separately)
and the timed region is its replay; ``--eager`` launches them one by one.

``e2e`` repeats the timed region's loop mix through ``Sampler.sample`` (one
call per loop, each a replay of that loop's captured schedule unless
``--eager``) with pinned host buffers: each loop copies its starting
positions host->device and reads the rows it wrote and its final positions
back, all inside the wall-clock timed region (after two untimed production
loops that warm the pinned host buffers). The rows' device->host copy of one
loop overlaps the next loop on a second stream.

``--impl reference`` times the CPU restatement of the same loop (the
reference flowMC itself needs JAX, which this image does not have).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "min-ESS/s & chain-steps/s: fused BF16 vs plain FP32 on 1 GB300 at equal moment error"

WORKLOADS = {
    "rosenbrock128": dict(d=128, n_chains=16384, local="hmc", step=0.01, n_leapfrog=16, n_local=40, n_global=40,
                          n_layers=12, hidden=[512, 512], n_bins=12, lr=5e-4, batch=65536, n_epochs=5,
                          n_max=65536, seed=4),
    "mixture64": dict(d=64, n_chains=4096, local="mala", step=0.05, n_leapfrog=0, n_local=50, n_global=50,
                      n_layers=8, hidden=[256, 256], n_bins=8, lr=1e-3, batch=32768, n_epochs=5, n_max=32768,
                      seed=3),
    "dualmoon5": dict(d=5, n_chains=20, local="mala", step=0.1, n_leapfrog=0, n_local=30, n_global=30,
                      n_layers=4, hidden=[32, 32], n_bins=8, lr=1e-3, batch=10000, n_epochs=5, n_max=10000,
                      seed=0),
}


def mixture_means():
    """The 64-D mixture's four means: +/-4 along the first two columns of a
    Haar-random orthogonal matrix (QR of a Gaussian matrix with the sign fix,
    seed 3)."""
    import numpy as np
    rng = np.random.default_rng(3)
    Q, R = np.linalg.qr(rng.normal(size=(64, 64)))
    Q = Q * np.sign(np.diag(R))
    u1, u2 = Q[:, 0], Q[:, 1]
    return np.stack([4 * u1, -4 * u1, 4 * u2, -4 * u2])


def make_target(name, w, device):
    import numpy as np
    from flowmc_gb300 import targets as TG
    from flowmc_gb300.diagnostics import dual_moon_moments, rosenbrock_chain_moments
    if name == "rosenbrock128":
        t = TG.Rosenbrock(w["d"], device=device)
        mean, var = rosenbrock_chain_moments(w["d"])
        return t, mean, var
    if name == "dualmoon5":
        t = TG.DualMoon(w["d"], device=device)
        mean, var = dual_moon_moments(w["d"], **t.p)
        return t, mean, var
    t = TG.GaussianMixture(mixture_means(), 0.5, device=device)
    mu, cov = t.mean_cov()
    return t, mu, np.diag(cov)


def useful_flow_flops(w):
    """Useful conditioner FLOPs per sample per flow pass: the packed GEMMs
    2(n_c H1 + H1 H2 + H2 n_t P) summed over layers."""
    d, H, P = w["d"], w["hidden"], 3 * w["n_bins"] + 1
    tot = 0
    for l in range(w["n_layers"]):
        nc = (d - (1 - (l & 1)) + 1) // 2
        nt = d - nc
        dims = [nc] + H + [nt * P]
        tot += sum(2 * a * b for a, b in zip(dims[:-1], dims[1:]))
    return tot


def build_sampler(name, w, n_train, n_prod, precision, device):
    import torch
    from flowmc_gb300.random import PRNGKey, split
    from flowmc_gb300.resource.kernel.HMC import HMC
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.resource_strategy_bundle.RQSpline_MALA import RQSpline_MALA_Bundle
    from flowmc_gb300.Sampler import Sampler
    target, mean, var = make_target(name, w, device)
    local = HMC(1, w["step"], w["n_leapfrog"]) if w["local"] == "hmc" else MALA(w["step"])
    key = PRNGKey(w["seed"])
    key, sub = split(key)
    bundle = RQSpline_MALA_Bundle(sub, w["n_chains"], w["d"], target, w["n_local"], w["n_global"], n_train, n_prod,
                                  w["n_epochs"], mala_step_size=w["step"], rq_spline_hidden_units=w["hidden"],
                                  rq_spline_n_bins=w["n_bins"], rq_spline_n_layers=w["n_layers"],
                                  learning_rate=w["lr"], batch_size=w["batch"], n_max_examples=w["n_max"],
                                  local_sampler=local, precision=precision, device=device, autotune=True,
                                  streaming_diagnostics=True)
    sampler = Sampler(w["d"], w["n_chains"], key, resource_strategy_bundles=bundle)
    g = torch.Generator().manual_seed(w["seed"])
    x0 = torch.randn(w["n_chains"], w["d"], generator=g)
    return sampler, bundle, target, mean, var, x0


def loop_segments(order, n_train, n_tr=6, n_pr=4):
    """The bundle's strategy order cut into loops (n_tr / n_pr strategies per
    training / production loop; the phase switch opens the first production loop)."""
    segs = [order[n_tr * i:n_tr * i + n_tr] for i in range(n_train)]
    rest = order[n_tr * n_train:]
    assert rest[:2] == ["reset_steppers", "update_state"]
    prod = rest[2:]
    for i in range(0, len(prod), n_pr):
        segs.append((rest[:2] if i == 0 else []) + prod[i:i + n_pr])
    return segs


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return float("nan")
        sm = sorted(num(r[1]) for r in rows)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": num(rows[0][2]), "samples": len(rows),
                "power_w_max": max(num(r[3]) for r in rows), "reasons": sorted(reasons)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), d.get("bf16_tflops_sustained", 1700.0), "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


# ---------------------------------------------------------------- local-step HBM probe
def local_hbm_probe(dev, chains=65536, steps=50, reps=5, lanes=(0,)):
    """The local-step kernel alone on the cheap 64-D 4-mode mixture
    (MALA and GRW, C chains x S steps, ~0.87 GB of buffer writes per launch):
    algorithmic bytes 4d+8 per chain-step / CUDA-event time, against the HBM
    peak. A derived probe of the mixture workload at a size the roofline can
    resolve."""
    import torch
    from flowmc_gb300.resource.kernel.Gaussian_random_walk import GaussianRandomWalk
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.resource.kernel.base import run_local_steps
    t, _, _ = make_target("mixture64", WORKLOADS["mixture64"], dev)
    d = t.n_dim
    x0 = torch.randn(chains, d, device=dev)
    pos = torch.empty(chains, steps, d, device=dev)
    lp = torch.empty(chains, steps, device=dev)
    acc = torch.empty(chains, steps, device=dev)
    hbm = measured_peaks()[0]
    out = {}
    from flowmc_gb300 import targets as TG
    diag = TG.DiagGaussian(d, device=dev)
    def timed(k, tt):
        for _ in range(2):
            run_local_steps(k, tt, x0, steps, 1, 7, 0, pos, lp, acc, 0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for r in range(reps):
            run_local_steps(k, tt, x0, steps, 1, 7, r + 1, pos, lp, acc, 0)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        gbs = chains * steps * (4 * d + 8) / (ms / 1e3) / 1e9
        return {"lanes_per_chain": k.lanes_per_chain, "ms_per_launch": ms, "achieved_gbs": gbs,
                "frac_hbm": gbs / hbm, "chain_steps_per_s": chains * steps / (ms / 1e3)}

    for name, k, tt in (("mala", MALA(0.05), t), ("grw", GaussianRandomWalk(0.05), t),
                        ("grw_diag_gaussian", GaussianRandomWalk(0.5), diag)):
        best = None
        for g in lanes:
            k.lanes_per_chain = g
            rec = timed(k, tt)
            if best is None or rec["achieved_gbs"] > best["achieved_gbs"]:
                best = rec
        # the same launch with Philox-4x32-7 noise (opt-in generator)
        k.lanes_per_chain = best["lanes_per_chain"]
        k.philox_rounds = 7
        best["philox7"] = timed(k, tt)
        k.philox_rounds = 10
        out[name] = best
    out["config"] = (f"64-D 4-mode mixture (mala, grw) and 64-D diagonal Gaussian (grw_diag_gaussian), "
                     f"{chains} chains x {steps} steps, bytes/chain-step {4 * d + 8}")
    return out


# ---------------------------------------------------------------- batched dense targets
def batched_probe(dev, kind="mala", steps=2000, thin=20, seed=1):
    """48 dense Gaussians sampled in one persistent launch: d_t ~ U{8..256},
    Sigma = Q diag(lambda) Q^T with Q Haar (QR of a Gaussian matrix, signs
    fixed) and lambda ~ logU[1e-2, 10]^d, chains per target round(exp(U[ln 512,
    ln 8192])), x0 ~ N(0, I); MALA step 0.5 sqrt(lambda_min) d^(-1/3), HMC 10
    leapfrog steps with step 0.2 sqrt(lambda_min). `steps` steps, every
    `thin`-th stored. Reports chain-steps/s, the FP32 rate of the target
    evaluations (2d^2 + 4d FLOPs each; MALA 1, HMC n_leapfrog + 1 per step)
    against the nominal FP32 peak (SMs x 128 lanes x 2 FLOPs x max clock), and
    the worst mean / covariance error over the targets (second half of the
    stored rows)."""
    import numpy as np
    import torch
    from flowmc_gb300 import targets as TG
    from flowmc_gb300 import _lib
    from flowmc_gb300.batched import BatchedDenseLocalSteps
    rng = np.random.default_rng(seed)
    dims = rng.integers(8, 257, size=48)
    chains = [int(round(math.exp(rng.uniform(math.log(512), math.log(8192))))) for _ in dims]
    ts, covs, lmins = [], [], []
    for d in dims:
        Q, R = np.linalg.qr(rng.normal(size=(d, d)))
        Q = Q * np.sign(np.diag(R))
        lam = np.exp(rng.uniform(math.log(1e-2), math.log(10.0), size=d))
        cov = Q @ np.diag(lam) @ Q.T
        ts.append(TG.DenseGaussian(Q @ np.diag(1.0 / lam) @ Q.T, device=dev))
        covs.append(cov)
        lmins.append(lam.min())
    nlf = 10
    step = [0.5 * math.sqrt(lm) * d ** (-1 / 3) if kind == "mala" else 0.2 * math.sqrt(lm) for lm, d in zip(lmins, dims)]
    b = BatchedDenseLocalSteps(ts, chains, step, kind=kind, n_leapfrog=nlf)
    g = torch.Generator(device=dev).manual_seed(seed)
    xs = [torch.randn(c, int(d), device=dev, generator=g) for c, d in zip(chains, dims)]
    b.run(xs, 4, seed=seed)   # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    outs, _, _ = b.run(xs, steps, thinning=thin, seed=seed + 1)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    C = sum(chains)
    evals = 1 if kind == "mala" else nlf + 1
    flops = sum(c * steps * evals * (2.0 * d * d + 4.0 * d) for c, d in zip(chains, dims))
    sms = ctypes_sm_count()
    fp32_peak = sms * 128 * 2 * measured_peaks_raw().get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    worst_mean = worst_cov = 0.0
    worst_pred = 0.0
    pred_long = {}
    kept = np.arange(steps // thin)[(steps // thin) // 2:] * thin + 1     # step index of each kept row
    for t, cov in enumerate(covs):
        pos = outs[t][0][:, outs[t][0].shape[1] // 2:].reshape(-1, int(dims[t])).double()
        mu = pos.mean(0).cpu().numpy()
        emp = torch.cov(pos.T).cpu().numpy()
        worst_mean = max(worst_mean, float(np.max(np.abs(mu) / np.sqrt(np.diag(cov)))))
        worst_cov = max(worst_cov, float(np.linalg.norm(emp - cov) / np.linalg.norm(cov)))
        if kind == "mala":
            lam = np.linalg.eigvalsh(cov)
            worst_pred = max(worst_pred, langevin_cov_error(lam, step[t], kept))
            for n in (2000, 20000, 200000):
                kn = np.arange(n // thin)[(n // thin) // 2:] * thin + 1
                pred_long[n] = max(pred_long.get(n, 0.0), langevin_cov_error(lam, step[t], kn))
    out = {"kind": kind, "targets": 48, "chains": C, "dims": [int(dims.min()), int(dims.max())],
           "mean_d": float(dims.mean()), "steps": steps, "thinning": thin, "ms": ms,
           "chain_steps_per_s": C * steps / (ms / 1e3), "fp32_tflops": flops / (ms / 1e3) / 1e12,
           "fp32_peak_nominal_tflops": fp32_peak, "frac_fp32": flops / (ms / 1e3) / 1e12 / fp32_peak,
           "worst_mean_error_sd": worst_mean, "worst_cov_rel_frobenius": worst_cov}
    if kind == "mala":
        out["predicted_worst_cov_rel_frobenius"] = worst_pred
        out["predicted_worst_cov_rel_frobenius_vs_steps"] = {str(k): v for k, v in sorted(pred_long.items())}
    return out


def langevin_cov_error(lam, h, kept_steps):
    """Covariance error that slow mixing alone explains for MALA on N(0, Sigma)
    from x0 ~ N(0, I): with every proposal accepted the chain is the
    unadjusted Langevin recursion x' = x - (h^2 / 2) Sigma^-1 x + h xi, so
    along an eigenvector (eigenvalue lam) the variance after n steps is
    v* + a^(2n) (1 - v*), a = 1 - h^2 / (2 lam), v* = h^2 / (1 - a^2). The
    sample covariance over the kept steps then has eigenvalues mean_n v_n;
    returns its relative Frobenius distance to Sigma (sampling noise not
    included)."""
    import numpy as np
    a = 1.0 - h * h / (2.0 * lam)
    vstar = h * h / (1.0 - a * a)
    vbar = np.array([np.mean(vs + a2 ** kept_steps * (1.0 - vs)) for vs, a2 in zip(vstar, a * a)])
    return float(np.linalg.norm(vbar - lam) / np.linalg.norm(lam))


def ctypes_sm_count():
    import ctypes
    from flowmc_gb300 import _lib
    n = ctypes.c_int32()
    _lib.check(_lib.lib().fmc_device_sm_count(ctypes.byref(n)))
    return n.value


def measured_peaks_raw():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def train_probe(dev, precision="bf16", seed=2):
    """Flow maximum-likelihood training on an 8-mode 32-D mixture: 262144
    samples, MaskedCouplingRQSpline 8 x [128, 128] x 10 bins, AdamW lr 1e-3,
    batch 16384, 20 epochs. Reports samples/s, useful TFLOP/s (3 x the
    forward's 2(n_c H1 + H1 H2 + H2 n_t P) per sample and layer) and the
    final loss."""
    import numpy as np
    import torch
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    from flowmc_gb300.resource.optimizer import Optimizer
    rng = np.random.default_rng(seed)
    d, N = 32, 262144
    means = rng.uniform(-5, 5, size=(8, d))
    scales = rng.uniform(0.3, 1.0, size=(8, d))
    lab = rng.integers(0, 8, size=N)
    data = torch.tensor(means[lab] + scales[lab] * rng.normal(size=(N, d)), dtype=torch.float32, device=dev)
    prec = "bf16" if precision == "bf16" else "float32"
    m = MaskedCouplingRQSpline(d, 8, [128, 128], 10, PRNGKey(seed), precision=prec, device=dev)
    opt = Optimizer(m, learning_rate=1e-3)
    m.train(PRNGKey(1), data, opt, opt.optim_state, 1, 16384, verbose=False)   # warm-up epoch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    _, m, st, losses = m.train(PRNGKey(2), data, opt, opt.optim_state, 20, 16384, verbose=False)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    H, P = 128, 31
    nc, nt = d // 2, d // 2
    per_layer = 2 * (nc * H + H * H + H * nt * P)
    flops = 3.0 * per_layer * 8 * N * 20
    bf16 = measured_peaks()[1]
    return {"precision": precision, "samples": N, "epochs": 20, "batch": 16384, "ms": ms,
            "samples_per_s": N * 20 / (ms / 1e3), "useful_tflops": flops / (ms / 1e3) / 1e12,
            "frac_bf16": flops / (ms / 1e3) / 1e12 / bf16, "final_loss": float(losses[-1])}


# ---------------------------------------------------------------- plain FP32 form
def _time(fn, reps=5):
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def pt_probe(dev, chains=16384, temps=8, steps=50):
    """Parallel tempering on the 64-D 4-mode mixture: one ParallelTempering
    call = tempered MALA (step 0.05) over chains x temps rows for `steps`
    steps, the exchange sweep and the adaptation. Reports (chain,
    temperature)-steps/s of the tempered local kernel and the exchange's
    achieved HBM bandwidth (reads T x 4d B per chain twice, the second from
    L2, writes T x 4d B)."""
    import torch
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.buffers import Buffer
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.resource.logPDF import TemperedPDF
    from flowmc_gb300.resource.states import State
    from flowmc_gb300.strategy.parallel_tempering import ParallelTempering, pt_exchange, pt_local_steps
    w = WORKLOADS["mixture64"]
    tgt, _, _ = make_target("mixture64", w, dev)
    d = w["d"]
    tlp = TemperedPDF(tgt, None, n_dims=d)
    temps_t = torch.linspace(1.0, 10.0, temps, device=dev)
    x = torch.randn(chains, temps, d, device=dev)
    kern = MALA(0.05)
    ms_local = _time(lambda: pt_local_steps(kern, tlp, x, temps_t, steps, 7))
    xl, _, _ = pt_local_steps(kern, tlp, x, temps_t, steps, 7)
    first = torch.empty(chains, d, device=dev)
    rest = torch.empty(chains, temps - 1, d, device=dev)
    ms_ex = _time(lambda: pt_exchange(tgt, xl, temps_t, 9, out_first=first, out_rest=rest))
    tp = Buffer("tempered_positions", (chains, temps - 1, d), 2, device=dev)
    tp.data.normal_()
    tb = Buffer("temperature", (temps,), 0, device=dev)
    tb.update_buffer(temps_t)
    res = {"tempered_logpdf": tlp, "local_sampler": kern, "tempered_positions": tp, "temperatures": tb,
           "sampler_state": State({"training": True})}
    strat = ParallelTempering(steps, "tempered_logpdf", "local_sampler", ["tempered_positions", "temperatures"],
                              "sampler_state")
    x0 = torch.randn(chains, d, device=dev)
    ms_call = _time(lambda: strat(PRNGKey(3), res, x0, {}))
    ex_bytes = chains * temps * d * 4 * 3
    hbm = measured_peaks()[0]
    return {"target": "64-D 4-mode mixture", "chains": chains, "temperatures": temps, "steps": steps,
            "local_ms": ms_local, "row_steps_per_s": chains * temps * steps / (ms_local / 1e3),
            "exchange_ms": ms_ex, "exchange_gbs": ex_bytes / (ms_ex / 1e3) / 1e9,
            "exchange_frac_hbm": ex_bytes / (ms_ex / 1e3) / 1e9 / hbm, "strategy_call_ms": ms_call}


def realnvp_probe(dev, d=32, layers=8, hidden=256, n=262144, batch=16384):
    """RealNVP(d, layers, hidden): log_prob over n rows and one loss+gradient
    on a batch. FP32 FLOPs per row and layer: 2 x (2 H d + 2 d H) forward;
    the gradient recomputes the forward and runs about twice its FLOPs."""
    import torch
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.model.nf_model.realNVP import RealNVP
    m = RealNVP(d, layers, hidden, PRNGKey(0), device=dev)
    x = torch.randn(n, d, device=dev)
    xb = x[:batch].contiguous()
    ms_lp = _time(lambda: m.log_prob(x))
    ms_g = _time(lambda: m.loss_and_grad(xb))
    fl = 2.0 * 4 * hidden * d * layers
    return {"n_dim": d, "layers": layers, "hidden": hidden, "log_prob_rows": n, "log_prob_ms": ms_lp,
            "log_prob_rows_per_s": n / (ms_lp / 1e3), "log_prob_fp32_tflops": fl * n / (ms_lp / 1e3) / 1e12,
            "grad_batch": batch, "grad_ms": ms_g, "grad_rows_per_s": batch / (ms_g / 1e3),
            "grad_fp32_tflops": 4 * fl * batch / (ms_g / 1e3) / 1e12}


def adam_probe(dev, chains=65536, steps=200):
    """AdamOptimization on the 64-D 4-mode mixture: chains x steps of Adam
    with gradient noise in one launch."""
    import torch
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.strategy.optimization import AdamOptimization
    w = WORKLOADS["mixture64"]
    tgt, _, _ = make_target("mixture64", w, dev)
    opt = AdamOptimization(tgt, n_steps=steps, learning_rate=1e-2, noise_level=1.0)
    x0 = torch.randn(chains, w["d"], device=dev)
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        ms = _time(lambda: opt.optimize(PRNGKey(0), None, x0, {}), reps=3)
    return {"target": "64-D 4-mode mixture", "chains": chains, "steps": steps, "ms": ms,
            "chain_steps_per_s": chains * steps / (ms / 1e3)}


def plain_arm(name, w, dev, n_train, n_prod, timed_from, mean_ref, var_ref, ess=True):
    """The plain FP32 PyTorch-eager form (flowmc_gb300.plain) on the same
    workload: chain-steps/s over the loops from `timed_from` on, and (when
    the production phase is long enough) its min-ESS/s and moment error."""
    import torch
    from flowmc_gb300 import diagnostics as D
    from flowmc_gb300 import plain as PL
    if name == "rosenbrock128":
        vg = PL.rosenbrock_value_grad
    elif name == "dualmoon5":
        vg = PL.dual_moon_value_grad
    else:
        t, _, _ = make_target(name, w, dev)
        means = torch.tensor(t.means, dtype=torch.float32, device=dev)
        iv = torch.tensor(1.0 / t.var, dtype=torch.float32, device=dev)
        lw = torch.tensor(t.log_w, dtype=torch.float32, device=dev)
        vg = lambda x: PL.mixture_value_grad(x, means, iv, lw)
    g = torch.Generator().manual_seed(w["seed"])
    x0 = torch.randn(w["n_chains"], w["d"], generator=g).to(dev)
    gen = torch.Generator(device=dev).manual_seed(w["seed"] + 100)
    prod, secs, rates = PL.run_plain(w, vg, n_train, n_prod, x0, gen, timed_from=timed_from)
    loops = n_train + n_prod - timed_from
    out = {"value": w["n_chains"] * (w["n_local"] + w["n_global"]) * loops / secs, "unit": "chain-steps/s",
           "loops_timed": loops, "n_training_loops": n_train, "n_production_loops": n_prod, "seconds": secs,
           "acceptance": rates}
    if ess and n_prod >= 2:
        e = D.ess_bulk(prod)
        out["min_ess"] = float(e.min())
        out["min_ess_per_s"] = float(e.min()) / secs
        out["moment_error"] = D.moment_error(prod, mean_ref, var_ref)
    return out


def compare_arms(name, w, dev, T, P, precision, seeds, plain=True, graph=True):
    """Equal-work comparison at each seed: the fused bundle and the plain FP32
    form each run T training + P production loops from the same seed. Wall
    clock covers the whole schedule (training included, as ESS/s is
    defined). One-time costs are excluded in both arms: the fused arm warms
    up once (autotuning, workspace growth) on a sampler that is then
    dropped, and with `graph` each seed's schedule is captured as a CUDA
    graph before its timed replay (capture reported separately); the plain
    arm runs one untimed training + production loop first. min-ESS:
    rank-normalised bulk ESS over the production samples; moment error
    against the workload's reference moments. Returns the per-seed results
    and their means, with the ratios of the means (fused / plain)."""
    import numpy as np
    import torch
    from flowmc_gb300 import diagnostics as D
    prec = "bf16" if precision == "bf16" else "float32"
    out = {"workload": name, "training_loops": T, "production_loops": P, "seeds": list(seeds),
           "cuda_graph": graph, "precision": precision, "fused": [], "plain_fp32": []}
    # fused warm-up (untimed): one full schedule at the first seed
    sampler, _, _, _, _, x0 = build_sampler(name, dict(w, seed=seeds[0]), T, P, prec, dev)
    sampler.sample(x0, {})
    torch.cuda.synchronize()
    del sampler
    for sd in seeds:
        ws = dict(w, seed=sd)
        sampler, bundle, target, mean_ref, var_ref, x0 = build_sampler(name, ws, T, P, prec, dev)
        cap_ms = None
        if graph:
            torch.cuda.synchronize()
            c0 = time.perf_counter()
            cap = sampler.capture(x0, {})
            torch.cuda.synchronize()
            cap_ms = 1e3 * (time.perf_counter() - c0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if graph:
            cap.replay(x0)
        else:
            sampler.sample(x0, {})
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        pos = sampler.resources["positions_production"].data
        ess = D.ess_bulk(pos)
        f = {"seed": sd, "seconds": secs, "min_ess": float(ess.min()), "min_ess_per_s": float(ess.min()) / secs,
             "moment_error": D.moment_error(pos, mean_ref, var_ref),
             "chain_steps_per_s": w["n_chains"] * (w["n_local"] + w["n_global"]) * (T + P) / secs}
        if cap_ms is not None:
            f["graph_capture_ms"] = cap_ms
        out["fused"].append(f)
        del sampler, bundle, pos
        if graph:
            del cap
        if plain:
            if len(out["plain_fp32"]) == 0:
                # one untimed training + production loop: module loading and the
                # allocator's first growth are one-time costs in the plain arm too
                plain_arm(name, ws, dev, 1, 1, 0, mean_ref, var_ref, ess=False)
            pl = plain_arm(name, ws, dev, T, P, 0, mean_ref, var_ref)
            out["plain_fp32"].append({"seed": sd, "seconds": pl["seconds"], "min_ess": pl.get("min_ess"),
                                      "min_ess_per_s": pl.get("min_ess_per_s"),
                                      "moment_error": pl.get("moment_error"), "chain_steps_per_s": pl["value"]})
        torch.cuda.empty_cache()

    def stat(rows, k, f):
        v = [r[k] for r in rows if r.get(k) is not None]
        return f(v) if len(v) > (1 if f is _sd else 0) else None

    summ = {}
    for arm in ("fused", "plain_fp32"):
        if out[arm]:
            summ[arm] = {k: stat(out[arm], k, _mean) for k in ("min_ess_per_s", "moment_error",
                                                                "chain_steps_per_s", "seconds")}
            summ[arm]["moment_error_sd"] = stat(out[arm], "moment_error", _sd)
    out["mean"] = summ
    if "plain_fp32" in summ and summ["plain_fp32"]["min_ess_per_s"]:
        fm, pm = summ["fused"], summ["plain_fp32"]
        out["ratio_min_ess_per_s"] = fm["min_ess_per_s"] / pm["min_ess_per_s"]
        out["ratio_moment_error"] = fm["moment_error"] / pm["moment_error"]
        out["ratio_chain_steps_per_s"] = fm["chain_steps_per_s"] / pm["chain_steps_per_s"]
    return out


def _mean(v):
    return float(sum(v) / len(v))


def _sd(v):
    m = _mean(v)
    return float((sum((x - m) ** 2 for x in v) / (len(v) - 1)) ** 0.5)


def moment_trajectory(name, w, dev, n_loops, precision):
    """The fused bundle for n_loops training + n_loops production loops; the
    moment error and min-ESS of the production rows written so far, after
    every production loop (does the workload converge on this schedule?)."""
    import torch
    from flowmc_gb300 import diagnostics as D
    prec = "bf16" if precision == "bf16" else "float32"
    sampler, bundle, target, mean_ref, var_ref, x0 = build_sampler(name, w, n_loops, n_loops, prec, dev)
    segs = loop_segments(bundle.strategy_order, n_loops, len(bundle.training_phase), len(bundle.production_phase))
    x, key = x0.to(dev), sampler.rng_key
    blk = w["n_local"] + w["n_global"]
    rows = []
    for i, seg in enumerate(segs):
        for s in seg:
            key, sampler.resources, x = sampler.strategies[s](key, sampler.resources, x, {})
        if i >= n_loops:
            k = i - n_loops + 1
            pos = sampler.resources["positions_production"].data[:, :k * blk]
            ess = D.ess_bulk(pos) if k >= 2 else None
            rows.append({"production_loops": k, "moment_error": D.moment_error(pos, mean_ref, var_ref),
                         "min_ess": float(ess.min()) if ess is not None else None})
    torch.cuda.synchronize()
    return {"workload": name, "training_loops": n_loops, "production_loops": n_loops, "rows": rows}


# ---------------------------------------------------------------- CPU baseline
def oracle_target(name, w):
    """The workload's target as an oracle target dict."""
    import numpy as np
    d = w["d"]
    if name == "rosenbrock128":
        return {"kind": "rosenbrock", "n_dim": d, "a": 20.0, "b": 1.0, "c": 5.0}
    if name == "dualmoon5":
        return {"kind": "dual_moon", "n_dim": d, "r0": 2.0, "sr": 0.1, "mu": 3.0, "s0": 0.6}
    return {"kind": "mixture", "mean": mixture_means(), "inv_var": np.full((4, 64), 2.0),
            "log_w": np.full(4, np.log(0.25) - 32 * np.log(2 * np.pi * 0.5))}


class OracleBundle:
    """The bundle's loop restated by the oracle (float64 NumPy on the host
    cores, BLAS threads on every core), on a bounded sample of the workload:
    `n_chains` chains of the same target, local kernel, step counts and flow
    shape. A training loop (between its local and global phase, as the
    bundle's schedule has it, RQSpline_MALA.py:251-273) selects `n_max` rows
    from the last 100 rows of every chain (train_model.py:66-80) and takes
    n_epochs AdamW steps on them, one full batch per epoch (the reference's
    rule when batch_size > n_max_examples, nf_model/base.py:148-149)."""

    def __init__(self, name, w, n_chains, n_max, seed=0):
        import numpy as np
        from oracle import flow as OF
        self.np = np
        self.w, self.C, self.n_max = w, n_chains, n_max
        self.rng = np.random.default_rng(seed)
        self.t = oracle_target(name, w)
        d = w["d"]
        P = 3 * w["n_bins"] + 1
        layers = []
        for i in range(w["n_layers"]):
            shape = [d] + w["hidden"] + [d * P]
            layers.append({"W": [self.rng.normal(size=(b, a)) * 0.05 / np.sqrt(a)
                                 for a, b in zip(shape[:-1], shape[1:])],
                           "b": [np.zeros(b) for b in shape[1:]], "scale": 0.0, "shift": 0.0,
                           "mask": ((np.arange(d) + i) % 2).astype(bool)})
        self.flow = OF.Flow(layers, w["n_bins"], np.zeros(d), np.eye(d))
        n_par = OF.flatten(self.flow).size
        self.st = OF.AdamWState(np.zeros(n_par), np.zeros(n_par))
        self.x = self.rng.normal(size=(n_chains, d))
        self.hist = np.zeros((n_chains, 0, d))

    def loop(self, train: bool):
        from oracle import flow as OF
        from oracle import flow_torch as OFT
        from oracle import kernels as OK
        np, w, C, d = self.np, self.w, self.C, self.w["d"]
        S1, S2 = w["n_local"], w["n_global"]
        pos, _, _, self.x = OK.take_serial_steps(w["local"], self.t, self.x, S1, self.rng.normal(size=(C, S1, d)),
                                                 self.rng.uniform(size=(C, S1)), step_size=w["step"],
                                                 n_leapfrog=w["n_leapfrog"], M=np.eye(d))
        self.hist = np.concatenate([self.hist, pos], 1)[:, -100:]
        if train:
            idx = self.rng.integers(0, self.hist.shape[0] * self.hist.shape[1], size=self.n_max)
            data = OF.select_training_data(self.hist, 100, idx)
            self.flow.data_mean = data.mean(0)
            self.flow.data_cov = np.diag(data.var(0, ddof=1))
            for _ in range(w["n_epochs"]):
                _, g = OFT.loss_and_grad(self.flow, data)
                p, _ = OF.adamw_update(OF.flatten(self.flow), g, self.st, w["lr"])
                OF.unflatten(self.flow, p)
        gx, _, _ = OK.nf_proposal_kernel(self.flow, self.t, self.x, self.rng.normal(size=(C, S2, d)),
                                         self.rng.uniform(1e-12, 1.0, size=(C, S2)))
        self.x = gx[:, -1]
        self.hist = np.concatenate([self.hist, gx], 1)[:, -100:]


REF_CHAINS, REF_MAX = 8, 64


def ref_sample_text(w, C, n_max):
    return (f"oracle float64 NumPy restatement of the bundle loop on {C} of the {w['n_chains']} chains "
            f"(same target, {w['local']} kernel, {w['n_local']} local + {w['n_global']} global steps, "
            f"{w['n_layers']}x{w['hidden']}x{w['n_bins']} flow); training loops select {n_max} of the "
            f"{w['n_max']} examples and take {w['n_epochs']} full-batch AdamW steps")


def cpu_baseline(name, w, budget_s: float = 20.0):
    """The oracle restatement timed on the host cores on a bounded sample of
    the workload (OracleBundle on REF_CHAINS chains): one training loop and
    then production loops until about `budget_s` seconds have passed. The
    value is the measured chain-steps/s of that sample, not a projection."""
    ob = OracleBundle(name, w, REF_CHAINS, REF_MAX, seed=w["seed"])
    t0 = time.perf_counter()
    ob.loop(True)
    loops = 1
    while time.perf_counter() - t0 < budget_s and loops < 40:
        ob.loop(False)
        loops += 1
    secs = time.perf_counter() - t0
    return {"value": REF_CHAINS * (w["n_local"] + w["n_global"]) * loops / secs, "unit": "chain-steps/s",
            "cores": os.cpu_count(), "kind": "port",
            "sample": ref_sample_text(w, REF_CHAINS, REF_MAX) + f"; measured over 1 training + {loops - 1} "
                      f"production loops in {secs:.1f} s"}


def schedule(W, K):
    """(training loops, production loops) of a W + K loop run: the first half
    (at least W) trains."""
    n_total = W + K
    n_train = max(W, n_total // 2)
    return n_train, n_total - n_train


def workload_config(name, w, W, K, world):
    n_train, n_prod = schedule(W, K)
    return {"workload": name, "n_dim": w["d"], "n_chains": w["n_chains"], "local_kernel": w["local"],
            "step_size": w["step"], "n_leapfrog": w["n_leapfrog"],
            "n_local_steps": w["n_local"], "n_global_steps": w["n_global"],
            "flow": f"{w['n_layers']}x{w['hidden']}x{w['n_bins']} bins", "learning_rate": w["lr"],
            "n_training_loops": n_train, "n_production_loops": n_prod, "timed_loops": K, "batch_size": w["batch"],
            "n_epochs": w["n_epochs"], "n_max_examples": w["n_max"], "parallelism": f"replicas{world}",
            "l2": "working set (chain buffers, flow weights) larger than L2; no flush"}


def reference_arm(args, w):
    """The reference's CPU path (the oracle restatement; JAX is not in the
    image) on the same workload and schedule: W untimed warm-up loops, then
    the K timed loops, each one loop of OracleBundle on REF_CHAINS chains
    (training loops first, as in the fused arm). value = the sample's
    chain-steps over the timed loops / their measured wall time."""
    W, K = max(1, args.warmup), max(1, args.steps)
    n_train, _ = schedule(W, K)
    ob = OracleBundle(args.workload, w, REF_CHAINS, REF_MAX, seed=w["seed"])
    for i in range(W):
        ob.loop(i < n_train)
    t0 = time.perf_counter()
    for i in range(W, W + K):
        ob.loop(i < n_train)
    secs = time.perf_counter() - t0
    value = REF_CHAINS * (w["n_local"] + w["n_global"]) * K / secs
    sample = ref_sample_text(w, REF_CHAINS, REF_MAX) + f"; {K} timed loops in {secs:.1f} s"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "chain-steps/s", "n_gpus": args.gpus,
            "steps": K, "warmup": W, "ms_per_step": 1e3 * secs / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.workload, w, W, K, args.gpus),
            "cpu_baseline": {"value": value, "unit": "chain-steps/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "chain-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- main
def kernel_trace(path, fn, cmd):
    """Per-kernel launch list of fn() from CUPTI activity records (torch.profiler):
    launches, total device time and share per kernel name, written as text."""
    import torch
    from torch.profiler import profile, ProfilerActivity
    import tempfile
    # the first activity session of a process can come back empty: open one
    # on a trivial op first
    with profile(activities=[ProfilerActivity.CUDA]):
        torch.ones(1, device="cuda").add_(1)
        torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with profile(activities=[ProfilerActivity.CUDA]) as p:
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
    elapsed = e0.elapsed_time(e1)
    # kernels launched outside torch ops only appear in the raw activity trace
    with tempfile.TemporaryDirectory() as td:
        tp = os.path.join(td, "trace.json")
        p.export_chrome_trace(tp)
        with open(tp) as f:
            events = json.load(f).get("traceEvents", [])
    rows = {}
    cats = {}
    for ev in events:
        cat = ev.get("cat", "")
        cats[cat] = cats.get(cat, 0) + 1
        if cat.lower() not in ("kernel", "gpu_memcpy", "gpu_memset"):
            continue
        name = ev.get("name", "")
        key = name.split("(")[0].replace("void ", "") if cat == "kernel" else cat + " " + name.split(" ")[0]
        n, t = rows.get(key, (0, 0.0))
        rows[key] = (n + 1, t + float(ev.get("dur", 0.0)) / 1e3)
    total = sum(t for _, t in rows.values())
    if not rows:
        print(json.dumps({"kernel_trace": path, "error": "no device activity records", "categories": cats}),
              flush=True)
        return
    with open(path, "w") as f:
        f.write(f"# {cmd} --kernel-trace {os.path.basename(path)}\n")
        f.write("# per kernel: launches, device ms (sum over launches), share of device time\n")
        for k, (n, t) in sorted(rows.items(), key=lambda kv: -kv[1][1]):
            f.write(f"{k:60s} {n:8d} {t:12.3f} {100 * t / total:7.2f}%\n")
        f.write(f"{'total':60s} {sum(n for n, _ in rows.values()):8d} {total:12.3f}\n")
        f.write(f"# elapsed (CUDA events around the loops, under the profiler): {elapsed:.3f} ms; "
                f"kernels busy {100 * total / elapsed:.1f} % of it\n")
    print(json.dumps({"kernel_trace": path, "device_ms": total, "elapsed_ms": elapsed, "kernels": len(rows)}),
          flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=37)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fused", choices=["fused", "reference"])
    ap.add_argument("--workload", default="rosenbrock128", choices=list(WORKLOADS))
    ap.add_argument("--precision", default="bf16", choices=["bf16", "fp32"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ess", action="store_true")
    ap.add_argument("--chains", type=int, default=0, help="override n_chains (small profiling cases)")
    ap.add_argument("--plain-loops", type=int, default=2,
                    help="loops of the plain FP32 form timed for its chain-steps/s (0 = skip)")
    ap.add_argument("--probe", default="", choices=["", "local", "batched", "train", "pt", "realnvp", "adam"],
                    help="run only the local-step HBM probe (a small profiling target)")
    ap.add_argument("--kernel-trace", default="",
                    help="write a per-kernel launch list (CUPTI activity timestamps) of the K loops to this "
                         "file instead of the bench line; its times are not bench values")
    ap.add_argument("--seeds", default="",
                    help="with --compare: comma-separated workload seeds; both arms run each")
    ap.add_argument("--compare", default="",
                    help="T,P: fused bundle and plain FP32 form on the same workload and seeds with T training + P "
                         "production loops each; prints their min-ESS/s and moment errors instead of the bench line")
    ap.add_argument("--no-plain", action="store_true", help="with --compare: the fused arm only")
    ap.add_argument("--cmp-workload", default="mixture64", choices=list(WORKLOADS),
                    help="workload of the equal-work comparison carried by the bench line")
    ap.add_argument("--cmp-loops", default="2,20", help="T,P of that comparison (empty: skip it)")
    ap.add_argument("--cmp-seeds", default="3,4,5,6", help="seeds of that comparison")
    ap.add_argument("--trajectory", type=int, default=0,
                    help="run T training + T production loops of the fused bundle and print the moment error of "
                         "the production rows after every production loop")
    ap.add_argument("--batched-steps", type=int, default=2000, help="steps of --probe batched")
    ap.add_argument("--eager", action="store_true",
                    help="launch the timed loops eagerly instead of replaying them as one captured CUDA graph")
    ap.add_argument("--plain-full", action="store_true",
                    help="run the plain FP32 form on the full schedule (min-ESS/s, moment error)")
    args = ap.parse_args()
    w = dict(WORKLOADS[args.workload])
    if args.chains > 0:
        w["n_chains"] = args.chains
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, w)
        return

    import torch
    import torch.distributed as dist
    from flowmc_gb300 import _lib
    from flowmc_gb300 import diagnostics as D
    from flowmc_gb300 import profiling

    from flowmc_gb300 import replicas

    if world > 1:
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", rank=rank, world_size=world)
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    # independent replicas: every rank samples its own chains
    w["seed"] = replicas.replica_seed(w["seed"], rank)
    if args.probe == "batched":
        print(json.dumps({"probe": "batched_dense", "mala": batched_probe(dev, "mala", steps=args.batched_steps),
                          "hmc": batched_probe(dev, "hmc", steps=args.batched_steps)}), flush=True)
        return
    if args.probe == "train":
        print(json.dumps({"probe": "flow_training_d32", "bf16": train_probe(dev, "bf16"),
                          "fp32": train_probe(dev, "fp32")}), flush=True)
        return
    if args.probe == "pt":
        print(json.dumps({"probe": "parallel_tempering", **pt_probe(dev)}), flush=True)
        return
    if args.probe == "realnvp":
        print(json.dumps({"probe": "realnvp", **realnvp_probe(dev)}), flush=True)
        return
    if args.probe == "adam":
        print(json.dumps({"probe": "adam_optimization", **adam_probe(dev)}), flush=True)
        return
    if args.probe == "local":
        print(json.dumps({"probe": "local_steps", **local_hbm_probe(dev, chains=w["n_chains"] if args.chains else 65536,
                                                                     lanes=(0, 8, 16, 32))}), flush=True)
        return
    if args.compare:
        T, P = (int(v) for v in args.compare.split(","))
        seeds = [int(v) for v in args.seeds.split(",")] if args.seeds else [w["seed"]]
        res = compare_arms(args.workload, w, dev, T, P, args.precision, seeds, plain=not args.no_plain,
                           graph=not args.eager)
        print(json.dumps({"compare": res}), flush=True)
        return
    if args.trajectory:
        print(json.dumps({"trajectory": moment_trajectory(args.workload, w, dev, args.trajectory,
                                                          args.precision)}), flush=True)
        return
    W, K = max(1, args.warmup), max(1, args.steps)
    n_total = W + K
    n_train, n_prod = schedule(W, K)
    precision = "bf16" if args.precision == "bf16" else "float32"
    sampler, bundle, target, mean_ref, var_ref, x0 = build_sampler(args.workload, w, n_train, n_prod, precision, dev)
    segs = loop_segments(bundle.strategy_order, n_train, len(bundle.training_phase), len(bundle.production_phase))
    assert len(segs) == n_total

    def run(segments, x, key):
        for seg in segments:
            for s in seg:
                key, sampler.resources, x = sampler.strategies[s](key, sampler.resources, x, {})
        return x, key

    x = x0.to(dev)
    key = sampler.rng_key
    x, key = run(segs[:W], x, key)
    torch.cuda.synchronize()
    if args.kernel_trace:
        kernel_trace(args.kernel_trace, lambda: run(segs[W:], x, key),
                     f"python bench.py --steps {K} --warmup {W} --workload {args.workload} "
                     f"--precision {args.precision}" + (f" --chains {args.chains}" if args.chains else ""))
        return
    graph = None
    capture_ms = None
    prof = profiling.Profiler()
    if not args.eager:
        # the K timed loops as one CUDA graph (untimed one-time setup, reported
        # as graph_capture_ms); the Profiler's regions become event-record
        # nodes, so the replay times the same phases
        epoch = _lib.rng_epoch(dev)
        l0 = _lib.launch_count()
        torch.cuda.synchronize()
        c0 = time.perf_counter()
        graph = torch.cuda.CUDAGraph()
        with prof, torch.cuda.graph(graph):
            _lib.rng_epoch_advance(epoch)
            x_g, key_g = run(segs[W:], x, key)
        capture_ms = (time.perf_counter() - c0) * 1e3
        launches = _lib.launch_count() - l0
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    if graph is not None:
        e0.record()
        graph.replay()
        e1.record()
        torch.cuda.synchronize()
        x, key = x_g, key_g
    else:
        l0 = _lib.launch_count()
        with prof:
            e0.record()
            x, key = run(segs[W:], x, key)
            e1.record()
            torch.cuda.synchronize()
        launches = _lib.launch_count() - l0
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    ms = replicas.max_over_ranks(e0.elapsed_time(e1), dev)
    if world > 1:
        dist.barrier()
    secs = ms / 1e3
    chain_steps = w["n_chains"] * (w["n_local"] + w["n_global"]) * K
    value = replicas.job_throughput(chain_steps, secs, world)

    # ---- diagnostics on the production samples
    pos = sampler.resources["positions_production"].data
    extra = {}
    if not args.no_ess:
        ess = D.ess_bulk(pos)
        extra["min_ess"] = float(ess.min())
        extra["min_ess_per_s"] = float(ess.min()) * world / secs
        extra["moment_error"] = D.moment_error(pos, mean_ref, var_ref)
    if bundle.production_moments is not None:
        # the device's streaming FP64 accumulators (updated inside the timed
        # region after every production loop) against the post-hoc values
        sm = bundle.production_moments.finalize()
        mu_p, var_p = D.moments(pos)
        extra["streaming"] = {
            "moment_error": D.moment_error_of(sm["mean"], sm["var"], mean_ref, var_ref),
            "min_ess_batch_means": float(torch.nan_to_num(sm["ess"], nan=float("inf")).min()),
            "max_rhat": float(sm["rhat"].max()), "batch": bundle.production_moments.batch,
            "max_abs_mean_diff_vs_posthoc": float((sm["mean"] - mu_p).abs().max()),
            "max_rel_var_diff_vs_posthoc": float(((sm["var"] - var_p) / var_p).abs().max())}
    acc_l = sampler.resources["local_accs_production"].data
    acc_g = sampler.resources["global_accs_production"].data
    # local rows are the first n_local of each 80-row loop block
    blk = w["n_local"] + w["n_global"]
    la = acc_l.reshape(w["n_chains"], -1, blk)[:, :, :w["n_local"]].mean().item()
    ga = acc_g.reshape(w["n_chains"], -1, blk)[:, :, w["n_local"]:].mean().item()
    extra["acceptance"] = {"local": la, "global": ga}

    # ---- per phase (device time from CUDA events inside the timed region)
    hbm, bf16, bf16_s, src = measured_peaks()
    tot = prof.totals_ms()
    cnt = prof.counts()
    kernels = {}
    ff = useful_flow_flops(w)
    if "local_steps" in tot:
        n_cs = prof.units["local_steps"]
        bytes_ = n_cs * (4 * w["d"] + 8)
        t_s = tot["local_steps"] / 1e3
        evals = (w["n_leapfrog"] + 1) if w["local"] == "hmc" else 1
        flops = n_cs * evals * 15 * w["d"]
        kernels["local_steps"] = {"ms": tot["local_steps"], "launches": cnt["local_steps"],
                                  "achieved_gbs": bytes_ / t_s / 1e9, "frac_hbm": bytes_ / t_s / 1e9 / hbm,
                                  "fp32_tflops": flops / t_s / 1e12,
                                  "bytes_per_chain_step": 4 * w["d"] + 8}
    if "nf_global" in tot:
        props = prof.units["nf_global"]
        flops = (2 * props + props / w["n_global"]) * ff
        t_s = tot["nf_global"] / 1e3
        kernels["nf_global"] = {"ms": tot["nf_global"], "launches": cnt["nf_global"],
                                "achieved_tflops": flops / t_s / 1e12, "frac_bf16_sustained": flops / t_s / 1e12 / bf16_s,
                                "useful_flops_per_sample_pass": ff}
    if "train" in tot:
        steps = prof.units["train"]
        flops = steps * w["batch"] * 3 * ff
        t_s = tot["train"] / 1e3
        kernels["train"] = {"ms": tot["train"], "launches": cnt["train"], "achieved_tflops": flops / t_s / 1e12,
                            "frac_bf16_sustained": flops / t_s / 1e12 / bf16_s}

    # ---- per kernel: CUDA events around every launch (library timers, on the
    # launch stream) over one eager training loop and one eager production
    # loop run after the timed region, weighted by the timed mix
    n_tr_timed = max(0, n_train - W)
    per_k = kernel_timing_pass(sampler, bundle, segs, x, key, n_train, n_tr_timed, K - n_tr_timed, w, hbm, bf16_s)
    kernels["per_kernel"] = per_k
    roof = roofline_line(per_k, hbm, bf16, bf16_s, src, w)

    kernels["local_steps_hbm_probe"] = local_hbm_probe(dev, lanes=(0, 8, 16, 32))
    # parallel tempering, RealNVP and Adam optimisation, each on its own probe workload (seconds in total)
    kernels["parallel_tempering_probe"] = pt_probe(dev)
    kernels["realnvp_probe"] = realnvp_probe(dev)
    kernels["adam_optimization_probe"] = adam_probe(dev)

    # ---- end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = end_to_end(sampler, bundle, w, dev, n_train - W, n_prod, x, graph=not args.eager)

    line = {
        "metric": METRIC, "value": value, "unit": "chain-steps/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16" if args.precision == "bf16" else "f32", "data": "synthetic",
        "config": workload_config(args.workload, w, W, K, world),
        "autotuned": {"lanes_per_chain": getattr(sampler.resources["local_sampler"], "lanes_per_chain", 0),
                      "flow_gemm_bn": getattr(sampler.resources["model"], "gemm_bn", 0),
                      "flow_tile_rows": getattr(sampler.resources["model"], "tile_rows", 0),
                      "flow_gemm_stages": getattr(sampler.resources["model"], "gemm_stages", 0),
                      "flow_tile_timings_ms": getattr(sampler.resources["model"], "tile_timings_ms", None),
                      "wgrad_splits": getattr(sampler.resources["model"], "wgrad_splits", 0),
                      "wgrad_timings_ms": getattr(sampler.resources["model"], "train_timings_ms", None)},
        "roofline": roof, "kernels": kernels, "gpu_launches": launches, "clocks": clk,
        "wall_s": wall, "cuda_graph": graph is not None, **extra,
    }
    if capture_ms is not None:
        line["graph_capture_ms"] = capture_ms
    if e2e is not None:
        line["e2e"] = e2e
    del sampler, bundle, pos
    graph = None
    torch.cuda.empty_cache()
    ratio = {}
    if rank == 0 and (args.plain_full or args.plain_loops > 0):
        if args.plain_full:
            pl = plain_arm(args.workload, w, dev, n_train, n_prod, W, mean_ref, var_ref)
        else:
            nt = max(1, args.plain_loops // 2)
            pl = plain_arm(args.workload, w, dev, nt, args.plain_loops - nt, 0, mean_ref, var_ref, ess=False)
        line["plain_fp32"] = pl
        ratio = {"workload": args.workload, "chain_steps_per_s": value / pl["value"]}
        if "min_ess_per_s" in pl and "min_ess_per_s" in line:
            ratio["min_ess_per_s"] = line["min_ess_per_s"] / pl["min_ess_per_s"]
            ratio["moment_error_ratio"] = line["moment_error"] / pl["moment_error"]
    if rank == 0 and args.cmp_loops:
        # the equal-work, converged comparison of the two forms (both arms
        # trained, several seeds), on its own workload
        T, P = (int(v) for v in args.cmp_loops.split(","))
        seeds = [int(v) for v in args.cmp_seeds.split(",")]
        wc = dict(WORKLOADS[args.cmp_workload])
        cmp_ = compare_arms(args.cmp_workload, wc, dev, T, P, args.precision, seeds, plain=True, graph=True)
        line["comparison"] = cmp_
        if "ratio_min_ess_per_s" in cmp_:
            ratio["comparison"] = {"workload": args.cmp_workload, "seeds": seeds,
                                   "min_ess_per_s": cmp_["ratio_min_ess_per_s"],
                                   "moment_error_ratio": cmp_["ratio_moment_error"],
                                   "chain_steps_per_s": cmp_["ratio_chain_steps_per_s"],
                                   "fused_moment_error": cmp_["mean"]["fused"]["moment_error"],
                                   "plain_moment_error": cmp_["mean"]["plain_fp32"]["moment_error"]}
            ratio["min_ess_per_s"] = cmp_["ratio_min_ess_per_s"]
            ratio["moment_error_ratio"] = cmp_["ratio_moment_error"]
    if ratio:
        line["fused_over_plain"] = ratio
    if rank == 0 and not args.no_cpu:
        try:
            line["cpu_baseline"] = cpu_baseline(args.workload, w)
        except Exception as ex:  # the baseline must not sink the GPU line
            line["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def kernel_timing_pass(sampler, bundle, segs, x, key, n_train, n_tr_timed, n_pr_timed, w, hbm, bf16_s):
    """Per-kernel CUDA-event times (the library's launch timers) over one
    training loop and one production loop of the same sampler, each captured
    as a CUDA graph with the timers' event nodes in it and replayed (kernels
    back to back, as in the timed region); totals are weighted to the timed
    mix (n_tr_timed training + n_pr_timed production loops). For the
    tensor-core kernels: algorithmic FLOPs per launch over the average launch
    time against the sustained BF16 peak (they run inside a long step); the
    others against HBM bandwidth."""
    import torch
    from flowmc_gb300 import _lib
    res = {}
    runs = (("train", segs[0], n_tr_timed), ("production", segs[-1], n_pr_timed))
    for tag, seg, weight in runs:
        torch.cuda.synchronize()
        _lib.kernel_timing(True)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for s in seg:
                key, sampler.resources, x = sampler.strategies[s](key, sampler.resources, x, {})
        _lib.kernel_timing(False)
        g.replay()          # warm (the first replay uploads the graph)
        g.replay()
        torch.cuda.synchronize()
        got = _lib.kernel_timing_read()
        del g
        for k, v in got.items():
            r = res.setdefault(k, {"launches_per_loop": {}, "ms": 0.0, "launches": 0.0, "flops": 0.0,
                                   "bytes": 0.0})
            r["launches_per_loop"][tag] = v["launches"]
            r["ms"] += weight * v["ms"]
            r["launches"] += weight * v["launches"]
            r["flops"] += weight * v["flops"]
            r["bytes"] += weight * v["bytes"]
    out = {}
    total = sum(r["ms"] for r in res.values()) or 1.0
    for k, r in sorted(res.items(), key=lambda kv: -kv[1]["ms"]):
        n = max(r["launches"], 1.0)
        o = {"launches_per_loop": r["launches_per_loop"], "avg_us": 1e3 * r["ms"] / n,
             "timed_mix_ms": r["ms"], "share_of_timed_kernels": r["ms"] / total}
        if r["flops"] > 0:
            o["flops_per_launch"] = r["flops"] / n
            o["achieved_tflops"] = r["flops"] / (r["ms"] / 1e3) / 1e12
            o["frac_bf16_sustained"] = o["achieved_tflops"] / bf16_s
        if r["bytes"] > 0:
            o["bytes_per_launch"] = r["bytes"] / n
            o["achieved_gbs"] = r["bytes"] / (r["ms"] / 1e3) / 1e9
            o["frac_hbm"] = o["achieved_gbs"] / hbm
        out[k] = o
    out["_how"] = ("CUDA events recorded by the library on each launch's stream around every launch of one "
                   "training loop and one production loop, each captured as a CUDA graph and replayed, weighted to "
                   "the timed loop mix")
    return out


def spline_operand_traffic(w, rows):
    """Operand traffic of one k_tc_spline launch over `rows` rows of the
    workload's flow (analytic): every (128-row, group) tile loads its A tile
    and the group's weights from L2 into shared memory, plus the epilogue's
    reads and writes of x and its log-det partials. Most of it is L2 -> SMEM
    (A and the weights are L2-resident); ncu is not run on the tcgen05
    kernels here, so this model stands in for dram__bytes."""
    P = 3 * w["n_bins"] + 1
    dg = 256 // P
    bn = ((dg * P + 15) // 16) * 16
    nt = w["d"] // 2
    groups = -(-nt // dg)
    H = w["hidden"][-1]
    tiles = -(-rows // 128) * groups
    return tiles * (128 * H * 2 + bn * H * 2) + rows * nt * 8 + rows * 3 * groups * 4


def roofline_line(per_k, hbm, bf16, bf16_s, src, w):
    """The dominant kernel of the timed mix (largest share of per-kernel event
    time) with its achieved rate against the sustained peak. For the fused
    spline kernels `traffic` is the analytic per-launch operand traffic
    (spline_operand_traffic); ncu is not run on the tcgen05 kernels here."""
    ks = [k for k in per_k if not k.startswith("_")]
    dom = max(ks, key=lambda k: per_k[k]["timed_mix_ms"])
    d = per_k[dom]
    if "achieved_tflops" in d and dom.startswith("k_tc"):
        r = {"bound": "tensor", "kernel": dom, "achieved": d["achieved_tflops"], "peak": bf16_s,
             "unit": "TFLOP/s", "frac": d["achieved_tflops"] / bf16_s, "traffic": None,
             "peak_source": f"{src} bf16_tflops_sustained (kernel timed inside a long step)",
             "avg_launch_us": d["avg_us"], "flops_per_launch": d["flops_per_launch"]}
        if dom in ("k_tc_spline_fwd", "k_tc_spline_inv"):
            P = 3 * w["n_bins"] + 1
            rows = d["flops_per_launch"] / (2.0 * (w["d"] // 2) * P * w["hidden"][-1])
            r["traffic"] = spline_operand_traffic(w, int(round(rows)))
            r["traffic_source"] = ("analytic: A and weight tiles loaded L2 -> shared memory per (128-row, group) "
                                   "tile plus the epilogue's x and partials, per launch; ncu is not run on the "
                                   "tcgen05 kernels on this pool")
            r["rows_per_launch"] = rows
        return r
    return {"bound": "hbm", "kernel": dom, "achieved": d.get("achieved_gbs"), "peak": hbm, "unit": "GB/s",
            "frac": (d.get("achieved_gbs") or 0.0) / hbm, "traffic": None, "peak_source": src,
            "avg_launch_us": d["avg_us"]}


def end_to_end(sampler, bundle, w, dev, n_train_loops, n_prod_loops, x_dev, graph=True):
    """The timed region's loop mix (n_train_loops training loops, then
    n_prod_loops production loops) driven through Sampler.sample with host
    buffers: every loop copies its starting positions host->device (pinned,
    inside Sampler.sample) and reads back the rows it wrote plus the final
    positions (device->host, pinned). With ``graph`` each loop is a replay of
    its schedule's CUDA graph (Sampler.sample(..., cuda_graph=True)); the two
    schedules are captured before the timed region. A loop's rows are staged
    to a device buffer (the next loop rewrites the same rows) and copied to
    one of two pinned host buffers on a second stream while the next loop
    runs; the final positions go back to the host on the compute stream, in
    order before the next loop's host->device copy of them. The clock stops
    after every copy has landed."""
    import torch
    train = ["local_stepper", "update_global_step", "model_trainer", "update_model", "global_stepper",
             "update_local_step"]
    prod = ["local_stepper", "update_global_step", "global_stepper", "update_local_step"]
    C, d = w["n_chains"], w["d"]
    blk = w["n_local"] + w["n_global"]
    x_host = torch.empty(C, d, pin_memory=True)
    x_host.copy_(x_dev)
    pos_h = [torch.empty(C, blk, d, pin_memory=True) for _ in range(2)]
    lp_h = [torch.empty(C, blk, pin_memory=True) for _ in range(2)]
    pos_s = [torch.empty(C, blk, d, device=dev) for _ in range(2)]
    lp_s = [torch.empty(C, blk, device=dev) for _ in range(2)]
    copy_stream = torch.cuda.Stream(device=dev)
    done = [None, None]
    res = sampler.resources
    state = res["sampler_state"]
    steppers = [sampler.strategies["local_stepper"], sampler.strategies["global_stepper"]]
    plan = [train] * n_train_loops + [prod] * n_prod_loops
    capture_ms = 0.0
    if graph:
        for order in (train, prod):
            if order in plan:
                sampler.strategy_order = order
                for s in steppers:
                    s.set_current_position(0)
                c0 = time.perf_counter()
                sampler.capture(x_dev, {})
                capture_ms += (time.perf_counter() - c0) * 1e3

    def loop(i, order):
        sampler.strategy_order = order
        for s in steppers:
            s.set_current_position(0)
        last = sampler.sample(x_host, {}, cuda_graph=graph)   # h2d inside Sampler.sample
        b = i % 2
        cur = torch.cuda.current_stream()
        if done[b] is not None:
            cur.wait_event(done[b])   # the copy of loop i - 2 has left staging buffer b
        pos_s[b].copy_(res[state.data["target_positions"]].data[:, :blk])
        lp_s[b].copy_(res[state.data["target_log_prob"]].data[:, :blk])
        x_host.copy_(last, non_blocking=True)   # ordered before the next loop's h2d on this stream
        staged = cur.record_event()
        copy_stream.wait_event(staged)
        with torch.cuda.stream(copy_stream):
            pos_h[b].copy_(pos_s[b], non_blocking=True)
            lp_h[b].copy_(lp_s[b], non_blocking=True)
            done[b] = copy_stream.record_event()

    # one untimed production loop per host buffer first: the first
    # device->host read into fresh pinned memory costs a one-time ~0.6 s on
    # the Grace host
    loop(0, prod)
    loop(1, prod)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i, order in enumerate(plan):
        loop(i, order)
    torch.cuda.synchronize()
    copy_stream.synchronize()
    secs = time.perf_counter() - t0
    h2d = C * d * 4
    d2h = C * blk * d * 4 + C * blk * 4 + C * d * 4
    out = {"value": C * blk * len(plan) / secs, "unit": "chain-steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "training_loops": n_train_loops, "production_loops": n_prod_loops,
           "cuda_graph": graph}
    if graph:
        out["graph_capture_ms"] = capture_ms
    return out


if __name__ == "__main__":
    main()
