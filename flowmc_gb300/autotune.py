"""Autotuners: the chain-block shape of the fused local-step kernel and the
tile width of the flow's tensor-core GEMMs.

The local-step kernel assigns each chain to a group of G lanes (4, 8, 16 or
32) holding V = next_pow2(d / G) coordinates each. Which G is fastest depends
on the kernel kind, the target's cost per coordinate and the number of
chains (occupancy versus shuffle depth), so it is measured: each candidate
runs a short probe of the real launch (same target, chain count and kernel,
a few steps into a scratch buffer), timed with CUDA events, and the fastest
is cached per (kernel kind, target kind, dimension, chain count) and written
to ``kernel.lanes_per_chain``.
"""
from __future__ import annotations

import torch

_cache: dict = {}


def candidates(d: int) -> list[int]:
    out = []
    for g in (4, 8, 16, 32):
        v = 1
        while g * v < d:
            v *= 2
        if v <= 8:
            out.append(g)
    return out


def tune_local_kernel(kernel, target, n_chains: int, probe_steps: int = 8, reps: int = 3) -> int:
    """Pick lanes_per_chain for (kernel, target, n_chains); returns it."""
    from .resource.kernel.base import run_local_steps
    d = target.n_dim
    key = (type(kernel).__name__, target.kind, d, n_chains, getattr(kernel, "n_leapfrog", 0))
    if key in _cache:
        kernel.lanes_per_chain = _cache[key]
        return _cache[key]
    dev = target.device if target.device.type == "cuda" else torch.device("cuda")
    x0 = torch.randn(n_chains, d, device=dev) * 0.1
    pos = torch.empty(n_chains, probe_steps, d, device=dev)
    lp = torch.empty(n_chains, probe_steps, device=dev)
    acc = torch.empty(n_chains, probe_steps, device=dev)
    saved = kernel.lanes_per_chain
    best, best_ms = saved, float("inf")
    for g in candidates(d):
        kernel.lanes_per_chain = g
        run_local_steps(kernel, target, x0, probe_steps, 1, 1, 0, pos, lp, acc, 0)   # warm
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for r in range(reps):
            run_local_steps(kernel, target, x0, probe_steps, 1, 1, r, pos, lp, acc, 0)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        if ms < best_ms:
            best, best_ms = g, ms
    kernel.lanes_per_chain = best
    _cache[key] = best
    return best


def tune_flow_gemm(model, n_rows: int = 65536, reps: int = 3) -> int:
    """Pick the BF16 flow's tensor-core tile shapes by measurement: the
    hidden-layer GEMM tile width (128 or 256 output columns, ``gemm_bn``)
    and the rows per tile of the fused spline and hidden GEMMs (128 rows on
    one CTA, or 256 rows on a CTA pair with tcgen05 cta_group::2 and half
    the weights per CTA, ``tile_rows``), then for one-CTA 256-column tiles
    the operand ring depth of the K >= 256 hidden GEMMs (``gemm_stages``: 4
    stages with one output staging buffer per epilogue warp, or 3 with two).
    Each candidate is timed on the forward (log_prob) and inverse (sample)
    passes over n_rows rows (the NF global step's chunk); no choice changes a
    result (every output's reduction over K is the same), only wave
    quantisation, operand traffic and the epilogue's share. Cached per model
    shape and row count; sets ``model.gemm_bn``, ``model.tile_rows`` and
    ``model.gemm_stages`` and returns the GEMM width."""
    if getattr(model, "precision", "float32") not in ("bf16", "bfloat16"):
        return 0
    key = ("flow_tiles", model.n_features, model.n_layers, tuple(model.hidden_size), model.num_bins, n_rows)
    if key in _cache:
        model.gemm_bn, model.tile_rows, model.gemm_stages = _cache[key]
        return model.gemm_bn
    x = torch.randn(n_rows, model.n_features, device=model.device)
    z = torch.randn(n_rows, model.n_features, device=model.device)
    best, best_ms = (0, 0), float("inf")
    timings = {}
    model.gemm_stages = 0
    for tile_rows in (256, 128):
        for bn in (256, 128):
            model.gemm_bn, model.tile_rows = bn, tile_rows
            ms = _time_passes(model, x, z, n_rows, reps)
            timings[f"tile_rows={tile_rows},gemm_bn={bn}"] = ms
            if ms < best_ms:
                best, best_ms = (bn, tile_rows), ms
    model.gemm_bn, model.tile_rows = best
    # operand ring depth of the K >= 256 hidden GEMMs (one-CTA tiles only):
    # four stages with one output staging buffer per warp, or three stages
    # with two and the bias in shared memory; same outputs either way
    model.gemm_stages = 0
    if model.tile_rows != 256 and model.gemm_bn == 256:
        stage_ms = {}
        for stages in (4, 3):
            model.gemm_stages = stages
            stage_ms[stages] = _time_passes(model, x, z, n_rows, reps)
            timings[f"tile_rows={model.tile_rows},gemm_bn={model.gemm_bn},gemm_stages={stages}"] = stage_ms[stages]
        model.gemm_stages = min(stage_ms, key=stage_ms.get)
    model.tile_timings_ms = timings
    _cache[key] = best + (model.gemm_stages,)
    return best[0]


def _time_passes(model, x, z, n_rows, reps):
    from .random import PRNGKey
    model.log_prob(x)   # warm
    model.sample(PRNGKey(0), n_rows, z=z)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        model.log_prob(x)
        model.sample(PRNGKey(0), n_rows, z=z)
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_flow_train(model, n_rows: int = 65536, reps: int = 3, candidates=(0, 2, 4, 8, 16)) -> int:
    """Pick the K (batch) slice count of the BF16 training's weight-gradient
    GEMMs by timing one loss + gradient of n_rows rows per candidate (0 =
    the library's choice, enough slices to fill the SMs). The slices' sums
    are added in a fixed order, so each choice is deterministic; they differ
    by float32 rounding. Cached per model shape and row count; sets
    ``model.wgrad_splits`` and ``model.train_timings_ms`` and returns the pick."""
    if getattr(model, "precision", "float32") not in ("bf16", "bfloat16"):
        return 0
    key = ("flow_wgrad", model.n_features, model.n_layers, tuple(model.hidden_size), model.num_bins, n_rows)
    if key in _cache:
        model.wgrad_splits = _cache[key]
        return model.wgrad_splits
    x = torch.randn(n_rows, model.n_features, device=model.device)
    loss = torch.empty((), device=model.device)
    grad = torch.empty(model.n_params, device=model.device)
    timings = {}
    for sl in candidates:
        model.wgrad_splits = sl
        model.loss_and_grad(x, loss, grad)   # warm (and grows the workspace)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            model.loss_and_grad(x, loss, grad)
        e1.record()
        e1.synchronize()
        timings[f"wgrad_splits={sl}"] = e0.elapsed_time(e1) / reps
    best = min(candidates, key=lambda sl: timings[f"wgrad_splits={sl}"])
    model.wgrad_splits = best
    model.train_timings_ms = timings
    _cache[key] = best
    return best
