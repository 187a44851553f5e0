"""Sampling diagnostics: rank-normalised bulk ESS and moment errors.

ESS follows Vehtari, Gelman, Simpson, Carpenter & Buerkner, "Rank-
normalization, folding, and localization: an improved R-hat" (Bayesian
Analysis, 2021): split chains, rank-normalise the pooled draws with Blom's
offset, then the multi-chain autocorrelation estimate truncated by Geyer's
initial monotone sequence (Geyer, Statistical Science, 1992). The reference
has no ESS code (its tutorials call arviz); this is the project's own, in
float64 torch on the GPU. It is a diagnostic, run after sampling.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def _normal_ppf(p: torch.Tensor) -> torch.Tensor:
    return math.sqrt(2.0) * torch.erfinv(2.0 * p - 1.0)


def _ess_from_chains(z: torch.Tensor) -> torch.Tensor:
    """z [m, n, k] (m chains, n draws, k independent series) -> ESS [k]."""
    m, n, k = z.shape
    zc = z - z.mean(dim=1, keepdim=True)
    nfft = 1 << (2 * n - 1).bit_length()
    f = torch.fft.rfft(zc, n=nfft, dim=1)
    acov = torch.fft.irfft(f * f.conj(), n=nfft, dim=1)[:, :n] / n          # biased autocovariance
    chain_var = acov[:, 0] * n / (n - 1)                                    # [m, k]
    W = chain_var.mean(0)
    means = z.mean(dim=1)
    B_over_n = means.var(dim=0, unbiased=True) if m > 1 else torch.zeros_like(W)
    var_plus = (n - 1) / n * W + B_over_n
    mean_acov = acov.mean(0)                                                # [n, k]
    rho = 1.0 - (W - mean_acov) / var_plus                                  # rho_0 ~ 1
    rho[0] = 1.0
    n_pairs = n // 2
    P = rho[: 2 * n_pairs].reshape(n_pairs, 2, k).sum(1)                    # Geyer pairs
    pos = P > 0
    # initial positive sequence: stop at the first non-positive pair
    first_bad = torch.where(pos.all(0), torch.full((k,), n_pairs, device=z.device),
                            (~pos).float().argmax(0))
    idx = torch.arange(n_pairs, device=z.device)[:, None]
    P = torch.where(idx < first_bad[None], P, torch.zeros_like(P))
    # initial monotone sequence
    P = torch.cummin(P, dim=0).values
    tau = -1.0 + 2.0 * P.sum(0)
    tau = torch.clamp(tau, min=1.0 / math.log10(max(m * n, 10)))
    return m * n / tau


def ess_bulk(draws: torch.Tensor, dims_per_batch: int = 4) -> torch.Tensor:
    """Bulk ESS per coordinate of draws [n_chains, n_draws, n_dim] -> [n_dim] (float64)."""
    C, S, d = draws.shape
    half = S // 2
    out = torch.empty(d, dtype=torch.float64, device=draws.device)
    for j0 in range(0, d, dims_per_batch):
        j1 = min(d, j0 + dims_per_batch)
        x = draws[:, :2 * half, j0:j1].to(torch.float64)
        # split chains
        x = torch.cat([x[:, :half], x[:, half:]], 0)                          # [2C, half, k]
        m, n, k = x.shape
        flat = x.permute(2, 0, 1).reshape(k, -1)
        r = torch.empty_like(flat)
        order = torch.argsort(flat, dim=1)
        ranks = torch.arange(1, flat.shape[1] + 1, dtype=torch.float64, device=draws.device).expand(k, -1)
        r.scatter_(1, order, ranks)
        z = _normal_ppf((r - 0.375) / (flat.shape[1] + 0.25))
        z = z.reshape(k, m, n).permute(1, 2, 0)
        out[j0:j1] = _ess_from_chains(z)
    return out


def moments(draws: torch.Tensor):
    """(mean [d], variance [d]) over chains and draws, float64."""
    x = draws.reshape(-1, draws.shape[-1]).to(torch.float64)
    return x.mean(0), x.var(0, unbiased=True)


def moment_error(draws: torch.Tensor, mean_ref, var_ref) -> float:
    """max_j max(|mu_j - m_j| / sigma_j, |s2_j / sigma2_j - 1|)."""
    mu, var = moments(draws)
    return moment_error_of(mu, var, mean_ref, var_ref)


def moment_error_of(mu: torch.Tensor, var: torch.Tensor, mean_ref, var_ref) -> float:
    """The moment error of given per-coordinate means and variances."""
    mr = torch.as_tensor(np.asarray(mean_ref), dtype=torch.float64, device=mu.device)
    vr = torch.as_tensor(np.asarray(var_ref), dtype=torch.float64, device=mu.device)
    e1 = (mu - mr).abs() / vr.sqrt()
    e2 = (var / vr - 1.0).abs()
    return float(torch.maximum(e1, e2).max())


def rosenbrock_chain_moments(d: int, a: float = 20.0, b: float = 1.0, c: float = 5.0, lo: float = -8.0,
                             hi: float = 24.0, m: int = 6000):
    """Exact (quadrature) per-coordinate mean and variance of
    p(x) ~ exp(-sum_{i<d-1} [(b - x_i)^2 / a + c (x_{i+1} - x_i^2)^2]).

    The density is a chain: unary exp(-(b - x_i)^2 / a) for i < d-1 and
    pairwise exp(-c (x_{i+1} - x_i^2)^2). The last coordinate has no unary
    term, so x_{d-1} | x_{d-2} ~ N(x_{d-2}^2, 1/(2c)) integrates out in closed
    form; the others get their marginals from forward/backward messages on a
    uniform grid (float64 numpy). Returns (mean [d], var [d])."""
    n = d - 1                      # coordinates handled on the grid
    x = np.linspace(lo, hi, m)
    dx = x[1] - x[0]
    unary = np.exp(-(b - x) ** 2 / a)
    psi = np.exp(-c * (x[None, :] - (x ** 2)[:, None]) ** 2)   # psi[x_i, x_{i+1}]
    fwd = np.empty((n, m))
    bwd = np.empty((n, m))
    fwd[0] = unary / unary.sum()
    for i in range(1, n):
        v = (fwd[i - 1] @ psi) * dx * unary
        fwd[i] = v / v.sum()
    bwd[n - 1] = 1.0
    for i in range(n - 2, -1, -1):
        v = psi @ (unary * bwd[i + 1]) * dx
        bwd[i] = v / v.sum()
    mean = np.empty(d)
    var = np.empty(d)
    edge = 0.0
    for i in range(n):
        p = fwd[i] * bwd[i]
        p /= p.sum()
        mean[i] = (p * x).sum()
        var[i] = (p * (x - mean[i]) ** 2).sum()
        edge = max(edge, p[:20].sum() + p[-20:].sum())
        if i == n - 1:
            m2 = (p * x ** 2).sum()
            m4 = (p * x ** 4).sum()
            mean[d - 1] = m2
            var[d - 1] = m4 - m2 * m2 + 1.0 / (2.0 * c)
    if edge > 1e-9:
        raise RuntimeError(f"quadrature grid too narrow (edge mass {edge:.2e})")
    return mean, var


def dual_moon_moments(d: int, r0: float = 2.0, sr: float = 0.1, mu: float = 3.0, s0: float = 0.6,
                      m_r: int = 2000, m_phi: int = 4000):
    """Exact (quadrature) per-coordinate mean and variance of
    p(x) ~ exp(-0.5((|x| - r0)/sr)^2) (exp(-0.5((x0 + mu)/s0)^2) + exp(-0.5((x0 - mu)/s0)^2)).

    The density depends on x only through r = |x| and the angle phi between x
    and the first axis, so in hyperspherical coordinates (volume element
    r^(d-1) sin(phi)^(d-2) dr dphi) it is a 2-D integral. The mixture in x0 is
    symmetric, so every mean is 0; var(x0) = E[r^2 cos^2 phi] and the other
    d - 1 coordinates share E[r^2 sin^2 phi] / (d - 1). Midpoint rule on a
    uniform (r, phi) grid in float64. Returns (mean [d], var [d])."""
    if d < 2:
        raise ValueError("dual_moon_moments needs d >= 2")
    lo, hi = max(0.0, r0 - 12.0 * sr), r0 + 12.0 * sr
    r = lo + (np.arange(m_r) + 0.5) * (hi - lo) / m_r
    phi = (np.arange(m_phi) + 0.5) * np.pi / m_phi
    R, F = np.meshgrid(r, phi, indexing="ij")
    x0 = R * np.cos(F)
    logw = (-0.5 * ((R - r0) / sr) ** 2 + (d - 1) * np.log(R) + (d - 2) * np.log(np.sin(F))
            + np.logaddexp(-0.5 * ((x0 + mu) / s0) ** 2, -0.5 * ((x0 - mu) / s0) ** 2))
    w = np.exp(logw - logw.max())
    w /= w.sum()
    mean = np.zeros(d)
    var = np.empty(d)
    var[0] = (w * x0 ** 2).sum()
    var[1:] = (w * (R * np.sin(F)) ** 2).sum() / (d - 1)
    return mean, var


class StreamingMoments:
    """FP64 moments, R-hat and batch-means ESS of chain rows accumulated on the
    device while the sampler runs (fmc_welford_ess_update / _finalize): per
    chain and coordinate Welford's running mean and squared deviations, and
    Welford over completed batch means of ``batch`` draws. ``update`` folds in
    rows [start, start + n_steps) of a chain buffer [n_chains, n, n_dim]; the
    draw count lives in the device state, so updates can be captured in a
    CUDA graph and replayed. ``finalize`` returns float64 tensors per
    coordinate: mean, var (of all draws), ess (multi-chain batch means;
    NaN before two complete batches) and rhat."""

    def __init__(self, n_chains: int, n_dim: int, batch: int, device=None):
        import ctypes
        from . import _lib
        self.n_chains, self.n_dim, self.batch = int(n_chains), int(n_dim), int(batch)
        nb = ctypes.c_size_t()
        _lib.check(_lib.lib().fmc_welford_state_size(self.n_chains, self.n_dim, ctypes.byref(nb)))
        dev = torch.device("cuda") if device is None else torch.device(device)
        self.state = torch.zeros(nb.value // 8, dtype=torch.float64, device=dev)
        self._out = torch.empty(4, self.n_dim, dtype=torch.float64, device=dev)
        self.reset()

    def reset(self):
        from . import _lib
        _lib.check(_lib.lib().fmc_welford_reset(self.state.data_ptr(), self.n_chains, self.n_dim, self.batch,
                                                _lib.stream_handle(self.state.device)))

    def update(self, buf: torch.Tensor, start: int, n_steps: int):
        from . import _lib
        _lib.require_cuda_f32(buf, "chain buffer", (self.n_chains, buf.shape[1], self.n_dim))
        _lib.check(_lib.lib().fmc_welford_ess_update(buf.data_ptr(), self.n_chains, buf.shape[1], self.n_dim,
                                                     int(start), int(n_steps), self.state.data_ptr(),
                                                     _lib.stream_handle(buf.device)))

    def finalize(self) -> dict:
        from . import _lib
        o = self._out
        _lib.check(_lib.lib().fmc_welford_ess_finalize(self.state.data_ptr(), self.n_chains, self.n_dim,
                                                       o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(),
                                                       o[3].data_ptr(), _lib.stream_handle(o.device)))
        return {"mean": o[0].clone(), "var": o[1].clone(), "ess": o[2].clone(), "rhat": o[3].clone()}

    def draws(self) -> int:
        """Draws per chain accumulated so far (synchronises)."""
        return int(self.state[:1].view(torch.int64).item())
