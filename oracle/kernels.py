"""Oracle local kernels, serial-step driver and NF global step (float64).

TEST INFRASTRUCTURE ONLY. Restates, with every random draw passed in:
  * MALA.kernel            resource/kernel/MALA.py:26-89
  * HMC.kernel / leapfrog  resource/kernel/HMC.py:38-151
  * GaussianRandomWalk     resource/kernel/Gaussian_random_walk.py:25-61
  * TakeSerialSteps        strategy/take_steps.py:60-180 (thinning, buffer rows)
  * NFProposal.kernel      resource/kernel/NF_proposal.py:27-128
Each kernel acts on a batch of chains at once (the reference vmaps a
single-chain kernel over chains, strategy/take_steps.py:126-132).
"""
from __future__ import annotations

import numpy as np

from . import targets as T


def _iso_normal_logpdf(a: np.ndarray, mean: np.ndarray, var: float) -> np.ndarray:
    """jax.scipy.stats.multivariate_normal.logpdf with scalar covariance."""
    d = a.shape[-1]
    r = a - mean
    return -0.5 * np.sum(r * r, axis=-1) / var - 0.5 * d * np.log(2.0 * np.pi * var)


def mala_kernel(t, x, dt, xi, u, return_ratio=False):
    """One MALA step for every chain (MALA.py:26-89).

    x [C, d], xi [C, d] standard normals (the key1 draw), u [C] uniforms
    (the key2 draw). Returns (x', lp', accept). The incoming log_prob is not
    used: the reference recomputes lp0 at x (MALA.py:59, 87-88).
    """
    dt2 = dt * dt
    lp0, g0 = T.value_grad(t, x)
    prop = x + dt2 * g0 / 2 + dt * xi                     # MALA.py:60-63
    lp1, g1 = T.value_grad(t, prop)                       # second scan iteration
    ratio = lp1 - lp0
    ratio = ratio - _iso_normal_logpdf(prop, x + dt2 * g0 / 2, dt2)   # MALA.py:76-78
    ratio = ratio + _iso_normal_logpdf(x, prop + dt2 * g1 / 2, dt2)   # MALA.py:79-81
    acc = np.log(u) < ratio                                # MALA.py:83-84
    x_new = np.where(acc[:, None], prop, x)
    lp_new = np.where(acc, lp1, lp0)
    return (x_new, lp_new, acc, ratio) if return_ratio else (x_new, lp_new, acc)


def leapfrog_coefs(n_leapfrog: int) -> np.ndarray:
    """HMC.py:47-50: rows [0, .5], [1, 1] * n_leapfrog, [1, .5]."""
    c = np.ones((n_leapfrog + 2, 2))
    c[0] = [0.0, 0.5]
    c[-1] = [1.0, 0.5]
    return c


def kinetic(p: np.ndarray, M: np.ndarray) -> np.ndarray:
    """HMC.py:118-121: 0.5 * (p**2 * metric).sum() with numpy broadcasting
    (for a matrix metric this sums p_j^2 M[i, j] over i and j)."""
    M = np.asarray(M, np.float64)
    if M.ndim == 2:
        return 0.5 * np.sum(p * p * M.sum(axis=0), axis=-1)
    return 0.5 * np.sum(p * p * M, axis=-1)


def grad_kinetic(p: np.ndarray, M: np.ndarray) -> np.ndarray:
    M = np.asarray(M, np.float64)
    return p * (M.sum(axis=0) if M.ndim == 2 else M)


def leapfrog(t, x, p, eps, n_leapfrog, M):
    """HMC.leapfrog_step (HMC.py:71-96): scan over the coefficient table."""
    coefs = leapfrog_coefs(n_leapfrog)
    for c0, c1 in coefs:
        x = x + eps * c0 * grad_kinetic(p, M)
        _, g = T.value_grad(t, x)
        p = p - eps * c1 * (-g)
    return x, p


def hmc_kernel(t, x, lp, eps, n_leapfrog, M, xi, u, return_ratio=False):
    """One HMC step (HMC.py:98-151); H uses the incoming log_prob (HMC.py:137)."""
    M = np.asarray(M, np.float64)
    Mm = M if M.ndim == 2 else np.diag(M)
    L = np.linalg.cholesky(np.linalg.inv(Mm))
    p = xi @ L.T                                          # HMC.py:133-136
    H = -lp + kinetic(p, M)
    xq, pq = leapfrog(t, x, p, eps, n_leapfrog, M)
    lpq = T.value(t, xq)
    Hq = -lpq + kinetic(pq, M)
    acc = np.log(u) < H - Hq                              # HMC.py:141-145
    out = (np.where(acc[:, None], xq, x), np.where(acc, lpq, lp), acc)
    return out + (H - Hq,) if return_ratio else out


def grw_kernel(t, x, lp, sigma, xi, u, return_ratio=False):
    """Gaussian_random_walk.py:48-61."""
    prop = x + xi * sigma
    lpp = T.value(t, prop)
    acc = np.log(u) < lpp - lp
    out = (np.where(acc[:, None], prop, x), np.where(acc, lpp, lp), acc)
    return out + (lpp - lp,) if return_ratio else out


def accept_margins(kind, t, x0, noise, unif, *, step_size, n_leapfrog=10, M=None):
    """Per chain and step, |log u - log ratio| / (1 + |log ratio|) along the
    oracle trajectory: small values mark near-ties, where a float32 kernel
    may legitimately decide the other way."""
    x = np.asarray(x0, np.float64)
    lp = T.value(t, x)
    C, d = x.shape
    M = np.eye(d) if M is None else M
    S = noise.shape[1]
    out = np.zeros((C, S))
    for s in range(S):
        xi, u = np.asarray(noise[:, s], np.float64), np.asarray(unif[:, s], np.float64)
        if kind == "mala":
            x, lp, _, r = mala_kernel(t, x, step_size, xi, u, return_ratio=True)
        elif kind == "hmc":
            x, lp, _, r = hmc_kernel(t, x, lp, step_size, n_leapfrog, M, xi, u, return_ratio=True)
        else:
            x, lp, _, r = grw_kernel(t, x, lp, step_size, xi, u, return_ratio=True)
        out[:, s] = np.abs(np.log(u) - r) / (1.0 + np.abs(r))
    return out


def take_serial_steps(kind, t, x0, n_steps, noise, unif, *, step_size, n_leapfrog=10, M=None,
                      thinning=1):
    """TakeSerialSteps.sample + the thinning of TakeSteps.__call__.

    noise [C, n_steps, d], unif [C, n_steps]. Returns
    (positions [C, R, d], log_probs [C, R], accepts [C, R], last_position [C, d])
    with R = ceil(n_steps / thinning) (take_steps.py:134-144).
    """
    x = np.asarray(x0, np.float64)
    lp = T.value(t, x)                                    # take_steps.py:177
    C, d = x.shape
    if M is None:
        M = np.eye(d)
    pos, lps, accs = [], [], []
    for s in range(n_steps):
        xi = np.asarray(noise[:, s], np.float64)
        u = np.asarray(unif[:, s], np.float64)
        if kind == "mala":
            x, lp, acc = mala_kernel(t, x, step_size, xi, u)
        elif kind == "hmc":
            x, lp, acc = hmc_kernel(t, x, lp, step_size, n_leapfrog, M, xi, u)
        elif kind == "grw":
            x, lp, acc = grw_kernel(t, x, lp, step_size, xi, u)
        else:
            raise ValueError(kind)
        pos.append(x)
        lps.append(lp)
        accs.append(acc)
    pos = np.stack(pos, 1)[:, ::thinning]
    lps = np.stack(lps, 1)[:, ::thinning]
    accs = np.stack(accs, 1)[:, ::thinning].astype(np.float64)
    return pos, lps, accs, pos[:, -1]


def buffer_update(buf: np.ndarray, upd: np.ndarray, start: int, axis: int) -> np.ndarray:
    """jax.lax.dynamic_update_slice_in_dim (buffers.py:39-41): the start index
    is clamped so the update fits."""
    n = upd.shape[axis]
    size = buf.shape[axis]
    if n > size:
        raise ValueError("update larger than buffer")
    s = min(max(int(start), 0), size - n)
    out = buf.copy()
    idx = [slice(None)] * buf.ndim
    idx[axis] = slice(s, s + n)
    out[tuple(idx)] = upd
    return out


def nf_proposal_kernel(flow, t, x, z, u, return_ratio=False):
    """NFProposal.kernel for every chain (NF_proposal.py:27-128).

    flow: an ``oracle.flow.Flow``; x [C, d] current positions; z [C, S, d]
    the base-distribution normals of the proposals; u [C, S] the MH
    uniforms. log_prob of the proposals is recomputed by the forward pass
    (NF_proposal.py:165-167), and the incoming log_prob is logpdf(x)
    (take_steps.py:200-206). With return_ratio the log acceptance ratio of
    every step [C, S] is returned as well (for tie margins in tests).
    """
    C, S, d = z.shape
    lp = T.value(t, x)
    lnf = flow.log_prob(x)                                # NF_proposal.py:44
    props = flow.sample(z.reshape(C * S, d))              # NF_proposal.py:165
    lnf_p = flow.log_prob(props).reshape(C, S)            # NF_proposal.py:166
    props = props.reshape(C, S, d)
    lp_p = T.value(t, props.reshape(C * S, d)).reshape(C, S)   # NF_proposal.py:86-89
    out_x = np.empty((C, S, d))
    out_lp = np.empty((C, S))
    out_acc = np.empty((C, S))
    out_ratio = np.empty((C, S))
    for s in range(S):                                    # NF_proposal.py:91-126
        ratio = (lp_p[:, s] - lp) - (lnf_p[:, s] - lnf)
        out_ratio[:, s] = ratio
        acc = np.log(u[:, s]) < ratio
        x = np.where(acc[:, None], props[:, s], x)
        lp = np.where(acc, lp_p[:, s], lp)
        lnf = np.where(acc, lnf_p[:, s], lnf)
        out_x[:, s], out_lp[:, s], out_acc[:, s] = x, lp, acc
    return (out_x, out_lp, out_acc, out_ratio) if return_ratio else (out_x, out_lp, out_acc)
