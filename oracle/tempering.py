"""Oracle parallel tempering (float64) -- TEST INFRASTRUCTURE ONLY.

Restates, with every random draw passed in:
  * ParallelTempering._ensemble_step / _individal_step
                        strategy/parallel_tempering.py:205-289
  * ParallelTempering._exchange / _exchange_step_body
                        strategy/parallel_tempering.py:291-398
  * ParallelTempering._adapt_temperature
                        strategy/parallel_tempering.py:400-436
  * ParallelTempering.__call__   strategy/parallel_tempering.py:47-133
on TemperedPDF.tempered_log_pdf (resource/logPDF.py:106-108).
Positions are [n_chains, n_temps, n_dim] as in the reference.
"""
from __future__ import annotations

import numpy as np

from . import kernels as K
from . import targets as T


def tempered(t: dict, temps, n_chains: int, prior=None) -> dict:
    """The tempered target over the n_chains * n_temps rows (row c * n_temps + t)."""
    temps = np.asarray(temps, np.float64)
    beta = np.tile(1.0 / temps, n_chains)
    return {"kind": "tempered", "base": t, "beta": beta, "prior": prior}


def ensemble_step(kind, t, x, temps, n_steps, noise, unif, *, step_size, n_leapfrog=10, M=None, prior=None):
    """n_steps of the local kernel on every (chain, temperature) row.

    x [C, T, d]; noise [C, T, n_steps, d]; unif [C, T, n_steps]. Returns the
    last positions [C, T, d], their tempered log-densities [C, T] and the
    per-step accept flags [C, T, n_steps] (parallel_tempering.py:236-248).
    """
    C, Tn, d = x.shape
    tt = tempered(t, temps, C, prior)
    pos, lps, accs, last = K.take_serial_steps(
        kind, tt, x.reshape(C * Tn, d), n_steps, noise.reshape(C * Tn, n_steps, d), unif.reshape(C * Tn, n_steps),
        step_size=step_size, n_leapfrog=n_leapfrog, M=M)
    return last.reshape(C, Tn, d), lps[:, -1].reshape(C, Tn), accs.reshape(C, Tn, n_steps)


def exchange(t, x, temps, u):
    """Sequential adjacent swaps for every chain (parallel_tempering.py:291-398).

    x [C, T, d]; u [C, T-1] uniforms. Returns positions [C, T, d], the
    untempered log-densities after the sweep [C, T] and the flags [C, T-1].
    """
    x = np.array(x, np.float64)
    C, Tn, d = x.shape
    temps = np.asarray(temps, np.float64)
    lp = T.value(t, x.reshape(C * Tn, d)).reshape(C, Tn)    # parallel_tempering.py:386
    acc = np.zeros((C, max(Tn - 1, 0)), bool)
    for i in range(Tn - 1):                                  # scan over idx
        ratio = (1.0 / temps[i + 1] - 1.0 / temps[i]) * (lp[:, i] - lp[:, i + 1])
        a = np.log(u[:, i]) < ratio
        acc[:, i] = a
        xi, xj = x[a, i].copy(), x[a, i + 1].copy()
        x[a, i], x[a, i + 1] = xj, xi
        li, lj = lp[a, i].copy(), lp[a, i + 1].copy()
        lp[a, i], lp[a, i + 1] = lj, li
    return x, lp, acc


def adapt_temperature(temps, do_accept):
    """parallel_tempering.py:400-436; do_accept [C, T-1]."""
    temps = np.asarray(temps, np.float64)
    do_accept = np.asarray(do_accept, np.float64)
    rate = do_accept.mean(axis=0)
    damping = (100.0 / do_accept.shape[0]) * (rate[:-1] - rate[1:])
    new = temps.copy()
    for i in range(1, len(temps) - 1):
        new[i] = new[i - 1] + (temps[i] - temps[i - 1]) * np.exp(damping[i - 1])
    return new


def parallel_tempering(kind, t, x_first, x_tempered, temps, n_steps, noise, unif, u_exchange, *, step_size,
                       training=True, n_leapfrog=10, M=None, prior=None):
    """ParallelTempering.__call__ (parallel_tempering.py:47-133).

    Returns (chain positions [C, d], new tempered positions [C, T-1, d] (the
    input when not training), new temperatures [T] (the input when not
    training)).
    """
    x = np.concatenate([np.asarray(x_first, np.float64)[:, None], np.asarray(x_tempered, np.float64)], axis=1)
    x, _, _ = ensemble_step(kind, t, x, temps, n_steps, noise, unif, step_size=step_size,
                            n_leapfrog=n_leapfrog, M=M, prior=prior)
    x, _, acc = exchange(t, x, temps, u_exchange)
    if training:
        return x[:, 0], x[:, 1:], adapt_temperature(temps, acc)
    return x[:, 0], np.asarray(x_tempered, np.float64), np.asarray(temps, np.float64)
