"""LogPDF resource (mirrors resource/logPDF.py:20-81 of the reference).

The wrapped log-density must be a registered device target
(``flowmc_gb300.targets``); its value and gradient run inside the fused
kernels. A plain Python callable is rejected when a kernel needs it,
because the GPU path cannot call back into Python and there is no CPU
fallback.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional

from .base import Resource
from ..targets import Target


@dataclass
class Variable:
    name: str
    continuous: bool


class LogPDF(Resource):
    log_pdf: Callable
    variables: list

    @property
    def n_dims(self):
        return len(self.variables)

    def __repr__(self):
        return "LogPDF with " + str(self.n_dims) + " dimensions"

    def __init__(self, log_pdf, variables: Optional[list] = None, n_dims: Optional[int] = None):
        self.log_pdf = log_pdf
        if variables is None and n_dims is not None:
            self.variables = [Variable("x_" + str(i), True) for i in range(n_dims)]
        elif variables is not None:
            self.variables = variables
        else:
            raise ValueError("Either variables or n_dims must be provided")

    @property
    def target(self) -> Target:
        """The device target the fused kernels evaluate."""
        t = self.log_pdf
        if isinstance(t, LogPDF):
            return t.target
        if not isinstance(t, Target):
            raise TypeError(
                "flowmc_gb300 kernels evaluate registered device targets "
                "(flowmc_gb300.targets.*); got a plain callable, which the fused GPU path cannot run")
        return t

    def __call__(self, x, data=None):
        return self.log_pdf(x, data)

    def print_parameters(self):
        print("LogPDF with variables:")
        for var in self.variables:
            print(var.name, var.continuous)

    def save_resource(self, path):
        raise NotImplementedError

    def load_resource(self, path):
        raise NotImplementedError


def as_target(logpdf) -> Target:
    """Target behind a LogPDF or a bare Target."""
    if isinstance(logpdf, LogPDF):
        return logpdf.target
    if isinstance(logpdf, Target):
        return logpdf
    raise TypeError("expected a LogPDF wrapping a flowmc_gb300 target, or a target")


class TemperedPDF(LogPDF):
    """TemperedPDF (mirrors resource/logPDF.py:84-115 of the reference):
    ``tempered_log_pdf(T, x) = (1 / T) * log_likelihood(x) + log_prior(x)``,
    evaluated inside the fused tempered local-step kernel.

    ``log_likelihood`` is a registered device target (or a LogPDF wrapping
    one). ``log_prior`` is None, the reference bundle's zero prior
    (``lambda x, _: 0.0`` -- recognised by returning exactly 0.0 on a zero
    vector without touching a GPU), or a ``targets.DiagGaussian``; other
    priors cannot run inside the fused kernel and are refused.
    ``__call__`` is the untempered likelihood, as in the reference (the
    exchange step compares those values, parallel_tempering.py:386).
    """

    def __init__(self, log_likelihood, log_prior=None, variables=None, n_dims=None, n_temps=5, max_temp=100):
        super().__init__(log_likelihood, variables, n_dims)
        self.log_prior = log_prior
        self.n_temps = n_temps
        self.max_temp = max_temp
        self._prior = _prior_arrays(log_prior, self.n_dims)

    def tempered_log_pdf(self, temperatures, x, data=None):
        """(1 / T) * log L(x) + log prior(x) for a batch x [n, d] and per-row T."""
        import torch
        lp = self.target(x, data)
        t = torch.as_tensor(temperatures, dtype=torch.float32, device=lp.device)
        out = (1.0 / t) * lp
        if self._prior is not None:
            m, iv, c = self._prior
            xx = x.reshape(-1, self.n_dims)
            out = out - 0.5 * (((xx - m.to(xx.device)) ** 2) * iv.to(xx.device)).sum(-1).reshape(out.shape) + c
        return out

    def prior_arrays(self, device):
        """(mean, inv_var, const) of the diagonal Gaussian prior on `device`, or None."""
        if self._prior is None:
            return None
        m, iv, c = self._prior
        return m.to(device), iv.to(device), c


def _prior_arrays(prior, n_dims):
    import numpy as np
    import torch
    from ..targets import DiagGaussian
    if prior is None:
        return None
    if isinstance(prior, DiagGaussian):
        if prior.n_dim != n_dims:
            raise ValueError(f"prior has {prior.n_dim} coordinates, likelihood has {n_dims}")
        m = torch.as_tensor(np.asarray(prior.mean, np.float32))
        iv = torch.as_tensor(np.asarray(prior.inv_var, np.float32))
        return m, iv, float(prior.const)
    if callable(prior) and not isinstance(prior, Target):
        rng = np.random.default_rng(0)
        probes = [np.zeros(n_dims), rng.normal(size=n_dims), 1e3 * rng.normal(size=n_dims)]
        def zero(v):
            # a Python number or a one-element array (the tutorials return jnp.array(0.0))
            try:
                a = np.asarray(v.detach().cpu() if hasattr(v, "detach") else v, dtype=np.float64)
            except Exception:
                return False
            return a.size == 1 and float(a.reshape(())) == 0.0

        try:
            vals = [prior(p, {}) for p in probes]
        except Exception:
            vals = [None]
        if all(zero(v) for v in vals):
            return None
    raise NotImplementedError(
        "the fused tempered kernel supports a zero log prior or a targets.DiagGaussian prior; "
        f"got {type(prior).__name__}")
