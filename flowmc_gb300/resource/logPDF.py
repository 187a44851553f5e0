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
