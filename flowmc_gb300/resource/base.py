"""Resource base class (mirrors resource/base.py:6-38 of the reference)."""
from __future__ import annotations

from abc import ABC, abstractmethod


class Resource(ABC):
    """Base class for resources: buffers, states, kernels, models, optimisers."""

    @abstractmethod
    def __init__(self):
        raise NotImplementedError

    @abstractmethod
    def print_parameters(self):
        raise NotImplementedError

    @abstractmethod
    def save_resource(self, path: str):
        raise NotImplementedError

    @abstractmethod
    def load_resource(self, path: str):
        raise NotImplementedError
