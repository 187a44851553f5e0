"""Strategy base class (mirrors strategy/base.py:8-31 of the reference)."""
from __future__ import annotations

from abc import ABC, abstractmethod


class Strategy(ABC):
    """A block of the sampling schedule: (rng_key, resources, position, data)
    -> (rng_key, resources, position)."""

    @abstractmethod
    def __init__(self):
        raise NotImplementedError

    @abstractmethod
    def __call__(self, rng_key, resources: dict, initial_position, data: dict):
        raise NotImplementedError
