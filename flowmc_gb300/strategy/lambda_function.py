"""Lambda strategy (mirrors strategy/lambda_function.py:6-37 of the reference)."""
from __future__ import annotations

from typing import Callable

from .base import Strategy


class Lambda(Strategy):
    """Apply a function to the resources; passes key and position through."""

    def __init__(self, lambda_function: Callable):
        self.lambda_function = lambda_function

    def __call__(self, rng_key, resources, initial_position, data):
        self.lambda_function(rng_key, resources, initial_position, data)
        return rng_key, resources, initial_position
