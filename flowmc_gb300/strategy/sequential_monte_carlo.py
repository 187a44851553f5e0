"""SequentialMonteCarlo (mirrors strategy/sequential_monte_carlo.py:5-20 of
the reference): declared there but not implemented. It subclasses Resource
without Resource's abstract methods, so constructing it raises TypeError
there and here; it is kept so that imports written against the reference
resolve."""
from __future__ import annotations

from ..resource.base import Resource


class SequentialMonteCarlo(Resource):
    def __init__(self):
        raise NotImplementedError

    def __call__(self, rng_key, resources: dict, initial_position, data: dict):
        raise NotImplementedError
