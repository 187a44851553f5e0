"""UpdateState strategy (mirrors strategy/update_state.py:7-47 of the reference)."""
from __future__ import annotations

from ..resource.states import State
from .base import Strategy


class UpdateState(Strategy):
    def __init__(self, state_name: str, keys: list, values: list):
        self.state_name = state_name
        self.keys = keys
        self.values = values

    def __call__(self, rng_key, resources, initial_position, data):
        state = resources[self.state_name]
        assert isinstance(state, State), f"Resource {self.state_name} is not a State resource."
        state.update(self.keys, self.values)
        return rng_key, resources, initial_position
