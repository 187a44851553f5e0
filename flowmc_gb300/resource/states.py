"""State resource (mirrors resource/states.py:11-63 of the reference)."""
from __future__ import annotations

import numpy as np

from .base import Resource


class State(Resource):
    """A dict of names and flags that strategies use to find their buffers."""

    name: str
    data: dict

    def __repr__(self):
        return "State " + self.name + " with shape " + str(len(self.data))

    def __init__(self, data: dict, name: str = "State"):
        self.name = name
        self.data = data

    def update(self, key: list, value: list):
        for k, v in zip(key, value):
            self.data[k] = v
            print(f"Updated state {k} to {v}")

    def print_parameters(self):
        print(f"State: {self.name} with shape {len(self.data)} and data {self.data}")

    def save_resource(self, path: str):
        np.savez(path + self.name, name=self.name, data=np.array(self.data, dtype=object))

    def load_resource(self, path: str) -> "State":
        d = np.load(path, allow_pickle=True)
        return State(d["data"].item(), str(d["name"]))
