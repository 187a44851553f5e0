"""Counter-based random keys replacing jax.random keys.

The reference threads JAX threefry keys through every call
(``jax.random.split``, e.g. strategy/take_steps.py:71-72). Here a key is a
64-bit integer: ``split`` derives new keys with the SplitMix64 finaliser
(Steele, Lea, Flood, "Fast splittable pseudorandom number generators",
OOPSLA 2014), and the kernels use the key as the Philox-4x32-10 seed with
the chain index and step in the counter. Key *streams* therefore differ
from JAX's; explicit-noise arguments exist for trajectory parity.
"""
from __future__ import annotations

import dataclasses

_MASK = (1 << 64) - 1


def _mix64(z: int) -> int:
    z = (z + 0x9E3779B97F4A7C15) & _MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
    return z ^ (z >> 31)


@dataclasses.dataclass(frozen=True)
class PRNGKey:
    """A random key (stand-in for jax.random.PRNGKey(seed))."""

    value: int

    def __init__(self, seed: int):
        object.__setattr__(self, "value", _mix64(int(seed) & _MASK))

    @classmethod
    def _raw(cls, v: int) -> "PRNGKey":
        k = cls.__new__(cls)
        object.__setattr__(k, "value", v & _MASK)
        return k

    @property
    def seed(self) -> int:
        return self.value


def split(key: PRNGKey, num: int = 2) -> list[PRNGKey]:
    """jax.random.split analogue: `num` independent child keys."""
    base = key.value
    return [PRNGKey._raw(_mix64(base ^ _mix64(i + 1))) for i in range(num)]


def fold_in(key: PRNGKey, data: int) -> PRNGKey:
    return PRNGKey._raw(_mix64(key.value ^ _mix64((int(data) + 0x632BE59BD9B4E019) & _MASK)))
