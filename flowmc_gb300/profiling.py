"""CUDA-event timing of the sampler's phases.

Strategies wrap their fused launches in ``region(name)``; when a Profiler is
active the region records a start/stop event pair on the launching stream
(as event-record nodes when the stream is being captured into a CUDA
graph, so that a replay times the same regions), otherwise it costs
nothing. ``Profiler.totals_ms()`` synchronises once at
the end and sums the device time per region.
"""
from __future__ import annotations

import contextlib

import torch

_active = None


class Profiler:
    def __init__(self):
        self.events: dict[str, list] = {}
        self.units: dict[str, float] = {}

    def __enter__(self):
        global _active
        self._prev = _active
        _active = self
        return self

    def __exit__(self, *exc):
        global _active
        _active = self._prev

    def totals_ms(self) -> dict:
        torch.cuda.synchronize()
        return {k: sum(a.elapsed_time(b) for a, b in v) for k, v in self.events.items()}

    def counts(self) -> dict:
        return {k: len(v) for k, v in self.events.items()}


@contextlib.contextmanager
def region(name: str, units: float = 0.0):
    p = _active
    if p is None:
        yield
        return
    kw = {"enable_timing": True}
    if torch.cuda.is_current_stream_capturing():
        kw["external"] = True       # event-record nodes of the captured graph
    a = torch.cuda.Event(**kw)
    b = torch.cuda.Event(**kw)
    a.record()
    try:
        yield
    finally:
        b.record()
        p.events.setdefault(name, []).append((a, b))
        p.units[name] = p.units.get(name, 0.0) + units
