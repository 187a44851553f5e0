"""CUDA-event timing of the sampler's phases, and NVTX ranges.

Strategies wrap their fused launches in ``region(name)``; when a Profiler is
active the region records a start/stop event pair on the launching stream
(as event-record nodes when the stream is being captured into a CUDA
graph, so that a replay times the same regions), otherwise it costs
nothing. ``Profiler.totals_ms()`` synchronises once at
the end and sums the device time per region.

With ``set_nvtx(True)`` (or FLOWMC_NVTX=1 in the environment) every region
and every strategy call of ``Sampler`` is also an NVTX range, so a timeline
profiler shows the schedule by name; off by default.
"""
from __future__ import annotations

import contextlib
import os

import torch

_active = None
_nvtx = os.environ.get("FLOWMC_NVTX", "") not in ("", "0")


def set_nvtx(enabled: bool) -> None:
    global _nvtx
    _nvtx = bool(enabled)


@contextlib.contextmanager
def nvtx_range(name: str):
    if not _nvtx:
        yield
        return
    torch.cuda.nvtx.range_push(name)
    try:
        yield
    finally:
        torch.cuda.nvtx.range_pop()


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
    if _nvtx:
        with nvtx_range(name), _timed(name, units):
            yield
        return
    with _timed(name, units):
        yield


@contextlib.contextmanager
def _timed(name: str, units: float):
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
