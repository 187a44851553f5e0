"""Sampler (mirrors Sampler.py:10-118 of the reference): the top-level driver
that runs the strategies in order, threading (rng_key, resources, position)."""
from __future__ import annotations

import torch

from .profiling import nvtx_range


class Sampler:
    n_dim: int
    n_chains: int
    rng_key: object
    resources: dict
    strategies: dict
    strategy_order: list | None

    verbose: bool = False
    logging: bool = True
    outdir: str = "./outdir/"

    def __init__(self, n_dim: int, n_chains: int, rng_key, resources=None, strategies=None, strategy_order=None,
                 resource_strategy_bundles=None, **kwargs):
        self.n_dim = n_dim
        self.n_chains = n_chains
        self.rng_key = rng_key
        if resources is not None and strategies is not None:
            print("Resources and strategies provided. Ignoring resource strategy bundles.")
            self.resources = resources
            self.strategies = strategies
            self.strategy_order = strategy_order
        else:
            print("Resources or strategies not provided. Using resource strategy bundles.")
            if resource_strategy_bundles is None:
                raise ValueError("Resource strategy bundles not provided."
                                 "Please provide either resources and strategies or resource strategy bundles.")
            self.resources = resource_strategy_bundles.resources
            self.strategies = resource_strategy_bundles.strategies
            self.strategy_order = resource_strategy_bundles.strategy_order
        class_keys = list(self.__class__.__dict__.keys())
        for key, value in kwargs.items():
            if key in class_keys and not key.startswith("__"):
                setattr(self, key, value)

    def _device(self):
        if "model" in self.resources:
            return self.resources["model"].device
        return torch.device("cuda") if torch.cuda.is_available() else None

    def _run(self, rng_key, x, data, order):
        for strategy in order:
            if strategy not in self.strategies:
                raise ValueError(f"Invalid strategy name '{strategy}' provided. "
                                 f"Available strategies are: {list(self.strategies.keys())}.")
            with nvtx_range(strategy):
                rng_key, self.resources, x = self.strategies[strategy](rng_key, self.resources, x, data)
        return rng_key, x

    def sample(self, initial_position, data: dict, cuda_graph: bool = False):
        """Run every strategy in strategy_order (Sampler.py:84-108).

        With ``cuda_graph=True`` the schedule runs as a CUDA graph: captured
        on the first call for this strategy_order (``capture``), then
        replayed. A replay re-executes exactly the captured launches --
        including the buffer rows they write -- with fresh random streams
        (the library's epoch word advances at the start of every replay);
        host-side strategy state (stepper cursors, sampler state) is not
        advanced by replays."""
        dev = self._device()
        x = torch.as_tensor(initial_position, dtype=torch.float32)
        if dev is not None:
            x = x.to(dev, non_blocking=True)
        initial_position = torch.atleast_2d(x)
        assert isinstance(self.strategy_order, list)
        if cuda_graph:
            cap = self._captured.get(tuple(self.strategy_order)) if hasattr(self, "_captured") else None
            if cap is None:
                cap = self.capture(initial_position, data)
            return cap.replay(initial_position)
        _, last_step = self._run(self.rng_key, initial_position, data, self.strategy_order)
        self.poll_errors()
        return last_step

    def _pollers(self):
        return [s for s in self.strategies.values() if hasattr(s, "poll_errors")]

    def poll_errors(self):
        """Raise the first error a strategy's device-side check recorded (a
        training-data selection whose finite rows do not split evenly over
        the chains). Waits only for the events recorded after those checks."""
        for s in self._pollers():
            s.poll_errors()

    def capture(self, initial_position, data: dict) -> "CapturedSchedule":
        """Capture strategy_order as one CUDA graph without running it. Work
        that cannot be captured (the autotuner's probes) runs first; the
        capture itself advances host-side strategy state once, as one eager
        run would."""
        from . import _lib
        dev = self._device()
        x0 = torch.atleast_2d(torch.as_tensor(initial_position, dtype=torch.float32).to(dev))
        for name in self.strategy_order:
            prep = getattr(self.strategies.get(name), "prepare", None)
            if prep is not None:
                prep(self.resources, x0.shape[0])
        epoch = _lib.rng_epoch(dev)
        static_x = x0.clone()
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            _lib.rng_epoch_advance(epoch)
            _, out = self._run(self.rng_key, static_x, data, self.strategy_order)
        cap = CapturedSchedule(g, static_x, out, self._pollers())
        if not hasattr(self, "_captured"):
            self._captured = {}
        self._captured[tuple(self.strategy_order)] = cap
        return cap

    def serialize(self):
        raise NotImplementedError

    def deserialize(self):
        raise NotImplementedError


class CapturedSchedule:
    """A strategy schedule captured as one CUDA graph: ``replay(x)`` copies the
    starting positions into the graph's input and launches the graph; the
    returned tensor (the schedule's last positions) is the graph's output
    and is overwritten by the next replay."""

    def __init__(self, graph, static_input, static_output, pollers=()):
        self.graph = graph
        self.static_input = static_input
        self.static_output = static_output
        self.pollers = list(pollers)

    def replay(self, initial_position):
        """Launch the graph. Errors that the previous replay's device-side
        checks recorded are raised first (that replay has finished by then,
        or this call waits for it)."""
        self.poll_errors()
        self.static_input.copy_(torch.atleast_2d(initial_position), non_blocking=True)
        self.graph.replay()
        if self.pollers:
            ev = torch.cuda.Event()
            ev.record()
            for p in self.pollers:
                p.mark_error_copy(ev)
        return self.static_output

    def poll_errors(self):
        """Raise the error recorded by the last replay's checks (waits for that replay)."""
        for p in self.pollers:
            p.poll_errors()
