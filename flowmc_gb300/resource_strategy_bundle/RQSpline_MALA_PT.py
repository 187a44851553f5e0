"""RQSpline_MALA_PT_Bundle (mirrors resource_strategy_bundle/RQSpline_MALA_PT.py:21-344).

The RQSpline_MALA bundle plus a parallel-tempering step at the head of every
training and production loop: the same resources, strategy names and
schedule as the reference, with the tempered resources ``tempered_logpdf``
(TemperedPDF), ``tempered_positions`` [n_chains, n_temperatures - 1, n_dims]
and ``temperature`` (linspace(1, max_temperature, n_temperatures)). The
tempered local steps, the exchange sweep and the temperature adaptation run
on the device (strategy/parallel_tempering.py of this package).

``logprior`` is the reference's zero prior by default; a
``targets.DiagGaussian`` prior also runs inside the fused kernel.
"""
from __future__ import annotations

import torch

from ..resource.buffers import Buffer
from ..resource.logPDF import TemperedPDF
from ..strategy.lambda_function import Lambda
from ..strategy.parallel_tempering import ParallelTempering
from .RQSpline_MALA import RQSpline_MALA_Bundle


class RQSpline_MALA_PT_Bundle(RQSpline_MALA_Bundle):
    """A Rational Quadratic Spline flow as the global proposal, MALA as the
    local sampler and an additional parallel-tempering step."""

    def __repr__(self):
        return "RQSpline MALA PT Bundle"

    def __init__(self, rng_key, n_chains: int, n_dims: int, logpdf, n_local_steps: int, n_global_steps: int,
                 n_training_loops: int, n_production_loops: int, n_epochs: int, mala_step_size: float = 1e-1,
                 chain_batch_size: int = 0, rq_spline_hidden_units: list = [32, 32], rq_spline_n_bins: int = 8,
                 rq_spline_n_layers: int = 4, learning_rate: float = 1e-3, batch_size: int = 10000,
                 n_max_examples: int = 10000, local_thinning: int = 1, global_thinning: int = 1,
                 n_NFproposal_batch_size: int = 10000, history_window: int = 100, n_temperatures: int = 5,
                 max_temperature: float = 5.0, n_tempered_steps: int = -1, logprior=None, verbose: bool = False,
                 local_sampler=None, precision: str = "float32", device=None, autotune: bool = False):
        super().__init__(rng_key, n_chains, n_dims, logpdf, n_local_steps, n_global_steps, n_training_loops,
                         n_production_loops, n_epochs, mala_step_size=mala_step_size,
                         chain_batch_size=chain_batch_size, rq_spline_hidden_units=rq_spline_hidden_units,
                         rq_spline_n_bins=rq_spline_n_bins, rq_spline_n_layers=rq_spline_n_layers,
                         learning_rate=learning_rate, batch_size=batch_size, n_max_examples=n_max_examples,
                         local_thinning=local_thinning, global_thinning=global_thinning,
                         n_NFproposal_batch_size=n_NFproposal_batch_size, verbose=verbose,
                         local_sampler=local_sampler, precision=precision, history_window=history_window,
                         device=device, autotune=autotune)
        logpdf = self.resources["logpdf"]
        # the tempered resources (RQSpline_MALA_PT.py:133-146)
        tempered_logpdf = TemperedPDF(logpdf, logprior, n_dims=n_dims, n_temps=n_temperatures)
        tempered_positions = Buffer("tempered_positions", (n_chains, n_temperatures - 1, n_dims), 2, device=device)
        temperatures = Buffer("temperature", (n_temperatures,), 0, device=device)
        temperatures.update_buffer(torch.linspace(1.0, max_temperature, n_temperatures, dtype=torch.float32))
        self.resources.update({
            "tempered_logpdf": tempered_logpdf,
            "tempered_positions": tempered_positions,
            "temperatures": temperatures,
        })

        if n_tempered_steps <= 0:
            print("n_tempered_steps value is not valid. Setting to n_local_steps")
            n_tempered_steps = n_local_steps
        parallel_tempering_strat = ParallelTempering(
            n_steps=n_tempered_steps, tempered_logpdf_name="tempered_logpdf", kernel_name="local_sampler",
            tempered_buffer_names=["tempered_positions", "temperatures"], state_name="sampler_state",
            verbose=verbose)

        def initialize_tempered_positions(rng_key, resources, initial_position, data):
            # every tempered chain starts at its chain's position (RQSpline_MALA_PT.py:298-316)
            x0 = torch.atleast_2d(initial_position).to(tempered_positions.data)
            tempered_positions.data.copy_(x0[:, None].expand(-1, n_temperatures - 1, -1))
            return rng_key, resources, initial_position

        self.strategies["parallel_tempering"] = parallel_tempering_strat
        self.strategies["initialize_tempered_positions"] = Lambda(initialize_tempered_positions)

        training_phase = ["parallel_tempering", "local_stepper", "update_global_step", "model_trainer",
                          "update_model", "global_stepper", "update_local_step"]
        production_phase = ["parallel_tempering", "local_stepper", "update_global_step", "global_stepper",
                            "update_local_step"]
        strategy_order = ["initialize_tempered_positions"]
        for _ in range(n_training_loops):
            strategy_order.extend(training_phase)
        strategy_order.append("reset_steppers")
        strategy_order.append("update_state")
        for _ in range(n_production_loops):
            strategy_order.extend(production_phase)
        self.strategy_order = strategy_order
