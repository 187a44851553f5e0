"""RQSpline_MALA_Bundle (mirrors resource_strategy_bundle/RQSpline_MALA.py:22-273).

Same resources, strategies, names and training -> production schedule as the
reference. Build-only keyword arguments (all optional, defaults keep the
reference's behaviour):
  local_sampler      a local kernel used instead of MALA(mala_step_size)
                     (e.g. HMC for the Rosenbrock workload)
  precision          "float32" (default) or "bf16" conditioner GEMMs
  history_window     TrainModel's per-chain window (the reference fixes 100)
  device             where buffers and the flow live
  autotune           measure the local kernel's chain-block shape, the flow
                     GEMMs' tile shapes and ring depth, and the training
                     weight-gradient split on first use
  streaming_diagnostics
                     accumulate FP64 moments, R-hat and batch-means ESS of
                     the production rows on the device as they are written
                     (``bundle.production_moments``, a
                     diagnostics.StreamingMoments; batches of
                     ``streaming_batch`` draws, default one production loop)
"""
from __future__ import annotations

from ..random import split
from ..resource.buffers import Buffer
from ..resource.kernel.MALA import MALA
from ..resource.kernel.NF_proposal import NFProposal
from ..resource.logPDF import LogPDF
from ..resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
from ..resource.optimizer import Optimizer
from ..resource.states import State
from ..strategy.lambda_function import Lambda
from ..strategy.take_steps import TakeGroupSteps, TakeSerialSteps
from ..strategy.train_model import TrainModel
from ..strategy.update_state import UpdateState
from .base import ResourceStrategyBundle


class RQSpline_MALA_Bundle(ResourceStrategyBundle):
    """A Rational Quadratic Spline flow as the global proposal and MALA as the
    local sampler (https://www.pnas.org/doi/full/10.1073/pnas.2109420119)."""

    def __repr__(self):
        return "RQSpline_MALA Bundle"

    def __init__(self, rng_key, n_chains: int, n_dims: int, logpdf, n_local_steps: int, n_global_steps: int,
                 n_training_loops: int, n_production_loops: int, n_epochs: int, mala_step_size: float = 1e-1,
                 chain_batch_size: int = 0, rq_spline_hidden_units: list = [32, 32], rq_spline_n_bins: int = 8,
                 rq_spline_n_layers: int = 4, learning_rate: float = 1e-3, batch_size: int = 10000,
                 n_max_examples: int = 10000, local_thinning: int = 1, global_thinning: int = 1,
                 n_NFproposal_batch_size: int = 10000, verbose: bool = False, local_sampler=None,
                 precision: str = "float32", history_window: int = 100, device=None, autotune: bool = False,
                 streaming_diagnostics: bool = False, streaming_batch: int = 0):
        n_training_steps = (n_local_steps // local_thinning * n_training_loops
                            + n_global_steps // global_thinning * n_training_loops)
        n_production_steps = (n_local_steps // local_thinning * n_production_loops
                              + n_global_steps // global_thinning * n_production_loops)
        n_total_epochs = n_training_loops * n_epochs

        positions_training = Buffer("positions_training", (n_chains, n_training_steps, n_dims), 1, device=device)
        log_prob_training = Buffer("log_prob_training", (n_chains, n_training_steps), 1, device=device)
        local_accs_training = Buffer("local_accs_training", (n_chains, n_training_steps), 1, device=device)
        global_accs_training = Buffer("global_accs_training", (n_chains, n_training_steps), 1, device=device)
        loss_buffer = Buffer("loss_buffer", (n_total_epochs,), 0, device=device)
        position_production = Buffer("positions_production", (n_chains, n_production_steps, n_dims), 1,
                                     device=device)
        log_prob_production = Buffer("log_prob_production", (n_chains, n_production_steps), 1, device=device)
        local_accs_production = Buffer("local_accs_production", (n_chains, n_production_steps), 1, device=device)
        global_accs_production = Buffer("global_accs_production", (n_chains, n_production_steps), 1, device=device)

        local_sampler = MALA(step_size=mala_step_size) if local_sampler is None else local_sampler
        rng_key, subkey = split(rng_key)
        model = MaskedCouplingRQSpline(n_dims, rq_spline_n_layers, rq_spline_hidden_units, rq_spline_n_bins, subkey,
                                       precision=precision, device=device)
        global_sampler = NFProposal(model, n_NFproposal_batch_size=n_NFproposal_batch_size)
        optimizer = Optimizer(model=model, learning_rate=learning_rate)
        logpdf = logpdf if isinstance(logpdf, LogPDF) else LogPDF(logpdf, n_dims=n_dims)

        sampler_state = State({
            "target_positions": "positions_training",
            "target_log_prob": "log_prob_training",
            "target_local_accs": "local_accs_training",
            "target_global_accs": "global_accs_training",
            "training": True,
        }, name="sampler_state")

        self.resources = {
            "logpdf": logpdf,
            "positions_training": positions_training,
            "log_prob_training": log_prob_training,
            "local_accs_training": local_accs_training,
            "global_accs_training": global_accs_training,
            "loss_buffer": loss_buffer,
            "positions_production": position_production,
            "log_prob_production": log_prob_production,
            "local_accs_production": local_accs_production,
            "global_accs_production": global_accs_production,
            "local_sampler": local_sampler,
            "global_sampler": global_sampler,
            "model": model,
            "optimizer": optimizer,
            "sampler_state": sampler_state,
        }

        local_stepper = TakeSerialSteps("logpdf", "local_sampler", "sampler_state",
                                        ["target_positions", "target_log_prob", "target_local_accs"], n_local_steps,
                                        thinning=local_thinning, chain_batch_size=chain_batch_size, verbose=verbose,
                                        autotune=autotune)
        global_stepper = TakeGroupSteps("logpdf", "global_sampler", "sampler_state",
                                        ["target_positions", "target_log_prob", "target_global_accs"],
                                        n_global_steps, thinning=global_thinning, chain_batch_size=chain_batch_size,
                                        verbose=verbose, autotune=autotune)
        model_trainer = TrainModel("model", "positions_training", "optimizer", loss_buffer_name="loss_buffer",
                                   n_epochs=n_epochs, batch_size=batch_size, n_max_examples=n_max_examples,
                                   history_window=history_window, verbose=verbose, autotune=autotune)
        update_state = UpdateState(
            "sampler_state",
            ["target_positions", "target_log_prob", "target_local_accs", "target_global_accs", "training"],
            ["positions_production", "log_prob_production", "local_accs_production", "global_accs_production",
             False])

        self.production_moments = None
        moments_cursor = [0]
        if streaming_diagnostics:
            from ..diagnostics import StreamingMoments
            per_loop = n_local_steps // local_thinning + n_global_steps // global_thinning
            self.production_moments = StreamingMoments(n_chains, n_dims, streaming_batch or per_loop,
                                                       device=position_production.data.device)

        def reset_steppers(rng_key, resources, initial_position, data):
            local_stepper.set_current_position(0)
            global_stepper.set_current_position(0)
            if self.production_moments is not None:
                self.production_moments.reset()
                moments_cursor[0] = 0
            return rng_key, resources, initial_position

        def update_moments(rng_key, resources, initial_position, data):
            # the production rows this loop wrote: [cursor, the steppers' position)
            end = global_stepper.current_position
            buf = resources["positions_production"].data
            end = min(end, buf.shape[1])
            if end > moments_cursor[0]:
                self.production_moments.update(buf, moments_cursor[0], end - moments_cursor[0])
                moments_cursor[0] = end
            return rng_key, resources, initial_position

        def update_model(rng_key, resources, initial_position, data):
            # RQSpline_MALA.py:215-232: point the global sampler at the trained model
            resources["global_sampler"].model = resources["model"]
            return rng_key, resources, initial_position

        self.strategies = {
            "local_stepper": local_stepper,
            "global_stepper": global_stepper,
            "model_trainer": model_trainer,
            "update_state": update_state,
            "update_global_step": Lambda(lambda k, r, x, d: global_stepper.set_current_position(
                local_stepper.current_position)),
            "update_local_step": Lambda(lambda k, r, x, d: local_stepper.set_current_position(
                global_stepper.current_position)),
            "reset_steppers": Lambda(reset_steppers),
            "update_model": Lambda(update_model),
        }
        training_phase = ["local_stepper", "update_global_step", "model_trainer", "update_model", "global_stepper",
                          "update_local_step"]
        production_phase = ["local_stepper", "update_global_step", "global_stepper", "update_local_step"]
        if streaming_diagnostics:
            self.strategies["update_moments"] = Lambda(update_moments)
            production_phase = production_phase + ["update_moments"]
        self.training_phase, self.production_phase = training_phase, production_phase
        strategy_order = []
        for _ in range(n_training_loops):
            strategy_order.extend(training_phase)
        strategy_order.append("reset_steppers")
        strategy_order.append("update_state")
        for _ in range(n_production_loops):
            strategy_order.extend(production_phase)
        self.strategy_order = strategy_order
