"""flowmc_gb300 -- a GB300-native (sm_103a) implementation of flowMC's
sampling hot path behind flowMC's Python API.

Layout mirrors the reference package (flowMC v0.4.5):
  resource/            Buffer, State, LogPDF, TemperedPDF, kernels (MALA,
                       HMC, GaussianRandomWalk, NFProposal), flow model,
                       Optimizer
  strategy/            TakeSerialSteps, TakeGroupSteps, TrainModel, Lambda,
                       UpdateState, ParallelTempering
  resource_strategy_bundle/  RQSpline_MALA_Bundle, RQSpline_MALA_PT_Bundle
  Sampler              the top-level driver
Device work runs in libflowmc.so (csrc/, C ABI in include/flowmc.h).
"""
__version__ = "0.1.0"
