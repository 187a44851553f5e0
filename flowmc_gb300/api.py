"""Public API in one namespace (and the import that registers every C entry point)."""
from .random import PRNGKey, split  # noqa: F401
from .resource.buffers import Buffer  # noqa: F401
from .resource.states import State  # noqa: F401
from .resource.logPDF import LogPDF, TemperedPDF, Variable  # noqa: F401
from .resource.kernel.MALA import MALA  # noqa: F401
from .resource.kernel.HMC import HMC  # noqa: F401
from .resource.kernel.Gaussian_random_walk import GaussianRandomWalk  # noqa: F401
from .strategy.take_steps import TakeSerialSteps, TakeGroupSteps  # noqa: F401
from .strategy.lambda_function import Lambda  # noqa: F401
from .strategy.update_state import UpdateState  # noqa: F401
from . import targets  # noqa: F401
from .resource.kernel.NF_proposal import NFProposal  # noqa: F401
from .resource.model.nf_model.rqSpline import MaskedCouplingRQSpline  # noqa: F401
from .resource.model.nf_model.realNVP import RealNVP  # noqa: F401
from .strategy.optimization import AdamOptimization  # noqa: F401
from .resource.optimizer import Optimizer  # noqa: F401
from .strategy.train_model import TrainModel  # noqa: F401
from .resource_strategy_bundle.RQSpline_MALA import RQSpline_MALA_Bundle  # noqa: F401
from .resource_strategy_bundle.RQSpline_MALA_PT import RQSpline_MALA_PT_Bundle  # noqa: F401
from .strategy.parallel_tempering import ParallelTempering  # noqa: F401
from .Sampler import Sampler  # noqa: F401
from . import batched  # noqa: F401
