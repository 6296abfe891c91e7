"""spinorbec — SpinorBEC.jl's split-step API on the GB300 engine (libsbec.so).

Host helpers (grid, potentials, initial states, parameter containers) stay in
Python, as they stay in Julia for the reference; every hot-path call goes
through the C ABI of ``include/sbec.h`` to CUDA kernels.  There is no CPU
fallback.
"""

from ._lib import (ArgumentError, CallbackStop, DeviceError, NumericError, OutOfMemoryError, SbecError,
                   UnsupportedError, load)
from .api import *  # noqa: F401,F403
from .host import *  # noqa: F401,F403
from .experiment import (ExperimentConfig, ExperimentResult, parse_experiment,  # noqa: F401
                         run_experiment)


def device_count() -> int:
    return int(load().sbec_device_count())
