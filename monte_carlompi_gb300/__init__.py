"""GB300-native photon random walk for monte_carloMPI's snowpack model.

The walk runs as hand-written sm_103a CUDA kernels behind the C ABI of
``include/mcwalk.h`` (libmcwalk.so, bound here with ctypes).  Python keeps the
reference's drop-in surface: ``MonteCarlo`` (constructor and ``run``), SSP
tables, the per-photon CSV and the BRF / albedo post-processing.
"""
from .config import WalkConfig, read_model_args  # noqa: F401
from .ssp import SSPTable  # noqa: F401

__all__ = ['MonteCarlo', 'Walker', 'WalkConfig', 'SSPTable', 'read_model_args']


def __getattr__(name):
    if name == 'MonteCarlo':
        from .monte_carlo import MonteCarlo
        return MonteCarlo
    if name == 'Walker':
        from .walker import Walker
        return Walker
    raise AttributeError(name)
