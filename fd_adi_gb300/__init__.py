"""fd_adi_gb300: GB300-native (sm_103a) FP64 ADI pricer for Heston and Black-Scholes.

Drop-in for the GPU path of johntyree/fd_adi (FiniteDifference.BandedOperatorGPU
and FiniteDifference.FiniteDifferenceEngineGPU) on torch CUDA tensors, with
every computation in libfdadi.so (include/fdadi.h).
"""
from .option import (Option, HestonOption, BarrierOption, HestonBarrierOption,
                     MeanRevertingProcess, Grid)
from . import mesh
from .mesh import sinh_space, exponential_space

__all__ = ["Option", "HestonOption", "BarrierOption", "HestonBarrierOption",
           "MeanRevertingProcess", "Grid", "mesh", "sinh_space", "exponential_space",
           "BandedOperator", "for_vector", "mixed_for_vector", "FiniteDifferenceEngineADI",
           "HestonFiniteDifferenceEngine", "BlackScholesFiniteDifferenceEngine", "HestonBatch"]


def __getattr__(name):
    # the GPU classes import torch and load libfdadi.so on first use
    if name in ("BandedOperator", "for_vector", "mixed_for_vector"):
        from . import banded_operator
        return getattr(banded_operator, name)
    if name in ("FiniteDifferenceEngineADI", "HestonFiniteDifferenceEngine",
                "BlackScholesFiniteDifferenceEngine", "FiniteDifferenceEngine"):
        from . import engine
        return getattr(engine, name)
    if name == "HestonBatch":
        from . import batch
        return batch.HestonBatch
    raise AttributeError(name)
