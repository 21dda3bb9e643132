"""relion_gb300: a GB300-native (sm_103a) expectation step for RELION.

The compute path is libgbrelion (CUDA kernels behind a C ABI,
include/gbrelion.h); this package holds its build script, the ctypes
binding, a Python mirror of the reference's MlDeviceBundle /
MlOptimiserCuda surface and the synthetic-data generator.
"""
from ._lib import GbrError, load  # noqa: F401
from .estep import MlDeviceBundle, MlOptimiserCuda, STAGES  # noqa: F401

__all__ = ["GbrError", "load", "MlDeviceBundle", "MlOptimiserCuda", "STAGES"]
