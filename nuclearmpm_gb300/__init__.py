"""GB300-native MLS-MPM time step with the reference's solver API.

The compute path is libnclr_gpu.so (hand-written sm_103a CUDA behind the C ABI of
include/nclr_gpu.h); this package binds it for Python callers.
"""
from .simulation import (BatchSimulation, GridArrays, MaterialModel, MPMSimulation,  # noqa: F401
                         Particle, ParticleArrays, diag)
from .capi import NclrError, OutOfRange  # noqa: F401
