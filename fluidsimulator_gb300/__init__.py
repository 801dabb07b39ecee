"""GB300 (sm_103a) Position Based Fluids timestep: a drop-in for the CUDA
backend of CTKnight/FluidSimulator behind the C ABI in include/fluid_gb300.h."""

from ._capi import FluidParams, FluidStats, default_params  # noqa: F401
