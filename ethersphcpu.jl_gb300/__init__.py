"""GB300-native WCSPH time step for EtherSPHCPU.jl models (host side).

The compute path is the CUDA library ``lib/libethersph_gpu.so`` (C ABI in
include/ethersph_gpu.h); this package mirrors the reference's type tree and its
`solve!` entry point on top of it.  Import name: ``ethersph_gb300``.
"""
from . import _abi
from ._abi import SphError, SphParams, SphStats, load_library
from .solver import Simulation, kernelValueInterpolation, make_params, solve, solve_inlet_outlet
from .batch import Batch
from .vtp import VTPIO
from .types import (AABBCheck, CommonLiquidParticles, CommonWeaklyCompressibleLiquidModel, CompulsiveWallParticles,
                    CubicSpline, DensityReinitializedFixedTimeIntervalForwardEuler, Gaussian, SmoothKernel,
                    StaticVelocityWallParticles, ThermalLiquidParticles, ThermalWeaklyCompressibleLiquidModel,
                    ThermostaticWallParticles, WendlandC2, WendlandC4, isCheckStep, isDensityReinitializedStep,
                    isOutputStep)

__all__ = [n for n in dir() if not n.startswith("_")]
