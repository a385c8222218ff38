"""GB300-native Metropolis dipole-lattice sweep (StarryNight hot path).

The compute path is the CUDA library ``lib/libsn_gpu.so`` behind the C ABI
declared in ``include/sn_gpu.h``; this package is its Python host side.
There is no CPU fallback: without the built library every entry point
raises.
"""
from .native import build, lib_path, driver_path
from ._abi import SnError
from .sim import (ModelParams, Replica, Simulation, check_flow, check_schedule, fp32_peak, neighbour_count, philox,
                  plan_candidates, plan_schedule)

__all__ = [
    "build", "lib_path", "driver_path", "SnError", "ModelParams", "Replica", "Simulation",
    "check_flow", "check_schedule", "fp32_peak", "neighbour_count", "philox", "plan_candidates", "plan_schedule",
]
