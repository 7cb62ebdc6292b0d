"""sassena_gb300 — GB300-native scattering-amplitude hot path of Sassena.

The compute path is the CUDA library behind include/sassena_gb300.h (sm_103a kernels,
C ABI); the C++ host devices in sassena_gb300/host drive it from the reference's XML
configuration. This Python package holds the ctypes binding used by tests and the
benchmark, the build recipe and the seeded synthetic workloads.
"""
from .abi import Batch, Plan, SassError, compute_workload, load  # noqa: F401

__all__ = ["Batch", "Plan", "SassError", "compute_workload", "load"]
