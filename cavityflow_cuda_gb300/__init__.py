"""GB300-native D3Q19 A-A lattice-Boltzmann lid-driven-cavity solver.

A drop-in for the solver of saleemayman/cavityflow_cuda: the C ABI in
include/lbm_gb300.h, implemented by hand-written sm_103a kernels in csrc/, and
this Python binding of it (``CLbmSolverGB300``).
"""
from .solver import (BACK, BOTTOM, DIRECTION_ALL, FLUID, FRONT, GHOST_LAYER, LEFT, OBSTACLE, RIGHT, STORAGE,
                     TOP, VELOCITY_INJECTION, CLbmSolverGB300, LbmBatch, LbmError, LbmServer, configuration_lattice,
                     declared_functions, derive_lattice, kernel_launches, load_library, read_configuration)

__all__ = [
    "CLbmSolverGB300", "LbmBatch", "LbmError", "LbmServer", "derive_lattice", "declared_functions", "kernel_launches", "load_library",
    "read_configuration", "configuration_lattice",
    "OBSTACLE", "FLUID", "VELOCITY_INJECTION", "GHOST_LAYER", "DIRECTION_ALL", "LEFT", "RIGHT", "BOTTOM", "TOP",
    "BACK", "FRONT", "STORAGE",
]
