"""GB300-native cell-centred finite-volume Euler solver for triangle meshes.

A drop-in for the solve path of GPUEularSolver2D behind a C ABI
(include/euler2d.h, libeuler2d.so).  This package holds the CUDA kernels and
C++ host code (csrc/), their build (build.py) and a thin ctypes view of the
C ABI (api.py) used by the tests and the benchmark.
"""
from .api import (E2D_FP32, E2D_FP64, E2D_LIMITER_CELL_BARTH, E2D_LIMITER_CELL_VENKAT, E2D_LIMITER_REFERENCE,
                  E2D_LIMITER_VENKAT, E2D_ORDER_FILE, E2D_ORDER_MORTON, E2D_ORDER_RCM, MLP, Batch, Mesh, Params,
                  Solver, default_params, read_input, state_integrals)

__all__ = ["Mesh", "Solver", "Batch", "MLP", "Params", "default_params", "read_input", "state_integrals",
           "E2D_FP32", "E2D_FP64", "E2D_LIMITER_REFERENCE", "E2D_LIMITER_VENKAT", "E2D_LIMITER_CELL_BARTH",
           "E2D_LIMITER_CELL_VENKAT",
           "E2D_ORDER_FILE", "E2D_ORDER_MORTON", "E2D_ORDER_RCM"]
