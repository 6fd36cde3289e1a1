"""fdfdpy_gb300: a GB300-native (sm_103a) engine for fdfdpy's hot path.

Drop-in Python API of fdfdpy (``Simulation``, ``construct_A``,
``solver_direct``) over a C-ABI CUDA library: fused PML operator assembly,
a matrix-free FP64 residual, and a nested-dissection multifrontal sparse LU
(complex128, or complex64 + FP64 iterative refinement).
"""
from .simulation import Simulation  # noqa: F401
from .linalg import construct_A, solver_direct, grid_average, dL  # noqa: F401

name = "fdfdpy_gb300"
