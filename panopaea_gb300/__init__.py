"""panopaea_gb300 -- the grid-fluid step of msiglreith/panopaea on GB300 (sm_103a).

The compute path is ``libpanopaea_gpu.so`` (hand-written CUDA behind the C ABI
of ``include/panopaea_gpu.h``); this package is the host-side mirror of the
reference's Rust API (grid/field types, DEC operators, PCG, advection, step).
"""

from . import _native
from .batch import Batch2d, partition_by_cost
from ._native import PgError
from .fluid import BFECC, MACCORMACK, SolverConfig, StepConfig, advect, advect2, advect_mac, solve_pressure, step
from .grid import Grid2d, Grid3d, Simplex1, Simplex2
from .learned import PressureNet, solve_with_guess
from .pcg import IDENTITY, JACOBI, LaplacianOperator, Preconditioner, precond_conjugate_gradient

__all__ = [
    "Grid2d", "Grid3d", "Simplex1", "Simplex2", "IDENTITY", "JACOBI", "LaplacianOperator", "Preconditioner",
    "precond_conjugate_gradient", "advect", "advect2", "MACCORMACK", "BFECC", "advect_mac", "step", "solve_pressure", "StepConfig", "SolverConfig",
    "Batch2d", "partition_by_cost", "PgError", "PressureNet", "solve_with_guess",
]


def load():
    """Load (building if needed) the native library; raises if unavailable."""
    return _native.load()
