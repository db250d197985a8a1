"""GB300-native FANS solve path: FFT-preconditioned CG over trilinear voxel
elements, hand-written sm_103a CUDA behind the C ABI in include/fans_gb300.h."""
from . import _lib
from ._lib import FansGpuError
from .materials import MaterialManager
from .solver import Context, Solver, SolverCG, SolverFP, create_solver, solve_batch

__all__ = ["solve_batch", "Context", "Solver", "SolverCG", "SolverFP", "create_solver", "MaterialManager", "FansGpuError", "_lib"]
