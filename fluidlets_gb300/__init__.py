"""fluidlets_gb300: the fluidlets hot path on one GB300 (sm_103a).

Drop-in for the reference package ``fluidlets``: the same kernel objects and
operator API (``evaluate``, ``assemble``, ``assemble_nearest``,
``resistance``, ``swimming_problem``), computed by hand-written CUDA kernels
in ``libfluidlets_gb300.so``.
"""
from .core import DENSE_MAX, SolveInfo, assemble, assemble_nearest, evaluate, evaluate_grid, nearest_neighbors, resistance
from .kernels import Brinkmanlet3D, Kernel, Stokeslet3D, VectorKernel, WallStokeslet3D
from .stokeslet3d import stokeslet3d_velocity
from .rigid import resistance_matrix, rigid_body_mobility
from .swimming import SwimmerShape, SwimState, Trajectory, swim, swimming_problem

__version__ = "1.0.0"
__all__ = [
    "evaluate_grid",
    "resistance_matrix",
    "rigid_body_mobility",
    "stokeslet3d_velocity",
    "Kernel",
    "VectorKernel",
    "Stokeslet3D",
    "WallStokeslet3D",
    "Brinkmanlet3D",
    "assemble",
    "assemble_nearest",
    "nearest_neighbors",
    "evaluate",
    "resistance",
    "SolveInfo",
    "DENSE_MAX",
    "SwimmerShape",
    "SwimState",
    "Trajectory",
    "swimming_problem",
    "swim",
]
