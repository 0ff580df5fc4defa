from .solver import Solver, SolverBase
from .loss import Loss

__all__ = ["Solver", "SolverBase", "Loss"]
