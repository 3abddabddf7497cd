"""GPU linear solvers with the reference's ``pyfoam.solvers`` interface."""

from .batched import BatchedPCGSolver
from .linear_solver import LinearSolverBase, create_solver, register_solver, solver_from_dict
from .mixed import MixedPrecisionPCGSolver
from .pbicgstab import PBiCGSTABSolver
from .pcg import PCGSolver
from .preconditioners import DICPreconditioner, DILUPreconditioner, Preconditioner
from .pressure_equation import assemble_pressure_equation, solve_pressure_equation
from .residual import ConvergenceInfo, ResidualMonitor

__all__ = [
    "LinearSolverBase", "create_solver", "solver_from_dict", "register_solver", "PCGSolver",
    "PBiCGSTABSolver", "MixedPrecisionPCGSolver", "DICPreconditioner", "DILUPreconditioner", "Preconditioner",
    "ConvergenceInfo", "ResidualMonitor", "BatchedPCGSolver", "assemble_pressure_equation",
    "solve_pressure_equation",
]
