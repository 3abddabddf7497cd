"""GPU linear solvers with the reference's ``pyfoam.solvers`` interface."""

from .batched import BatchedPCGSolver
from .diagonal import DiagonalSolver
from .gamg import GAMGSolver
from .linear_solver import LinearSolverBase, create_solver, register_solver, solver_from_dict
from .mixed import MixedPrecisionPBiCGSTABSolver, MixedPrecisionPCGSolver
from .pbicg import PBiCGSolver
from .pbicgstab import PBiCGSTABSolver
from .pcg import PCGSolver
from .preconditioners import DICPreconditioner, DILUPreconditioner, Preconditioner
from .pressure_equation import (adjust_phi, assemble_pressure_equation, correct_face_flux,
                                correct_velocity, solve_pressure_equation)
from .residual import ConvergenceInfo, ResidualMonitor
from .smooth_solver import SmoothSolver
from .smoothers import DICGSmoother, GaussSeidelSmoother, JacobiSmoother

__all__ = [
    "LinearSolverBase", "create_solver", "solver_from_dict", "register_solver", "PCGSolver",
    "PBiCGSTABSolver", "MixedPrecisionPCGSolver", "MixedPrecisionPBiCGSTABSolver", "SmoothSolver", "DICPreconditioner",
    "DILUPreconditioner", "Preconditioner", "ConvergenceInfo", "ResidualMonitor",
    "BatchedPCGSolver", "assemble_pressure_equation", "solve_pressure_equation",
    "correct_velocity", "correct_face_flux", "adjust_phi", "GaussSeidelSmoother",
    "JacobiSmoother", "DICGSmoother", "GAMGSolver", "PBiCGSolver", "DiagonalSolver",
]
