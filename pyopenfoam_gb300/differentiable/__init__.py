"""Differentiation through the linear solve, the Laplacian assembly and the
explicit Laplacian."""

from .linear_solver import DifferentiableLinearSolve, dls_grads
from .operators import DifferentiableLaplacian

__all__ = ["DifferentiableLaplacian", "DifferentiableLinearSolve", "dls_grads"]
