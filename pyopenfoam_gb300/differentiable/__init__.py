"""Differentiation through the linear solve and the Laplacian assembly."""

from .linear_solver import DifferentiableLinearSolve, dls_grads

__all__ = ["DifferentiableLinearSolve", "dls_grads"]
