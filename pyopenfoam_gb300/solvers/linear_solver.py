"""Linear-solver base class and factory, drop-in for
``pyfoam.solvers.linear_solver`` (``src/pyfoam/solvers/linear_solver.py``).
"""

from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Any

import torch

from ..core.dtype import assert_floating
from ..core.ldu_matrix import LduMatrix
from .residual import ConvergenceInfo, ResidualMonitor

__all__ = ["LinearSolverBase", "create_solver", "solver_from_dict"]


class LinearSolverBase(ABC):
    """Validation, residual monitoring and the ``(x, iterations,
    final_residual)`` return convention (linear_solver.py:41-160)."""

    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, max_iter: int = 1000,
                 min_iter: int = 0, verbose: bool = False) -> None:
        self._tolerance = tolerance
        self._rel_tol = rel_tol
        self._max_iter = max_iter
        self._min_iter = min_iter
        self._verbose = verbose
        self.last_info: ConvergenceInfo | None = None

    @property
    def tolerance(self) -> float:
        return self._tolerance

    @property
    def rel_tol(self) -> float:
        return self._rel_tol

    @property
    def max_iter(self) -> int:
        return self._max_iter

    def __call__(self, matrix: LduMatrix, source: torch.Tensor, x0: torch.Tensor,
                 tolerance: float | None = None, max_iter: int | None = None
                 ) -> tuple[torch.Tensor, int, float]:
        """Solve A x = b (linear_solver.py:88-126)."""
        assert_floating(source, "source")
        assert_floating(x0, "x0")
        tol = tolerance if tolerance is not None else self._tolerance
        max_it = max_iter if max_iter is not None else self._max_iter
        monitor = ResidualMonitor(tolerance=tol, rel_tol=self._rel_tol, min_iter=self._min_iter,
                                  verbose=self._verbose)
        solution, info = self._solve(matrix, source, x0, monitor, max_it)
        self.last_info = info
        return solution, info.iterations, info.final_residual

    @abstractmethod
    def _solve(self, matrix: LduMatrix, source: torch.Tensor, x0: torch.Tensor,
               monitor: ResidualMonitor, max_iter: int) -> tuple[torch.Tensor, ConvergenceInfo]:
        ...

    def __repr__(self) -> str:
        return (f"{self.__class__.__name__}(tolerance={self._tolerance}, "
                f"rel_tol={self._rel_tol}, max_iter={self._max_iter})")


_SOLVER_REGISTRY: dict[str, type[LinearSolverBase]] = {}


def _register_defaults() -> None:
    if _SOLVER_REGISTRY:
        return
    from .mixed import MixedPrecisionPBiCGSTABSolver, MixedPrecisionPCGSolver
    from .pbicgstab import PBiCGSTABSolver
    from .pcg import PCGSolver
    from .diagonal import DiagonalSolver
    from .gamg import GAMGSolver
    from .pbicg import PBiCGSolver
    from .smooth_solver import SmoothSolver

    _SOLVER_REGISTRY["PBICG"] = PBiCGSolver
    _SOLVER_REGISTRY["DIAGONAL"] = DiagonalSolver
    _SOLVER_REGISTRY["GAMG"] = GAMGSolver
    _SOLVER_REGISTRY["PCG"] = PCGSolver
    _SOLVER_REGISTRY["PBICGSTAB"] = PBiCGSTABSolver
    _SOLVER_REGISTRY["SMOOTHSOLVER"] = SmoothSolver
    _SOLVER_REGISTRY["MIXEDPCG"] = MixedPrecisionPCGSolver
    _SOLVER_REGISTRY["MIXEDPBICGSTAB"] = MixedPrecisionPBiCGSTABSolver


def register_solver(name: str, cls: type[LinearSolverBase]) -> None:
    _register_defaults()
    _SOLVER_REGISTRY[name.upper().replace("-", "").replace("_", "")] = cls


def create_solver(name: str, *, tolerance: float = 1e-6, rel_tol: float = 0.01,
                  max_iter: int = 1000, min_iter: int = 0, verbose: bool = False,
                  **kwargs: Any) -> LinearSolverBase:
    """Solver by case-insensitive name (linear_solver.py:163-256); unknown
    names raise ``ValueError`` listing the available ones."""
    _register_defaults()
    key = name.upper().replace("-", "").replace("_", "")
    if key not in _SOLVER_REGISTRY:
        available = ", ".join(sorted(_SOLVER_REGISTRY))
        raise ValueError(f"Unknown solver '{name}'. Available: {available}")
    return _SOLVER_REGISTRY[key](tolerance=tolerance, rel_tol=rel_tol, max_iter=max_iter,
                                 min_iter=min_iter, verbose=verbose, **kwargs)


def solver_from_dict(solver_name: str, solver_dict: dict[str, Any]) -> LinearSolverBase:
    """Solver from an fvSolution sub-dictionary (linear_solver.py:259-304):
    ``tolerance``, ``relTol``, ``maxIter``, ``preconditioner`` and, for
    smoothSolver, ``smoother`` and ``nSweeps``."""
    extra: dict[str, Any] = {}
    if solver_name.upper().replace("-", "").replace("_", "") == "SMOOTHSOLVER":
        if "smoother" in solver_dict:
            extra["smoother"] = solver_dict["smoother"]
        if "nSweeps" in solver_dict:
            extra["n_sweeps"] = int(solver_dict["nSweeps"])
    if "preconditioner" in solver_dict:
        extra["preconditioner"] = solver_dict["preconditioner"]
    return create_solver(
        solver_name,
        tolerance=float(solver_dict.get("tolerance", 1e-6)),
        rel_tol=float(solver_dict.get("relTol", 0.01)),
        max_iter=int(solver_dict.get("maxIter", 1000)),
        **extra,
    )
