"""Residual monitoring, drop-in for ``pyfoam.solvers.residual``
(``src/pyfoam/solvers/residual.py:27-168``).

The GPU solvers evaluate the same rules on the device (L2 norm per check,
``|r| < tolerance`` or ``|r|/|r0| < rel_tol`` once ``iteration >= min_iter``)
and hand the residual history back through :meth:`ResidualMonitor.record`,
so ``build_info`` reports exactly what the reference's monitor would.
"""

from __future__ import annotations

import logging
from dataclasses import dataclass, field

import torch

__all__ = ["ResidualMonitor", "ConvergenceInfo"]

logger = logging.getLogger(__name__)


@dataclass
class ConvergenceInfo:
    converged: bool
    iterations: int
    final_residual: float
    initial_residual: float
    residual_ratio: float
    tolerance: float
    residual_history: list[float] = field(default_factory=list)


class ResidualMonitor:
    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, min_iter: int = 0,
                 verbose: bool = False) -> None:
        self._tolerance = tolerance
        self._rel_tol = rel_tol
        self._min_iter = min_iter
        self._verbose = verbose
        self._history: list[float] = []
        self._initial_residual: float | None = None

    @property
    def tolerance(self) -> float:
        return self._tolerance

    @property
    def rel_tol(self) -> float:
        return self._rel_tol

    @property
    def min_iter(self) -> int:
        return self._min_iter

    @property
    def history(self) -> list[float]:
        return self._history

    @property
    def initial_residual(self) -> float | None:
        return self._initial_residual

    def reset(self) -> None:
        self._history.clear()
        self._initial_residual = None

    def _ratio(self, res_norm: float) -> float:
        """|r| / |r0|, taken as 0 while the first norm is zero or unknown."""
        r0 = self._initial_residual
        return res_norm / r0 if r0 else 0.0

    def _log(self, label: str, k: int, res_norm: float) -> None:
        logger.info("  %s %d: |r| %.6e, |r|/|r0| %.6e", label, k, res_norm,
                    self._ratio(res_norm))

    def check(self, res_norm: float, iteration: int) -> bool:
        """Record one residual norm and apply the convergence rules
        (residual.py:112-145): from ``min_iter`` on, an absolute norm below
        ``tolerance`` or a ratio to the first norm below ``rel_tol`` stops
        the solve."""
        self._history.append(res_norm)
        if self._initial_residual is None:
            self._initial_residual = res_norm
        if self._verbose:
            self._log("iteration", iteration, res_norm)
        if iteration < self._min_iter:
            return False
        r0 = self._initial_residual
        return res_norm < self._tolerance or (r0 > 0 and res_norm / r0 < self._rel_tol)

    def update(self, residual: torch.Tensor, iteration: int) -> bool:
        return self.check(float(torch.linalg.vector_norm(residual).item()), iteration)

    def record(self, history: list[float]) -> None:
        """Adopt a residual history produced on the device."""
        self._history = list(history)
        self._initial_residual = self._history[0] if self._history else None
        if self._verbose:
            for k, res_norm in enumerate(self._history):
                self._log("check", k, res_norm)

    def build_info(self, converged: bool) -> ConvergenceInfo:
        """Summary of the recorded checks: their count is the iteration
        count, the last norm the final residual (0.0 for an empty history)."""
        hist = list(self._history)
        last = hist[-1] if hist else 0.0
        first = self._initial_residual if self._initial_residual else 0.0
        return ConvergenceInfo(converged, len(hist), last, first,
                               self._ratio(last) if first > 0 else 0.0, self._tolerance, hist)
