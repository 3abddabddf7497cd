"""Preconditioned BiCGStab on the GPU, drop-in for
``pyfoam.solvers.pbicgstab.PBiCGSTABSolver``
(``src/pyfoam/solvers/pbicgstab.py:49-239``).

Same iteration, breakdown tests (rho, rt.v, t.t branch, omega) and residual
checks (on s and on r, two history entries per iteration) as the reference,
run by libgbfoam's ``gbf_pbicgstab_solve_f64``.
"""

from __future__ import annotations

import torch

from ..core.ldu_matrix import LduMatrix
from .linear_solver import LinearSolverBase
from .preconditioners import DICPreconditioner, DILUPreconditioner, Preconditioner
from .residual import ConvergenceInfo, ResidualMonitor
from ._krylov import run_solver

__all__ = ["PBiCGSTABSolver"]


class PBiCGSTABSolver(LinearSolverBase):
    """PBiCGStab for general LDU matrices; ``preconditioner`` is ``"DILU"``
    (default), ``"DIC"`` or ``"none"``.

    ``omega`` (keyword only): ``"reference"`` (default) takes the
    stabilisation step omega = (t.z)/(t.t) exactly as the reference
    (pbicgstab.py:210); ``"standard"`` takes BiCGStab's minimal-residual step
    (t.s)/(t.t).  The reference form is not scale invariant: on unscaled FV
    systems (diagonal >> 1) it stagnates, which the standard form avoids."""

    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, max_iter: int = 1000,
                 min_iter: int = 0, verbose: bool = False, preconditioner: str = "DILU", *,
                 omega: str = "reference", check_every: int = 16) -> None:
        super().__init__(tolerance=tolerance, rel_tol=rel_tol, max_iter=max_iter,
                         min_iter=min_iter, verbose=verbose)
        self._precond_type = preconditioner.upper()
        if omega not in ("reference", "standard"):
            raise ValueError(f"omega must be 'reference' or 'standard', got {omega!r}")
        self._omega = omega
        self._check_every = int(check_every)

    def _make_preconditioner(self, matrix: LduMatrix) -> Preconditioner | None:
        if self._precond_type == "DILU":
            return DILUPreconditioner(matrix)
        if self._precond_type == "DIC":
            return DICPreconditioner(matrix)
        if self._precond_type == "NONE":
            return None
        raise ValueError(
            f"Unknown preconditioner '{self._precond_type}'. Use 'DILU', 'DIC', or 'none'."
        )

    def _solve(self, matrix: LduMatrix, source: torch.Tensor, x0: torch.Tensor,
               monitor: ResidualMonitor, max_iter: int) -> tuple[torch.Tensor, ConvergenceInfo]:
        precond = self._make_preconditioner(matrix)
        pd = None if precond is None else precond.precond_diag
        x, info, _ = run_solver("gbf_pbicgstab_solve_f64", "gbf_pbicgstab_workspace_bytes",
                                matrix, source, x0, monitor, max_iter, pd, 2 * max_iter + 1,
                                self._check_every, variant=1 if self._omega == "standard" else 0)
        return x, info
