"""Preconditioned conjugate gradient on the GPU, drop-in for
``pyfoam.solvers.pcg.PCGSolver`` (``src/pyfoam/solvers/pcg.py:43-187``).

The iteration is the reference's, step for step (alpha = rz/pAp with the
|pAp| < 1e-30 breakdown test, x += alpha p, r -= alpha Ap, z = r/d,
beta = rz'/rz, p = z + beta p), run by libgbfoam's ``gbf_pcg_solve_f64``:
three kernels per iteration with device-resident scalars and no host
synchronisation inside the loop.
"""

from __future__ import annotations

import torch

from ..core.ldu_matrix import LduMatrix
from .linear_solver import LinearSolverBase
from .preconditioners import DICPreconditioner, DILUPreconditioner, Preconditioner
from .residual import ConvergenceInfo, ResidualMonitor
from ._krylov import run_solver

__all__ = ["PCGSolver"]


class PCGSolver(LinearSolverBase):
    """PCG for symmetric positive-definite LDU matrices.

    ``preconditioner`` is ``"DIC"`` (default), ``"DILU"`` or ``"none"``.
    GPU knobs (keyword only): ``check_every`` is the number of iterations
    between host reads of the device status block; ``launch`` is
    ``"auto"`` (default: the whole solve in one cooperative launch with grid
    barriers up to 2^21 cells, where per-iteration launches would dominate,
    three kernels per iteration above), ``"kernels"`` or ``"single"``."""

    _LAUNCH = {"auto": 0, "kernels": 1, "single": 2}

    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, max_iter: int = 1000,
                 min_iter: int = 0, verbose: bool = False, preconditioner: str = "DIC", *,
                 check_every: int = 32, launch: str = "auto") -> None:
        super().__init__(tolerance=tolerance, rel_tol=rel_tol, max_iter=max_iter,
                         min_iter=min_iter, verbose=verbose)
        self._precond_type = preconditioner.upper()
        self._check_every = int(check_every)
        if launch not in self._LAUNCH:
            raise ValueError(f"launch must be one of {sorted(self._LAUNCH)}, got {launch!r}")
        self._launch = launch

    def _make_preconditioner(self, matrix: LduMatrix) -> Preconditioner | None:
        if self._precond_type == "DIC":
            return DICPreconditioner(matrix)
        if self._precond_type == "DILU":
            return DILUPreconditioner(matrix)
        if self._precond_type == "NONE":
            return None
        raise ValueError(
            f"Unknown preconditioner '{self._precond_type}'. Use 'DIC', 'DILU', or 'none'."
        )

    def _solve(self, matrix: LduMatrix, source: torch.Tensor, x0: torch.Tensor,
               monitor: ResidualMonitor, max_iter: int) -> tuple[torch.Tensor, ConvergenceInfo]:
        precond = self._make_preconditioner(matrix)
        pd = None if precond is None else precond.precond_diag
        x, info, R = run_solver("gbf_pcg_solve_f64", "gbf_pcg_workspace_bytes", matrix, source,
                                x0, monitor, max_iter, pd, max_iter + 1, self._check_every,
                                variant=self._LAUNCH[self._launch])
        self.last_result = R
        return x, info
