"""Smoothing solver on the GPU, drop-in for ``pyfoam.solvers.smooth_solver.
SmoothSolver`` (``src/pyfoam/solvers/smooth_solver.py:37-232``).

Each outer iteration applies ``n_sweeps`` smoothing passes, then checks the
residual with ``ResidualMonitor``'s rules:

* ``"GaussSeidel"`` (default): in-place sweeps x_c = (b_c - sum_{j!=c} a_cj
  x_j) / a_cc over the cells in ascending order -- a level-scheduled
  wavefront that keeps the reference's update order and row sums, so x is
  bitwise the reference's;
* ``"DIC"`` / ``"DILU"``: preconditioned Richardson, x += omega M^-1 (b - A x)
  with the full DIC / DILU solve.

The residual norm of each check is a deterministic device reduction
(``gbf_norm2_f64``), read once per outer iteration as the reference does.
"""

from __future__ import annotations

import torch

from .. import _lib
from ..core.ldu_matrix import LduMatrix
from .linear_solver import LinearSolverBase
from .preconditioners import DICPreconditioner, DILUPreconditioner
from .residual import ConvergenceInfo, ResidualMonitor
from .smoothers import gs_sweep, relax, residual

__all__ = ["SmoothSolver"]


class SmoothSolver(LinearSolverBase):
    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, max_iter: int = 1000,
                 min_iter: int = 0, verbose: bool = False, smoother: str = "GaussSeidel",
                 n_sweeps: int = 2, omega: float = 1.0) -> None:
        super().__init__(tolerance=tolerance, rel_tol=rel_tol, max_iter=max_iter,
                         min_iter=min_iter, verbose=verbose)
        self._smoother = smoother
        self._n_sweeps = n_sweeps
        self._omega = omega

    def _solve(self, matrix: LduMatrix, source: torch.Tensor, x0: torch.Tensor,
               monitor: ResidualMonitor, max_iter: int) -> tuple[torch.Tensor, ConvergenceInfo]:
        if self._smoother not in ("GaussSeidel", "DIC", "DILU"):
            raise ValueError(f"Unknown smoother '{self._smoother}'. "
                             f"Use 'GaussSeidel', 'DIC', or 'DILU'.")
        if matrix.dtype != torch.float64:
            raise TypeError("SmoothSolver runs on float64 matrices")
        dev, n = matrix.device, matrix.n_cells
        b = source.to(device=dev, dtype=torch.float64).contiguous()
        x = x0.to(device=dev, dtype=torch.float64).clone().contiguous()
        if b.shape[0] != n or x.shape[0] != n:
            raise ValueError(f"source/x0 have {b.shape[0]}/{x.shape[0]} elements, expected {n}")
        r = torch.empty_like(x)
        L = _lib.lib()
        ws = torch.empty(int(L.gbf_norm2_workspace_bytes()), device=dev, dtype=torch.uint8)
        nrm = torch.empty(1, device=dev, dtype=torch.float64)

        def check(it: int) -> bool:
            residual(matrix, b, x, r)
            _lib.check(L.gbf_norm2_f64(n, r.data_ptr(), nrm.data_ptr(), ws.data_ptr(),
                                       _lib.stream_ptr(dev)), "gbf_norm2_f64")
            return monitor.check(float(nrm.item()), it)

        if check(0):
            return x, monitor.build_info(converged=True)
        pre = None
        if self._smoother == "DIC":
            pre = DICPreconditioner(matrix)
        elif self._smoother == "DILU":
            pre = DILUPreconditioner(matrix)
        for i in range(1, max_iter + 1):
            for _ in range(self._n_sweeps):
                if pre is None:
                    gs_sweep(matrix, x, b)
                else:
                    residual(matrix, b, x, r)
                    relax(x, pre.apply_full(r), self._omega)
            if check(i):
                return x, monitor.build_info(converged=True)
        return x, monitor.build_info(converged=False)
