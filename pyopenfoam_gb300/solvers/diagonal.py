"""Diagonal solver on the GPU, drop-in for ``pyfoam.solvers.diagonal.
DiagonalSolver`` (``src/pyfoam/solvers/diagonal.py:25-85``): x = b /
max(|diag|, 1e-30) in one kernel (``gbf_diagonal_solve_f64``), the residual
b - diag x reported through the monitor, always "converged" after the single
iteration-0 check, as in the reference."""

from __future__ import annotations

import torch

from .. import _lib
from ..core.ldu_matrix import LduMatrix
from .linear_solver import LinearSolverBase
from .residual import ConvergenceInfo, ResidualMonitor

__all__ = ["DiagonalSolver"]


class DiagonalSolver(LinearSolverBase):
    def _solve(self, matrix: LduMatrix, source: torch.Tensor, x0: torch.Tensor,
               monitor: ResidualMonitor, max_iter: int) -> tuple[torch.Tensor, ConvergenceInfo]:
        if matrix.dtype != torch.float64:
            raise TypeError("DiagonalSolver runs on float64 matrices")
        dev, n = matrix.device, matrix.n_cells
        b = source.to(device=dev, dtype=torch.float64).contiguous()
        if b.shape[0] != n:
            raise ValueError(f"source has {b.shape[0]} elements, expected {n}")
        x = torch.empty_like(b)
        r = torch.empty_like(b)
        L = _lib.lib()
        st = _lib.stream_ptr(dev)
        _lib.check(L.gbf_diagonal_solve_f64(n, matrix.diag.data_ptr(), b.data_ptr(), x.data_ptr(),
                                            r.data_ptr(), st), "gbf_diagonal_solve_f64")
        ws = torch.empty(int(L.gbf_norm2_workspace_bytes()), device=dev, dtype=torch.uint8)
        nrm = torch.empty(1, device=dev, dtype=torch.float64)
        _lib.check(L.gbf_norm2_f64(n, r.data_ptr(), nrm.data_ptr(), ws.data_ptr(), st),
                   "gbf_norm2_f64")
        monitor.check(float(nrm.item()), 0)
        return x, monitor.build_info(converged=True)
