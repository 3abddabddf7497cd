"""Preconditioned bi-conjugate gradient on the GPU, drop-in for
``pyfoam.solvers.pbicg.PBiCGSolver`` (``src/pyfoam/solvers/pbicg.py:40-220``).

The reference's recurrence, step for step (including its shadow update
r~ -= alpha A^T p with the primal direction p): every matrix product is the
bitwise reference ``Ax`` / ``Ax_T`` gather, the preconditioner the DIC/DILU
diagonal apply, vector updates ``gbf_xpay_f64`` and the dot products and
residual norms deterministic device reductions.  The host reads rho, the
breakdown denominators and the residual each iteration, as the reference does.
"""

from __future__ import annotations

import torch

from .. import _lib
from ..core.ldu_matrix import LduMatrix
from .linear_solver import LinearSolverBase
from .preconditioners import DICPreconditioner, DILUPreconditioner, Preconditioner
from .residual import ConvergenceInfo, ResidualMonitor
from .smoothers import residual

__all__ = ["PBiCGSolver"]


class PBiCGSolver(LinearSolverBase):
    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, max_iter: int = 1000,
                 min_iter: int = 0, verbose: bool = False, preconditioner: str = "DILU") -> None:
        super().__init__(tolerance=tolerance, rel_tol=rel_tol, max_iter=max_iter,
                         min_iter=min_iter, verbose=verbose)
        self._precond_type = preconditioner.upper()

    def _make_preconditioner(self, matrix: LduMatrix) -> Preconditioner | None:
        if self._precond_type == "DILU":
            return DILUPreconditioner(matrix)
        if self._precond_type == "DIC":
            return DICPreconditioner(matrix)
        if self._precond_type == "NONE":
            return None
        raise ValueError(f"Unknown preconditioner '{self._precond_type}'. "
                         f"Use 'DILU', 'DIC', or 'none'.")

    def _solve(self, matrix: LduMatrix, source: torch.Tensor, x0: torch.Tensor,
               monitor: ResidualMonitor, max_iter: int) -> tuple[torch.Tensor, ConvergenceInfo]:
        if matrix.dtype != torch.float64:
            raise TypeError("PBiCGSolver runs on float64 matrices")
        dev, n = matrix.device, matrix.n_cells
        b = source.to(device=dev, dtype=torch.float64).contiguous()
        x = x0.to(device=dev, dtype=torch.float64).clone().contiguous()
        if b.shape[0] != n or x.shape[0] != n:
            raise ValueError(f"source/x0 have {b.shape[0]}/{x.shape[0]} elements, expected {n}")
        L = _lib.lib()
        st = _lib.stream_ptr(dev)
        ws = torch.empty(int(L.gbf_norm2_workspace_bytes()), device=dev, dtype=torch.uint8)
        sc = torch.empty(1, device=dev, dtype=torch.float64)
        pre = self._make_preconditioner(matrix)

        def norm(v) -> float:
            _lib.check(L.gbf_norm2_f64(n, v.data_ptr(), sc.data_ptr(), ws.data_ptr(), st),
                       "gbf_norm2_f64")
            return float(sc.item())

        def dot(a, c) -> float:
            _lib.check(L.gbf_dot_f64(n, a.data_ptr(), c.data_ptr(), sc.data_ptr(), ws.data_ptr(),
                                     st), "gbf_dot_f64")
            return float(sc.item())

        def xpay(xv, a, yv, out):
            _lib.check(L.gbf_xpay_f64(n, xv.data_ptr(), float(a), yv.data_ptr(), out.data_ptr(),
                                      st), "gbf_xpay_f64")

        def apply(v):
            return pre.apply(v) if pre is not None else v.clone()

        r = residual(matrix, b, x)
        if monitor.check(norm(r), 0):
            return x, monitor.build_info(converged=True)
        rt = r.clone()
        z, zt = apply(r), apply(rt)
        p = z.clone()
        rho = dot(zt, r)
        for i in range(1, max_iter + 1):
            if abs(rho) < 1e-30:
                return x, monitor.build_info(converged=False)
            v = matrix.Ax(p)
            ztv = dot(zt, v)
            if abs(ztv) < 1e-30:
                return x, monitor.build_info(converged=False)
            alpha = rho / ztv
            xpay(x, alpha, p, x)
            xpay(r, -alpha, v, r)
            if monitor.check(norm(r), i):
                return x, monitor.build_info(converged=True)
            z = apply(r)
            xpay(rt, -alpha, matrix.Ax_T(p), rt)
            zt = apply(rt)
            rho_new = dot(zt, r)
            beta = rho_new / rho
            rho = rho_new
            xpay(z, beta, p, p)
        return x, monitor.build_info(converged=False)
