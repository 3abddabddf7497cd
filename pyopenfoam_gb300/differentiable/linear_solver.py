"""Differentiable linear solve, drop-in for
``pyfoam.differentiable.linear_solver.DifferentiableLinearSolve``
(``src/pyfoam/differentiable/linear_solver.py:26-151``).

Forward: x = A^-1 b with any solver of this package.  Backward (implicit
function theorem): the adjoint system A^T lam = dL/dx is solved with the same
solver on the transposed matrix (lower and upper swapped), then
dL/db = lam, dL/ddiag = -lam*x, dL/dlower_f = -lam[own]*x[nei],
dL/dupper_f = -lam[nei]*x[own] come from one kernel (``gbf_dls_grads_f64``).
As in the reference, the backward solve uses the forward's tolerance and
iteration limit with the solver's own ``rel_tol``.
"""

from __future__ import annotations

from typing import Any

import torch

from .. import _lib
from ..core.ldu_matrix import LduMatrix

__all__ = ["DifferentiableLinearSolve", "dls_grads"]


def dls_grads(matrix: LduMatrix, lam: torch.Tensor, x: torch.Tensor):
    """(dL/ddiag, dL/dlower, dL/dupper) from the adjoint lam and solution x."""
    n, nf = matrix.n_cells, matrix.n_internal_faces
    dev = matrix.device
    topo = matrix.topology()
    gd = torch.empty(max(n, 1), device=dev, dtype=torch.float64)
    gl = torch.empty(max(nf, 1), device=dev, dtype=torch.float64)
    gu = torch.empty(max(nf, 1), device=dev, dtype=torch.float64)
    lam = lam.to(device=dev, dtype=torch.float64).contiguous()
    x = x.to(device=dev, dtype=torch.float64).contiguous()
    _lib.check(_lib.lib().gbf_dls_grads_f64(topo.layout_ref, lam.data_ptr(), x.data_ptr(),
                                            gd.data_ptr(), gl.data_ptr(), gu.data_ptr(),
                                            _lib.stream_ptr(dev)), "gbf_dls_grads_f64")
    return gd[:n], gl[:nf], gu[:nf]


class DifferentiableLinearSolve(torch.autograd.Function):
    """``DifferentiableLinearSolve.apply(A_diag, A_lower, A_upper, b, solver,
    owner, neighbour, x0, tolerance=1e-6, max_iter=1000) -> x``; backward
    returns 10 gradients (None for the non-tensor inputs)."""

    @staticmethod
    def forward(ctx: Any, A_diag: torch.Tensor, A_lower: torch.Tensor, A_upper: torch.Tensor,
                b: torch.Tensor, solver: Any, owner: torch.Tensor, neighbour: torch.Tensor,
                x0: torch.Tensor, tolerance: float = 1e-6, max_iter: int = 1000) -> torch.Tensor:
        n_cells = A_diag.shape[0]
        matrix = LduMatrix(n_cells, owner, neighbour, device=A_diag.device, dtype=A_diag.dtype)
        matrix.diag = A_diag.detach()
        matrix.lower = A_lower.detach()
        matrix.upper = A_upper.detach()
        x, _, _ = solver(matrix, b.detach(), x0.detach(), tolerance, max_iter)
        ctx.save_for_backward(A_diag, A_lower, A_upper, x, owner, neighbour)
        ctx.solver = solver
        ctx.tolerance = tolerance
        ctx.max_iter = max_iter
        ctx.n_cells = n_cells
        return x

    @staticmethod
    def backward(ctx: Any, grad_output: torch.Tensor) -> tuple:
        A_diag, A_lower, A_upper, x, owner, neighbour = ctx.saved_tensors
        n = ctx.n_cells
        dev, dt = grad_output.device, grad_output.dtype
        matrix_T = LduMatrix(n, owner, neighbour, device=dev, dtype=dt)
        matrix_T.diag = A_diag.detach()
        matrix_T.lower = A_upper.detach()  # transpose: lower' = upper
        matrix_T.upper = A_lower.detach()  # upper' = lower
        lam, _, _ = ctx.solver(matrix_T, grad_output.contiguous(),
                               torch.zeros(n, device=dev, dtype=dt), ctx.tolerance, ctx.max_iter)
        gd, gl, gu = dls_grads(matrix_T, lam, x)
        return gd, gl, gu, lam, None, None, None, None, None, None
