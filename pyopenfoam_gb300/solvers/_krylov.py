"""Shared plumbing of the GPU Krylov solvers: workspace, parameter blocks and
the hand-back of the device residual history to the ResidualMonitor."""

from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ..core.device import to_device
from ..core.ldu_matrix import LduMatrix
from .residual import ConvergenceInfo, ResidualMonitor

__all__ = ["run_solver"]


def run_solver(fn_name: str, ws_name: str, matrix: LduMatrix, source: torch.Tensor,
               x0: torch.Tensor, monitor: ResidualMonitor, max_iter: int,
               precond_diag: torch.Tensor | None, hist_len: int, check_every: int,
               variant: int = 0) -> tuple[torch.Tensor, ConvergenceInfo, _lib.SolveResult]:
    if matrix.dtype != torch.float64:
        raise TypeError(
            f"{fn_name}: the reference-faithful solvers run on float64 matrices "
            f"(got {matrix.dtype}); use MixedPrecisionPCGSolver for FP32 inner iterations"
        )
    if max_iter < 0:
        raise ValueError(f"max_iter must be >= 0, got {max_iter}")
    dev = matrix.device
    n = matrix.n_cells
    if source.shape[0] != n or x0.shape[0] != n:
        raise ValueError(
            f"source/x0 have {source.shape[0]}/{x0.shape[0]} elements, expected {n}"
        )
    b = to_device(source, dev, torch.float64)
    x = x0.to(device=dev, dtype=torch.float64).clone().contiguous()
    topo = matrix.topology()
    coef = matrix.packed()
    L = _lib.lib()
    hist = torch.zeros(max(hist_len, 1), device=dev, dtype=torch.float64)
    ws = torch.empty(max(int(getattr(L, ws_name)(n)), 1), device=dev, dtype=torch.uint8)
    P = _lib.SolveParams(float(monitor.tolerance), float(monitor.rel_tol), int(max_iter),
                         int(monitor.min_iter), int(check_every), int(variant))
    R = _lib.SolveResult()
    _lib.check(
        getattr(L, fn_name)(topo.layout_ref, coef.data_ptr(), matrix.diag.data_ptr(),
                            None if precond_diag is None else precond_diag.data_ptr(),
                            b.data_ptr(), x.data_ptr(), hist.data_ptr(), ctypes.byref(P),
                            ctypes.byref(R), ws.data_ptr(), ws.numel(), _lib.stream_ptr(dev)),
        fn_name,
    )
    if R.status == _lib.GBF_DEVICE_TIMEOUT:
        raise RuntimeError(f"{fn_name}: a bounded wait inside the solver kernel ran out; "
                           "the result is invalid")
    if R.iterations > 0 and n > 0:
        monitor.record(hist[: R.iterations].tolist())
    else:
        monitor.record([0.0] * max(R.iterations, 0))
    info = monitor.build_info(converged=(R.status == _lib.GBF_CONVERGED))
    return x, info, R
