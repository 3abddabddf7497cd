"""Mixed-precision refined PCG (FP32 inner iterations, FP64 reliable
updates) with the reference solver interface.

There is no reference counterpart: this is the precision pattern of the
build's target -- FP32 Amul, preconditioner and Krylov vectors; FP64 for the
outer residual b - A x, the solution update and the dot-product
reductions.  The FP32 recurrence is periodically re-anchored to the true FP64
residual (reliable updates, Sleijpen & van der Vorst 1996) while the search
direction is kept, so the iteration count stays close to FP64 PCG and the
final accuracy is FP64's.  Convergence uses ResidualMonitor's rules on the
true residual; ``iterations`` counts inner iterations plus the
iteration-0 check, and ``last_info.residual_history`` holds the true residual
at every update.
"""

from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ..core.device import to_device
from ..core.ldu_matrix import LduMatrix
from .linear_solver import LinearSolverBase
from .preconditioners import DICPreconditioner, DILUPreconditioner, Preconditioner
from .residual import ConvergenceInfo, ResidualMonitor

__all__ = ["MixedPrecisionPCGSolver", "MixedPrecisionPBiCGSTABSolver"]


class MixedPrecisionPCGSolver(LinearSolverBase):
    """PCG with FP32 inner iterations and FP64 reliable updates.

    ``delta`` (keyword only) is the residual reduction between FP64 updates.
    ``symmetric_storage`` (keyword only, default False): when the matrix is
    symmetric bit for bit and its layout allows it, the FP32 inner Amul
    reads only the owner-side half of the off-diagonals (same results, 35 %
    fewer DRAM bytes, but three more gathered loads per cell: on GB300 at
    256^3 the kernel is then latency-bound and slower, 139.6 vs 121.8 us per
    launch, so it is off by default)."""

    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, max_iter: int = 1000,
                 min_iter: int = 0, verbose: bool = False, preconditioner: str = "DIC", *,
                 delta: float = 0.1, check_every: int = 32,
                 symmetric_storage: bool = False) -> None:
        super().__init__(tolerance=tolerance, rel_tol=rel_tol, max_iter=max_iter,
                         min_iter=min_iter, verbose=verbose)
        self._precond_type = preconditioner.upper()
        if not 0.0 < delta < 1.0:
            raise ValueError(f"delta must be in (0, 1), got {delta}")
        self._delta = float(delta)
        self._check_every = int(check_every)
        self._symmetric_storage = bool(symmetric_storage)
        self.last_result: _lib.SolveResult | None = None

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
        if matrix.dtype != torch.float64:
            raise TypeError("MixedPrecisionPCGSolver takes the float64 matrix and makes its "
                            f"own FP32 copy (got {matrix.dtype})")
        dev = matrix.device
        n = matrix.n_cells
        if source.shape[0] != n or x0.shape[0] != n:
            raise ValueError(f"source/x0 have {source.shape[0]}/{x0.shape[0]} elements, "
                             f"expected {n}")
        b = to_device(source, dev, torch.float64)
        x = x0.to(device=dev, dtype=torch.float64).clone().contiguous()
        precond = self._make_preconditioner(matrix)
        pd = None if precond is None else precond.precond_diag
        topo = matrix.topology()
        coef64 = matrix.packed()
        # symmetric matrices: the inner Amul streams only the owner-side half
        coef32 = matrix.packed_sym32() if self._symmetric_storage else None
        sym = coef32 is not None
        if not sym:
            coef32 = matrix.packed(dtype=torch.float32)
        L = _lib.lib()
        cap = 4096
        hist = torch.zeros(cap, device=dev, dtype=torch.float64)
        ws = torch.empty(max(int(L.gbf_mixed_pcg_workspace_bytes(n)), 1), device=dev,
                         dtype=torch.uint8)
        P = _lib.SolveParams(float(monitor.tolerance), float(monitor.rel_tol), int(max_iter),
                             int(monitor.min_iter), self._check_every, 0)
        R = _lib.SolveResult()
        _lib.check(
            L.gbf_mixed_pcg_solve(topo.layout_ref, coef64.data_ptr(), matrix.diag.data_ptr(),
                                  coef32.data_ptr(), int(sym),
                                  None if pd is None else pd.data_ptr(),
                                  b.data_ptr(), x.data_ptr(), self._delta, hist.data_ptr(), cap,
                                  ctypes.byref(P), ctypes.byref(R), ws.data_ptr(), ws.numel(),
                                  _lib.stream_ptr(dev)),
            "gbf_mixed_pcg_solve",
        )
        self.last_result = R
        if R.status == _lib.GBF_DEVICE_TIMEOUT:
            raise RuntimeError("gbf_mixed_pcg_solve: a bounded wait on a staged copy ran out "
                               "inside the Amul kernel; the result is invalid")
        nh = min(R.outer_updates + 1, cap) if n > 0 else 1
        monitor.record(hist[:nh].tolist() if n > 0 else [0.0])
        info = monitor.build_info(converged=(R.status == _lib.GBF_CONVERGED))
        info.iterations = R.iterations
        info.final_residual = R.final_residual
        return x, info


class MixedPrecisionPBiCGSTABSolver(LinearSolverBase):
    """PBiCGStab with FP32 inner iterations and FP64 reliable updates, for
    the asymmetric momentum solve.

    The iteration and its breakdown tests are those of ``PBiCGSTABSolver``
    (solvers/pbicgstab.py:103-239); the vectors, the Amul and the diagonal
    DILU/DIC preconditioner run in FP32, and the FP32 correction is folded
    into the FP64 solution (with the residual replaced by the true
    b - A x) whenever the iterated residual has dropped by ``delta``.
    Convergence is checked on the true residual only, once per update, so
    the half-step check on s is not taken.  ``omega`` (keyword only):
    ``"standard"`` (default here) takes (t.s)/(t.t); ``"reference"`` takes
    the reference's (t.z)/(t.t).  ``form`` (keyword only): ``"persistent"``
    runs the whole inner loop in one cooperative launch, ``"kernels"`` six
    launches per iteration (bulk-copy staged Amul on hex layouts),
    ``"gather"`` the same with the plain L2 gather Amul, ``"fused"`` three
    kernels per iteration (one per reduction: the p update folded into the
    next v = A y, the s / z update into t = A z; hex 3+3 layouts, others run
    the gather kernels); ``"auto"`` takes
    the persistent form up to 2^16 cells, the fused form up to 2^19, the
    gather kernels up to 2^22 and the staged kernels above (the fastest in a
    sweep of the forms on GB300)."""

    FORMS = {"auto": 0, "kernels": 1, "gather": 2, "persistent": 3, "fused": 4}

    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, max_iter: int = 1000,
                 min_iter: int = 0, verbose: bool = False, preconditioner: str = "DILU", *,
                 omega: str = "standard", delta: float = 0.1, check_every: int = 32,
                 form: str = "auto") -> None:
        super().__init__(tolerance=tolerance, rel_tol=rel_tol, max_iter=max_iter,
                         min_iter=min_iter, verbose=verbose)
        self._precond_type = preconditioner.upper()
        if omega not in ("reference", "standard"):
            raise ValueError(f"omega must be 'reference' or 'standard', got {omega!r}")
        if not 0.0 < delta < 1.0:
            raise ValueError(f"delta must be in (0, 1), got {delta}")
        if form not in self.FORMS:
            raise ValueError(f"form must be one of {sorted(self.FORMS)}, got {form!r}")
        self._omega = omega
        self._form = form
        self._delta = float(delta)
        self._check_every = int(check_every)
        self.last_result: _lib.SolveResult | None = None

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
        if matrix.dtype != torch.float64:
            raise TypeError("MixedPrecisionPBiCGSTABSolver takes the float64 matrix and makes "
                            f"its own FP32 copy (got {matrix.dtype})")
        dev = matrix.device
        n = matrix.n_cells
        if source.shape[0] != n or x0.shape[0] != n:
            raise ValueError(f"source/x0 have {source.shape[0]}/{x0.shape[0]} elements, "
                             f"expected {n}")
        b = to_device(source, dev, torch.float64)
        x = x0.to(device=dev, dtype=torch.float64).clone().contiguous()
        precond = self._make_preconditioner(matrix)
        pd = None if precond is None else precond.precond_diag
        topo = matrix.topology()
        coef64 = matrix.packed()
        coef32 = matrix.packed(dtype=torch.float32)
        L = _lib.lib()
        cap = 4096
        hist = torch.zeros(cap, device=dev, dtype=torch.float64)
        ws = torch.empty(max(int(L.gbf_mixed_pbicgstab_workspace_bytes(n)), 1), device=dev,
                         dtype=torch.uint8)
        P = _lib.SolveParams(float(monitor.tolerance), float(monitor.rel_tol), int(max_iter),
                             int(monitor.min_iter), self._check_every,
                             (1 if self._omega == "standard" else 0)
                             | (self.FORMS[self._form] << 1))
        R = _lib.SolveResult()
        _lib.check(
            L.gbf_mixed_pbicgstab_solve(topo.layout_ref, coef64.data_ptr(),
                                        matrix.diag.data_ptr(), coef32.data_ptr(),
                                        None if pd is None else pd.data_ptr(), b.data_ptr(),
                                        x.data_ptr(), self._delta, hist.data_ptr(), cap,
                                        ctypes.byref(P), ctypes.byref(R), ws.data_ptr(),
                                        ws.numel(), _lib.stream_ptr(dev)),
            "gbf_mixed_pbicgstab_solve",
        )
        self.last_result = R
        if R.status == _lib.GBF_DEVICE_TIMEOUT:
            raise RuntimeError("gbf_mixed_pbicgstab_solve: a bounded wait (a staged copy in the "
                               "Amul kernel, or a grid barrier of the persistent form) ran out; "
                               "the result is invalid")
        nh = min(R.outer_updates + 1, cap) if n > 0 else 1
        monitor.record(hist[:nh].tolist() if n > 0 else [0.0])
        info = monitor.build_info(converged=(R.status == _lib.GBF_CONVERGED))
        info.iterations = R.iterations
        info.final_residual = R.final_residual
        return x, info
