"""Smoothers on the GPU, drop-in for ``pyfoam.solvers.smoothers``
(``src/pyfoam/solvers/smoothers.py:45-260``): ``GaussSeidelSmoother``
(forward + backward relaxed sweeps), ``JacobiSmoother`` (damped Jacobi) and
``DICGSmoother`` (residual, full DIC solve, relaxed update), each with the
reference's ``smooth(x, b, n_iterations)`` interface.

The reference loops over cells (and, inside, over every face) in Python.
Here a Gauss-Seidel sweep is a level-scheduled wavefront of libgbfoam
kernels (``gbf_gauss_seidel_f64``) that keeps the sequential loop's update
order and each row's face order, so the sweeps are bitwise the reference's;
Jacobi and DICG are a residual kernel, the full DIC sweeps and a relaxation
kernel.
"""

from __future__ import annotations

import ctypes
from typing import Protocol

import numpy as np
import torch

from .. import _lib
from ..core.ldu_matrix import LduMatrix
from .preconditioners import DICPreconditioner

__all__ = ["Smoother", "GaussSeidelSmoother", "JacobiSmoother", "DICGSmoother", "gs_sweep",
           "residual"]


class Smoother(Protocol):
    def smooth(self, x: torch.Tensor, b: torch.Tensor, n_iterations: int) -> torch.Tensor: ...


def _f64(matrix: LduMatrix, v: torch.Tensor, name: str) -> torch.Tensor:
    if matrix.dtype != torch.float64:
        raise TypeError("the smoothers run on float64 matrices")
    t = torch.as_tensor(v).to(device=matrix.device, dtype=torch.float64).contiguous()
    if t.shape[0] != matrix.n_cells:
        raise ValueError(f"{name} has {t.shape[0]} elements, expected {matrix.n_cells}")
    return t


class _GsSchedule:
    """Device and host copies of one Gauss-Seidel level schedule."""

    def __init__(self, topo, reverse: bool) -> None:
        n = topo.n_cells
        ptr = np.empty(n + 1, np.int32)
        cells = np.empty(max(n, 1), np.int32)
        nl, mx = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(_lib.lib().gbf_gs_schedule(n, topo.n_faces, topo._own_h.ctypes.data,
                                              topo._nei_h.ctypes.data, int(reverse),
                                              ptr.ctypes.data, cells.ctypes.data,
                                              ctypes.byref(nl), ctypes.byref(mx)),
                   "gbf_gs_schedule")
        self.n_levels = nl.value
        self.ptr_h = np.ascontiguousarray(ptr[: nl.value + 1])
        self.ptr = torch.from_numpy(self.ptr_h.copy()).to(topo.device)
        self.cells = torch.from_numpy(cells).to(topo.device)


def _gs_schedule(matrix: LduMatrix, reverse: bool) -> _GsSchedule:
    topo = matrix.topology()
    cache = topo.__dict__.setdefault("_gs", {})
    if reverse not in cache:
        cache[reverse] = _GsSchedule(topo, reverse)
    return cache[reverse]


#: How a Gauss-Seidel sweep walks its level schedule (the same bits):
#: "flow" -- one cooperative launch in which a cell waits only on the new
#: values it reads (gbf_gauss_seidel_flow_f64); "levels" -- one cooperative
#: launch with a grid barrier per level; "per_level" -- a launch per level.
GS_FORMS = ("flow", "levels", "per_level")


def gs_sweep(matrix: LduMatrix, x: torch.Tensor, b: torch.Tensor, reverse: bool = False,
             omega: float = 1.0, relax: bool = False, form: str = "flow") -> None:
    """One Gauss-Seidel sweep over x in place: cells ascending (or
    descending with ``reverse``); ``relax`` uses x_c += omega (new - x_c)
    (GaussSeidelSmoother), otherwise x_c = new (SmoothSolver).  If a bounded
    wait of a cooperative form runs out, x becomes NaN."""
    if form not in GS_FORMS:
        raise ValueError(f"form must be one of {GS_FORMS}, got {form!r}")
    sch = _gs_schedule(matrix, reverse)
    topo = matrix.topology()
    coef = matrix.packed()
    st = _lib.stream_ptr(matrix.device)
    if form == "flow":
        scratch = torch.empty(max(matrix.n_cells, 1), dtype=torch.float64, device=matrix.device)
        _lib.check(_lib.lib().gbf_gauss_seidel_flow_f64(
            topo.layout_ref, coef.data_ptr(), matrix.diag.data_ptr(), b.data_ptr(),
            sch.cells.data_ptr(), int(reverse), float(omega), int(relax), x.data_ptr(),
            scratch.data_ptr(), _lib.wavefront_barrier(matrix.device).data_ptr(), st),
            "gbf_gauss_seidel_flow_f64")
        return
    bar = _lib.wavefront_barrier(matrix.device) if form == "levels" else None
    _lib.check(_lib.lib().gbf_gauss_seidel_f64(
        topo.layout_ref, coef.data_ptr(), matrix.diag.data_ptr(), b.data_ptr(), sch.ptr.data_ptr(),
        sch.cells.data_ptr(), sch.ptr_h.ctypes.data, sch.n_levels, float(omega), int(relax),
        x.data_ptr(), None if bar is None else bar.data_ptr(), st), "gbf_gauss_seidel_f64")


def residual(matrix: LduMatrix, b: torch.Tensor, x: torch.Tensor,
             out: torch.Tensor | None = None) -> torch.Tensor:
    """r = b - A x with A x bitwise ``LduMatrix.Ax``."""
    r = torch.empty_like(x) if out is None else out
    topo = matrix.topology()
    _lib.check(_lib.lib().gbf_residual_f64(topo.layout_ref, matrix.packed().data_ptr(),
                                           matrix.diag.data_ptr(), b.data_ptr(), x.data_ptr(),
                                           r.data_ptr(), _lib.stream_ptr(matrix.device)),
               "gbf_residual_f64")
    return r


def relax(x: torch.Tensor, z: torch.Tensor, omega: float, diag: torch.Tensor | None = None) -> None:
    """x += (omega / max(|diag|, 1e-30)) z, or x += omega z, in place."""
    _lib.check(_lib.lib().gbf_relax_f64(x.shape[0], float(omega),
                                        None if diag is None else diag.data_ptr(), z.data_ptr(),
                                        x.data_ptr(), _lib.stream_ptr(x.device)), "gbf_relax_f64")


class GaussSeidelSmoother:
    """Symmetric Gauss-Seidel: per iteration a forward then a backward
    relaxed sweep (smoothers.py:63-149)."""

    def __init__(self, matrix: LduMatrix, omega: float = 1.0) -> None:
        self._matrix = matrix
        self._omega = omega

    def smooth(self, x: torch.Tensor, b: torch.Tensor, n_iterations: int) -> torch.Tensor:
        m = self._matrix
        x = _f64(m, x, "x").clone()
        b = _f64(m, b, "b")
        for _ in range(n_iterations):
            gs_sweep(m, x, b, reverse=False, omega=self._omega, relax=True)
            gs_sweep(m, x, b, reverse=True, omega=self._omega, relax=True)
        return x


class JacobiSmoother:
    """Damped Jacobi, x += omega D^-1 (b - A x) (smoothers.py:152-200)."""

    def __init__(self, matrix: LduMatrix, omega: float = 2.0 / 3.0) -> None:
        self._matrix = matrix
        self._omega = omega

    def smooth(self, x: torch.Tensor, b: torch.Tensor, n_iterations: int) -> torch.Tensor:
        m = self._matrix
        x = _f64(m, x, "x").clone()
        b = _f64(m, b, "b")
        r = torch.empty_like(x)
        for _ in range(n_iterations):
            residual(m, b, x, r)
            relax(x, r, self._omega, m.diag)
        return x


class DICGSmoother:
    """x += omega DIC^-1 (b - A x) with the full DIC solve
    (smoothers.py:203-260)."""

    def __init__(self, matrix: LduMatrix, omega: float = 1.0) -> None:
        self._matrix = matrix
        self._omega = omega
        self._dic = DICPreconditioner(matrix)

    def smooth(self, x: torch.Tensor, b: torch.Tensor, n_iterations: int) -> torch.Tensor:
        m = self._matrix
        x = _f64(m, x, "x").clone()
        b = _f64(m, b, "b")
        r = torch.empty_like(x)
        for _ in range(n_iterations):
            residual(m, b, x, r)
            relax(x, self._dic.apply_full(r), self._omega)
        return x
