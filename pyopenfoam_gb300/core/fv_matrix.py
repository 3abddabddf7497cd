"""Finite-volume matrix, drop-in for ``pyfoam.core.fv_matrix.FvMatrix``
(``src/pyfoam/core/fv_matrix.py:66-317``): an :class:`LduMatrix` plus a
source vector, under-relaxation, reference-cell pinning and ``solve``.
"""

from __future__ import annotations

from typing import Any, Protocol

import torch

from .. import _lib
from .dtype import assert_floating
from .ldu_matrix import LduMatrix

__all__ = ["FvMatrix", "LinearSolver"]


class LinearSolver(Protocol):
    """``solver(matrix, source, x0, tolerance, max_iter) -> (x, iters, res)``
    (core/fv_matrix.py:37-63)."""

    def __call__(self, matrix: LduMatrix, source: torch.Tensor, x0: torch.Tensor,
                 tolerance: float, max_iter: int) -> tuple[torch.Tensor, int, float]: ...


class FvMatrix(LduMatrix):
    def __init__(self, n_cells: int, owner: torch.Tensor, neighbour: torch.Tensor, *,
                 device=None, dtype=None) -> None:
        super().__init__(n_cells, owner, neighbour, device=device, dtype=dtype)
        self._source = torch.zeros(n_cells, device=self._device, dtype=self._dtype)
        self._field_old: torch.Tensor | None = None
        self._relaxation_factor: float = 1.0

    @property
    def source(self) -> torch.Tensor:
        return self._source

    @source.setter
    def source(self, value: torch.Tensor) -> None:
        self._source = self._coerce(value, self._n_cells, "source")

    @property
    def relaxation_factor(self) -> float:
        return self._relaxation_factor

    def add_boundary_contribution(self, bc: Any, field: torch.Tensor | None = None) -> None:
        """Adds ``bc.matrix_contributions`` (core/fv_matrix.py:139-174)."""
        if field is None:
            field = torch.zeros(self._n_cells, device=self._device, dtype=self._dtype)
        else:
            field = field.to(device=self._device, dtype=self._dtype)
        diag, source = bc.matrix_contributions(field, self._n_cells, diag=self._diag,
                                               source=self._source)
        self._diag = diag.to(device=self._device, dtype=self._dtype).contiguous()
        self._source = source.to(device=self._device, dtype=self._dtype).contiguous()
        self.invalidate_cache()

    def add_explicit_source(self, values: torch.Tensor) -> None:
        if values.dim() == 0:
            self._source = self._source + values.to(self._device)
        else:
            self._source = self._source + values.to(device=self._device, dtype=self._dtype)

    def relax(self, field_old: torch.Tensor, under_relaxation_factor: float = 1.0) -> None:
        """Implicit under-relaxation (core/fv_matrix.py:192-235):
        diag' = diag / a; source' = source + (1 - a) * diag' * field_old."""
        assert_floating(field_old, "field_old")
        if under_relaxation_factor <= 0.0 or under_relaxation_factor > 1.0:
            raise ValueError(
                f"under_relaxation_factor must be in (0, 1], got {under_relaxation_factor}"
            )
        self._field_old = field_old.to(device=self._device, dtype=self._dtype)
        self._relaxation_factor = under_relaxation_factor
        if under_relaxation_factor < 1.0:
            a = float(under_relaxation_factor)
            if self._dtype != torch.float64:
                self._diag = (self._diag / a).contiguous()
                self._source = self._source + ((1.0 - a) * self._diag * self._field_old)
            else:
                self._diag = self._diag.clone().contiguous()
                self._source = self._source.clone().contiguous()
                old = self._field_old.contiguous()
                _lib.check(_lib.lib().gbf_fv_relax_f64(
                    self._n_cells, a, 1.0 - a, self._diag.data_ptr(), self._source.data_ptr(),
                    old.data_ptr(), _lib.stream_ptr(self._device)), "gbf_fv_relax_f64")
            self.invalidate_cache()

    def set_reference(self, cell_index: int, value: float = 0.0) -> None:
        """Pin one cell with a 1e10*max(|diag|,1) penalty
        (core/fv_matrix.py:241-259)."""
        if cell_index < 0 or cell_index >= self._n_cells:
            raise ValueError(f"cell_index {cell_index} out of range [0, {self._n_cells})")
        large = self._diag[cell_index].abs().clamp(min=1.0) * 1e10
        self._diag[cell_index] += large
        self._source[cell_index] += large * value
        self.invalidate_cache()

    def solve(self, solver: LinearSolver, x0: torch.Tensor, tolerance: float = 1e-6,
              max_iter: int = 1000) -> tuple[torch.Tensor, int, float]:
        """core/fv_matrix.py:265-290."""
        assert_floating(x0, "x0")
        x0 = x0.to(device=self._device, dtype=self._dtype)
        return solver(self, self._source, x0, tolerance, max_iter)

    def residual(self, x: torch.Tensor) -> torch.Tensor:
        """r = b - A x (core/fv_matrix.py:296-305)."""
        return self._source - self.Ax(x)

    def __repr__(self) -> str:
        return (
            f"FvMatrix(n_cells={self._n_cells}, n_internal_faces={self._n_internal_faces}, "
            f"relaxation={self._relaxation_factor:.2f}, device={self._device}, dtype={self._dtype})"
        )
