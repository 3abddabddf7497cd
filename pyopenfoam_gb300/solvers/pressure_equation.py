"""Pressure-equation caller of the linear solve, drop-in for
``pyfoam.solvers.pressure_equation`` (``assemble_pressure_equation`` and
``solve_pressure_equation``, ``src/pyfoam/solvers/pressure_equation.py:49-184``).

``assemble_pressure_equation(phiHbyA, A_p, mesh, face_weights=None)`` builds
laplacian(1/A_p, p) = div(phiHbyA) in per-unit-volume form on the GPU in
one call (``gbf_pressure_assemble_f64``): 1/max(|A_p|, 1e-30) per cell,
linearly interpolated to the faces with ``face_weights`` (default: the
mesh's ``face_weights``, else the distance weights of its centres), face
coefficient ((1/A_p)_f |S_f|) delta_f, lower/upper = -coeff/V, a diagonal
without boundary term, and the source -div(phiHbyA)/V -- the reference's
roundings and summation order, so the matrix and source are bitwise its own.

``solve_pressure_equation`` pins the reference cell with the reference's
1e10 * max(|diag|, 1) penalty and solves with any solver of this package.
"""

from __future__ import annotations

from typing import Any

import torch

from .. import _lib
from ..core.fv_matrix import FvMatrix
from ..discretisation.operators import _make_fvmatrix, mesh_data
from .linear_solver import LinearSolverBase

__all__ = ["assemble_pressure_equation", "solve_pressure_equation"]


def assemble_pressure_equation(phiHbyA: torch.Tensor, A_p: torch.Tensor, mesh: Any,
                               face_weights: torch.Tensor | None = None) -> FvMatrix:
    md = mesh_data(mesh)
    dev = md.device
    mat = _make_fvmatrix(md)
    topo = mat.topology()
    if face_weights is None:
        face_weights = getattr(mesh, "face_weights", None)
    w = md.weights(topo) if face_weights is None else face_weights
    w = w.to(device=dev, dtype=torch.float64).contiguous()
    A = A_p.detach().to(device=dev, dtype=torch.float64).contiguous()
    phi = phiHbyA.detach().to(device=dev, dtype=torch.float64).contiguous()
    if A.shape[0] != md.n_cells:
        raise ValueError(f"A_p has {A.shape[0]} entries, expected n_cells={md.n_cells}")
    if phi.shape[0] < md.n_faces or w.shape[0] < md.n_internal:
        raise ValueError("phiHbyA needs n_faces entries and face_weights n_internal_faces")
    nint, n = md.n_internal, md.n_cells
    lower = torch.empty(max(nint, 1), device=dev, dtype=torch.float64)
    upper = torch.empty(max(nint, 1), device=dev, dtype=torch.float64)
    diag = torch.empty(max(n, 1), device=dev, dtype=torch.float64)
    source = torch.empty(max(n, 1), device=dev, dtype=torch.float64)
    _lib.check(_lib.lib().gbf_pressure_assemble_f64(
        topo.layout_ref, md.n_faces, md.bnd_ptr.data_ptr(), md.bnd_face.data_ptr(),
        md.field("face_areas").data_ptr(), md.field("delta_coefficients").data_ptr(),
        w.data_ptr(), A.data_ptr(), md.field("cell_volumes").data_ptr(), phi.data_ptr(),
        lower.data_ptr(), upper.data_ptr(), diag.data_ptr(), source.data_ptr(),
        _lib.stream_ptr(dev)), "gbf_pressure_assemble_f64")
    mat._lower, mat._upper, mat._diag = lower[:nint], upper[:nint], diag[:n]
    mat.source = source[:n]
    return mat


def solve_pressure_equation(p_eqn: FvMatrix, p: torch.Tensor, solver: LinearSolverBase,
                            tolerance: float = 1e-6, max_iter: int = 1000,
                            reference_cell: int = 0) -> tuple[torch.Tensor, int, float]:
    """Pins ``reference_cell`` to 0 and solves; returns
    ``(p_new, iterations, residual)`` (pressure_equation.py:151-184)."""
    p_eqn.set_reference(reference_cell, value=0.0)
    return p_eqn.solve(solver, p, tolerance=tolerance, max_iter=max_iter)
