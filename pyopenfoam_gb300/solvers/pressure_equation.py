"""Pressure-equation caller of the linear solve, drop-in for
``pyfoam.solvers.pressure_equation`` (``assemble_pressure_equation``,
``solve_pressure_equation``, ``correct_velocity``, ``correct_face_flux`` and
``adjust_phi``, ``src/pyfoam/solvers/pressure_equation.py:49-377``).

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

``correct_velocity`` (U = HbyA - alpha/|A_p| grad p, Gauss gradient),
``correct_face_flux`` (phi += (1/A_p)_f (p_P - p_N) |S_f| delta_f) and
``adjust_phi`` run as libgbfoam face / cell kernels (``csrc/pressure.cu``),
bitwise the reference's except adjust_phi's boundary-flux sum, which is a
deterministic tree sum.
"""

from __future__ import annotations

from typing import Any

import torch

from .. import _lib
from ..core.fv_matrix import FvMatrix
from ..discretisation.operators import _make_fvmatrix, mesh_data
from .linear_solver import LinearSolverBase

__all__ = ["assemble_pressure_equation", "solve_pressure_equation", "correct_velocity",
           "correct_face_flux", "adjust_phi"]


def _f64(t: torch.Tensor, dev, n: int | None = None, name: str = "") -> torch.Tensor:
    v = torch.as_tensor(t).detach().to(device=dev, dtype=torch.float64).contiguous()
    if n is not None and v.shape[0] != n:
        raise ValueError(f"{name} has {v.shape[0]} rows, expected {n}")
    return v


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


def correct_velocity(U: torch.Tensor, HbyA: torch.Tensor, p: torch.Tensor, A_p: torch.Tensor,
                     mesh: Any, alpha: float = 1.0) -> torch.Tensor:
    """U = HbyA - alpha/|A_p| grad(p) with |U| limited to 1e4
    (pressure_equation.py:187-266); returns a new (n_cells, 3) tensor."""
    md = mesh_data(mesh)
    dev, n = md.device, md.n_cells
    topo = md.topology()
    H = _f64(HbyA, dev, n, "HbyA").reshape(n, 3)
    pp, A = _f64(p, dev, n, "p"), _f64(A_p, dev, n, "A_p")
    w = _f64(mesh.face_weights, dev)
    out = torch.empty(n, 3, device=dev, dtype=torch.float64)
    _lib.check(_lib.lib().gbf_correct_velocity_f64(
        topo.layout_ref, md.bnd_ptr.data_ptr(), md.bnd_face.data_ptr(),
        md.field("face_areas").data_ptr(), w.data_ptr(), md.field("cell_volumes").data_ptr(),
        pp.data_ptr(), A.data_ptr(), H.data_ptr(), float(alpha), out.data_ptr(),
        _lib.stream_ptr(dev)), "gbf_correct_velocity_f64")
    return out


def correct_face_flux(phi: torch.Tensor, p: torch.Tensor, A_p: torch.Tensor, mesh: Any,
                      face_weights: torch.Tensor | None = None) -> torch.Tensor:
    """phi + (1/A_p)_f (p_P - p_N) |S_f| delta_f on internal faces
    (pressure_equation.py:269-332); returns a new tensor."""
    md = mesh_data(mesh)
    dev = md.device
    topo = md.topology()
    ph = _f64(phi, dev, md.n_faces, "phi")
    from .rhie_chow import inv_abs_clamped

    pp = _f64(p, dev, md.n_cells, "p")
    A = inv_abs_clamped(_f64(A_p, dev, md.n_cells, "A_p"))
    w = _f64(mesh.face_weights if face_weights is None else face_weights, dev)
    out = torch.empty_like(ph)
    _lib.check(_lib.lib().gbf_rhie_chow_f64(
        md.n_faces, md.n_internal, md.owner_all32.data_ptr(), topo.neighbour32.data_ptr(),
        pp.data_ptr(), A.data_ptr(), md.field("face_areas").data_ptr(),
        md.field("delta_coefficients").data_ptr(), w.data_ptr(), ph.data_ptr(), out.data_ptr(),
        _lib.stream_ptr(dev)), "gbf_rhie_chow_f64")
    return out


def adjust_phi(phi: torch.Tensor, mesh: Any, closed: bool = True) -> bool:
    """Removes the net boundary flux of a closed domain from its boundary
    faces, in place (pressure_equation.py:335-377); True if it did."""
    nint, nf = int(mesh.n_internal_faces), int(mesh.n_faces)
    if nf <= nint or not closed:
        return False
    if phi.device.type != "cuda" or phi.dtype != torch.float64 or not phi.is_contiguous():
        raise ValueError("adjust_phi works in place on a contiguous float64 CUDA tensor")
    dev = phi.device
    s = torch.empty(1, device=dev, dtype=torch.float64)
    L = _lib.lib()
    _lib.check(L.gbf_boundary_flux_sum_f64(nf, nint, phi.data_ptr(), s.data_ptr(),
                                           _lib.stream_ptr(dev)), "gbf_boundary_flux_sum_f64")
    if abs(float(s.item())) < 1e-30:
        return False
    _lib.check(L.gbf_adjust_phi_f64(nf, nint, s.data_ptr(), phi.data_ptr(),
                                    _lib.stream_ptr(dev)), "gbf_adjust_phi_f64")
    return True
