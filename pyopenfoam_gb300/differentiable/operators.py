"""Differentiable explicit Laplacian, drop-in for
``pyfoam.differentiable.operators.DifferentiableLaplacian``
(``src/pyfoam/differentiable/operators.py:409-643``).

``DifferentiableLaplacian.apply(phi, D, mesh)`` returns the explicit
Laplacian div(D grad phi) per unit volume of a cell field:

* forward -- one cell-gather kernel (``gbf_explicit_laplacian_f64``) with the
  reference's face flux ((D_f (phi_N - phi_P)) |S_f|) delta_f, its per-cell
  summation order (owner-side faces, then neighbour-side faces, then the
  boundary term ((D_b |S_b|) delta_b) phi_P) and the division by the cell
  volume clamped at 1e-30, so the result is bitwise the reference's;
* backward -- the phi-gradient is the same operator applied to grad_output,
  as the reference's backward computes it (exact for uniform cell volumes);
  the D-gradient comes from one face kernel
  (``gbf_explicit_laplacian_grad_d_f64``) and is mapped back to D's shape:
  per face as is, per cell by the reference's half-to-each-side rule, a 0-d
  D as the fixed-order sum over faces.

D may be a Python number, a 0-d tensor, a per-cell tensor (linearly
interpolated to faces) or a per-face tensor (``n_faces``).  As in the
reference, D gets a gradient only when it is a tensor that requires grad.
The mesh is duck-typed like the reference's ``FvMesh`` (the attributes
``fvm.laplacian`` reads); its tensors live on a CUDA device.
"""

from __future__ import annotations

from typing import Any

import torch

from .. import _lib
from ..discretisation.operators import mesh_data

__all__ = ["DifferentiableLaplacian"]


def _resolve_d(D: Any, md) -> tuple[int, float, torch.Tensor | None, torch.Tensor | None]:
    """(mode, value, per-face D, per-cell D) as operators.py:450-466 resolves
    D: numbers and 0-d tensors are constant, n_cells entries are per cell,
    anything else per face."""
    if isinstance(D, (int, float)):
        return 0, float(D), None, None
    if not isinstance(D, torch.Tensor):
        return 0, float(torch.as_tensor(D, dtype=torch.float64)), None, None
    Dd = D.detach().to(device=md.device, dtype=torch.float64)
    if Dd.dim() == 0:
        return 0, float(Dd), None, None
    if Dd.shape[0] == md.n_cells:
        return 2, 0.0, None, Dd.contiguous()
    if Dd.dim() != 1 or Dd.shape[0] != md.n_faces:
        raise ValueError(f"D has shape {tuple(D.shape)}; expected a scalar, n_cells="
                         f"{md.n_cells} or n_faces={md.n_faces} entries")
    return 1, 0.0, Dd.contiguous(), None


def _apply(md, topo, spec, field: torch.Tensor) -> torch.Tensor:
    mode, value, d_face, d_cell = spec
    dev = md.device
    weights = md.weights(topo) if mode == 2 else None
    out = torch.empty(max(md.n_cells, 1), device=dev, dtype=torch.float64)
    ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    _lib.check(_lib.lib().gbf_explicit_laplacian_f64(
        topo.layout_ref, md.n_faces, md.bnd_ptr.data_ptr(), md.bnd_face.data_ptr(),
        md.field("face_areas").data_ptr(), md.field("delta_coefficients").data_ptr(), int(mode),
        float(value), ptr(d_face), ptr(d_cell), ptr(weights), md.field("cell_volumes").data_ptr(),
        field.data_ptr(), out.data_ptr(), _lib.stream_ptr(dev)), "gbf_explicit_laplacian_f64")
    return out[: md.n_cells]


class DifferentiableLaplacian(torch.autograd.Function):
    """Explicit Laplacian div(D grad phi) with the reference's backward."""

    @staticmethod
    def forward(ctx: Any, phi: torch.Tensor, D: Any, mesh: Any) -> torch.Tensor:
        md = mesh_data(mesh)
        topo = md.topology()
        if phi.shape[0] != md.n_cells:
            raise ValueError(f"phi has {phi.shape[0]} entries, expected n_cells={md.n_cells}")
        phi_d = phi.detach().to(device=md.device, dtype=torch.float64).contiguous()
        spec = _resolve_d(D, md)
        out = _apply(md, topo, spec, phi_d)
        ctx.md, ctx.topo, ctx.spec = md, topo, spec
        ctx.d_grad = isinstance(D, torch.Tensor) and D.requires_grad
        ctx.d_shape = D.shape if ctx.d_grad else None
        ctx.save_for_backward(phi_d)
        return out

    @staticmethod
    def backward(ctx: Any, grad_output: torch.Tensor):
        (phi_d,) = ctx.saved_tensors
        md, topo, spec = ctx.md, ctx.topo, ctx.spec
        dev = md.device
        g = grad_output.to(device=dev, dtype=torch.float64).contiguous()
        grad_phi = _apply(md, topo, spec, g)
        grad_D = None
        if ctx.d_grad:
            mode = spec[0]
            nf = md.n_faces
            g_face = torch.empty(max(nf, 1), device=dev, dtype=torch.float64)
            g_cell = (torch.empty(max(md.n_cells, 1), device=dev, dtype=torch.float64)
                      if mode == 2 else None)
            g_sum = (torch.zeros(1, device=dev, dtype=torch.float64)
                     if mode == 0 else None)
            ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
            _lib.check(_lib.lib().gbf_explicit_laplacian_grad_d_f64(
                topo.layout_ref, nf, md.owner_all32.data_ptr(), md.bnd_ptr.data_ptr(),
                md.bnd_face.data_ptr(), md.field("face_areas").data_ptr(),
                md.field("delta_coefficients").data_ptr(), md.field("cell_volumes").data_ptr(),
                phi_d.data_ptr(), g.data_ptr(), g_face.data_ptr(), ptr(g_cell), ptr(g_sum),
                _lib.stream_ptr(dev)), "gbf_explicit_laplacian_grad_d_f64")
            if mode == 0:
                grad_D = g_sum.reshape(ctx.d_shape)
            elif mode == 2:
                grad_D = g_cell[: md.n_cells]
            else:
                grad_D = g_face[:nf]
        return grad_phi, grad_D, None
