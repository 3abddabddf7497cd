"""Implicit finite-volume operators of the linear-solve path, drop-in for
``pyfoam.discretisation.operators.fvm`` (``laplacian`` and the upwind
``div``; ``src/pyfoam/discretisation/operators.py:351-518``).

The coefficients are assembled on the GPU by libgbfoam
(``gbf_laplacian_assemble_f64``, ``gbf_div_upwind_assemble_f64``) in the
reference's rounding and summation order, so the matrices are bitwise equal
to the reference's.  ``fvm.laplacian`` is differentiable with respect to a
per-face diffusivity tensor: its backward is a face kernel giving
dL/dD_f from the gradients of lower, upper and diag.

The mesh is duck-typed like the reference's ``FvMesh``: ``n_cells``,
``n_internal_faces``, ``n_faces``, ``owner`` (all faces), ``neighbour``,
``face_areas`` (n_faces, 3), ``delta_coefficients``, ``cell_volumes``,
``device``, ``dtype`` and, for per-cell diffusivity, ``cell_centres`` and
``face_centres``.  Its tensors must be on a CUDA device.
"""

from __future__ import annotations

import ctypes
from typing import Any

import numpy as np
import torch

from .. import _lib
from ..core.device import resolve_device
from ..core.fv_matrix import FvMatrix
from ..core.topology import get_topology

__all__ = ["fvm", "MeshData", "mesh_data"]


class MeshData:
    """Per-mesh device data of the assembly (int32 addressing, boundary
    lists, interpolation weights), built once and cached on the mesh."""

    def __init__(self, mesh: Any) -> None:
        self.device = resolve_device(mesh.device)
        if mesh.dtype != torch.float64:
            raise TypeError(f"assembly runs in float64; mesh dtype is {mesh.dtype}")
        self.n_cells = int(mesh.n_cells)
        self.n_internal = int(mesh.n_internal_faces)
        self.n_faces = int(mesh.n_faces)
        own = mesh.owner.to(self.device)
        nei = mesh.neighbour.to(self.device)
        if own.shape[0] != self.n_faces or nei.shape[0] != self.n_internal:
            raise ValueError("mesh owner/neighbour sizes do not match n_faces/n_internal_faces")
        self.owner = own[: self.n_internal].to(torch.int64)
        self.neighbour = nei.to(torch.int64)
        self.owner_all32 = own.to(torch.int32).contiguous()
        own_b = own[self.n_internal:].to("cpu", torch.int32).numpy()
        ptr = np.empty(self.n_cells + 1, np.int32)
        faces = np.empty(max(own_b.shape[0], 1), np.int32)
        _lib.check(_lib.lib().gbf_boundary_lists(self.n_cells, self.n_internal, own_b.shape[0],
                                                 own_b.ctypes.data, ptr.ctypes.data,
                                                 faces.ctypes.data), "gbf_boundary_lists")
        self.bnd_ptr = torch.from_numpy(ptr).to(self.device)
        self.bnd_face = torch.from_numpy(faces).to(self.device)
        self._mesh = mesh
        self._weights: torch.Tensor | None = None

    def field(self, name: str) -> torch.Tensor:
        t = getattr(self._mesh, name)
        return t.to(device=self.device, dtype=torch.float64).contiguous()

    def topology(self):
        """Slot layout of the internal-face addressing (shared through the
        topology cache with every LduMatrix on the same tensors)."""
        return get_topology(self.n_cells, self.owner, self.neighbour)

    def weights(self, topo) -> torch.Tensor:
        if self._weights is None:
            w = torch.empty(max(self.n_faces, 1), device=self.device, dtype=torch.float64)
            cc = self.field("cell_centres")
            fc = self.field("face_centres")
            _lib.check(_lib.lib().gbf_centre_weights_f64(
                self.n_internal, self.n_faces, topo.owner32.data_ptr(),
                topo.neighbour32.data_ptr(), cc.data_ptr(), fc.data_ptr(), w.data_ptr(),
                _lib.stream_ptr(self.device)), "gbf_centre_weights_f64")
            self._weights = w
        return self._weights


def mesh_data(mesh: Any) -> MeshData:
    md = getattr(mesh, "_gbf_mesh_data", None)
    if md is None or md._mesh is not mesh:
        md = MeshData(mesh)
        try:
            mesh._gbf_mesh_data = md
        except AttributeError:
            pass
    return md


def _resolve_mesh(phi: Any, mesh: Any):
    if hasattr(phi, "mesh"):
        return phi.mesh
    if mesh is None:
        raise ValueError("mesh is required when phi is not a GeometricField")
    return mesh


def _make_fvmatrix(md: MeshData) -> FvMatrix:
    """FvMatrix on the mesh's internal-face addressing
    (operators.py:205-213)."""
    return FvMatrix(md.n_cells, md.owner, md.neighbour, device=md.device, dtype=torch.float64)


class _LaplacianCoeffs(torch.autograd.Function):
    """(lower, upper, diag) of fvm.laplacian for a per-face diffusivity,
    with dL/dD_f from a face kernel in backward."""

    @staticmethod
    def forward(ctx, D_face, md, topo, areas, delta, volumes):
        lower, upper, diag = _assemble(md, topo, areas, delta, volumes, 1, 0.0, D_face, None, None)
        ctx.md, ctx.topo = md, topo
        ctx.save_for_backward(areas, delta, volumes)
        return lower, upper, diag

    @staticmethod
    def backward(ctx, g_lower, g_upper, g_diag):
        areas, delta, volumes = ctx.saved_tensors
        md, topo = ctx.md, ctx.topo
        dev = md.device
        z_f = torch.zeros(md.n_internal, device=dev, dtype=torch.float64)
        g_lower = z_f if g_lower is None else g_lower.contiguous()
        g_upper = z_f if g_upper is None else g_upper.contiguous()
        g_diag = (torch.zeros(md.n_cells, device=dev, dtype=torch.float64) if g_diag is None
                  else g_diag.contiguous())
        gD = torch.empty(max(md.n_faces, 1), device=dev, dtype=torch.float64)
        _lib.check(_lib.lib().gbf_laplacian_grad_gamma_f64(
            topo.layout_ref, md.n_faces, md.owner_all32.data_ptr(), areas.data_ptr(),
            delta.data_ptr(), volumes.data_ptr(), g_lower.data_ptr(), g_upper.data_ptr(),
            g_diag.data_ptr(), gD.data_ptr(), _lib.stream_ptr(dev)),
            "gbf_laplacian_grad_gamma_f64")
        return gD[: md.n_faces], None, None, None, None, None


def _assemble(md, topo, areas, delta, volumes, mode, value, d_face, d_cell, weights):
    dev = md.device
    lower = torch.empty(max(md.n_internal, 1), device=dev, dtype=torch.float64)
    upper = torch.empty(max(md.n_internal, 1), device=dev, dtype=torch.float64)
    diag = torch.empty(max(md.n_cells, 1), device=dev, dtype=torch.float64)
    ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    _lib.check(_lib.lib().gbf_laplacian_assemble_f64(
        topo.layout_ref, md.n_faces, md.owner_all32.data_ptr(), md.bnd_ptr.data_ptr(),
        md.bnd_face.data_ptr(), areas.data_ptr(), delta.data_ptr(), int(mode), float(value),
        ptr(d_face), ptr(d_cell), ptr(weights), volumes.data_ptr(), lower.data_ptr(),
        upper.data_ptr(), diag.data_ptr(), _lib.stream_ptr(dev)), "gbf_laplacian_assemble_f64")
    return lower[: md.n_internal], upper[: md.n_internal], diag[: md.n_cells]


class fvm:  # noqa: N801 -- the reference's name
    @staticmethod
    def laplacian(D: Any, phi: Any, scheme: str = "Gauss linear corrected", *,
                  mesh: Any = None) -> FvMatrix:
        """Implicit Laplacian del.(D del phi) per unit volume
        (operators.py:432-518).  D: scalar, 0-d tensor, per-cell tensor
        (linearly interpolated to faces), per-face tensor (n_faces) or a
        field with ``internal_field``.  A per-face tensor that requires
        grad makes the returned coefficients differentiable."""
        mesh = _resolve_mesh(phi, mesh)
        md = mesh_data(mesh)
        mat = _make_fvmatrix(md)
        topo = mat.topology()
        areas = md.field("face_areas")
        delta = md.field("delta_coefficients")
        volumes = md.field("cell_volumes")
        n_cells, n_faces = md.n_cells, md.n_faces
        mode, value, d_face, d_cell, w = 0, 0.0, None, None, None
        if isinstance(D, (int, float)):
            value = float(D)
        elif hasattr(D, "internal_field"):
            mode, d_cell = 2, D.internal_field.to(device=md.device, dtype=torch.float64).contiguous()
        else:
            Dt = D if isinstance(D, torch.Tensor) else torch.tensor(D, dtype=torch.float64)
            if Dt.dim() == 0:
                value = float(Dt)
            elif Dt.shape[0] == n_cells:
                mode, d_cell = 2, Dt.to(device=md.device, dtype=torch.float64).contiguous()
            else:
                if Dt.shape[0] != n_faces:
                    raise ValueError(f"D has {Dt.shape[0]} entries; expected 1, n_cells="
                                     f"{n_cells} or n_faces={n_faces}")
                mode = 1
                d_face = Dt.to(device=md.device, dtype=torch.float64)
        if mode == 2:
            w = md.weights(topo)
        if mode == 1 and d_face.requires_grad and torch.is_grad_enabled():
            lower, upper, diag = _LaplacianCoeffs.apply(d_face.contiguous(), md, topo, areas,
                                                        delta, volumes)
        else:
            lower, upper, diag = _assemble(md, topo, areas, delta, volumes, mode, value,
                                           None if d_face is None else d_face.detach().contiguous(),
                                           d_cell, w)
        mat._lower, mat._upper, mat._diag = lower, upper, diag
        return mat

    @staticmethod
    def div(phi: Any, U: Any, scheme: str = "Gauss upwind", *, mesh: Any = None) -> FvMatrix:
        """Implicit convection del.(phi U) with the upwind scheme
        (operators.py:351-429, no deferred correction).  Interpolation
        schemes other than upwind are outside the linear-solve path."""
        name = scheme.strip()
        if name.startswith("Gauss "):
            name = name[6:].strip()
        if name != "upwind":
            raise ValueError(f"fvm.div: scheme '{scheme}' is not supported here; the GPU "
                             f"assembly implements 'Gauss upwind'")
        mesh = _resolve_mesh(U, mesh)
        md = mesh_data(mesh)
        flux = phi.internal_field if hasattr(phi, "internal_field") else phi
        flux = torch.as_tensor(flux).to(device=md.device, dtype=torch.float64)
        flux = flux[: md.n_internal].contiguous()
        mat = _make_fvmatrix(md)
        topo = mat.topology()
        volumes = md.field("cell_volumes")
        dev = md.device
        lower = torch.empty(max(md.n_internal, 1), device=dev, dtype=torch.float64)
        upper = torch.empty(max(md.n_internal, 1), device=dev, dtype=torch.float64)
        diag = torch.empty(max(md.n_cells, 1), device=dev, dtype=torch.float64)
        _lib.check(_lib.lib().gbf_div_upwind_assemble_f64(
            topo.layout_ref, flux.data_ptr(), volumes.data_ptr(), lower.data_ptr(),
            upper.data_ptr(), diag.data_ptr(), _lib.stream_ptr(dev)), "gbf_div_upwind_assemble_f64")
        mat._lower, mat._upper, mat._diag = (lower[: md.n_internal], upper[: md.n_internal],
                                             diag[: md.n_cells])
        return mat
