"""Polyhedral meshes with GPU-computed finite-volume geometry, drop-in for
``pyfoam.mesh.PolyMesh`` / ``pyfoam.mesh.FvMesh``
(``src/pyfoam/mesh/poly_mesh.py:30-242``, ``src/pyfoam/mesh/fv_mesh.py:34-251``).

The reference computes the geometry in Python loops over faces and cells
(``mesh/mesh_geometry.py:35-395``: hours at 128^3).  Here the same formulas
run as libgbfoam kernels, one thread per face or cell
(``gbf_face_geometry_f64``, ``gbf_cell_geometry_f64``,
``gbf_face_interp_f64``); the cell -> face lists come from one host pass
(``gbf_cell_faces``).  Geometry is lazy and cached like the reference's;
``compute_geometry()`` computes everything at once.

Conventions are the reference's: faces are lists of point indices (or a
CSR pair ``face_ptr`` / ``face_pts``), ``owner`` covers all faces,
``neighbour`` the internal ones, ``owner < neighbour`` on internal faces,
``n_cells = max(owner) + 1``; boundary faces get weight 1 and delta 0.
Geometry is float64 on a CUDA device; there is no CPU fallback.
"""

from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from .. import _lib
from ..core.device import resolve_device

__all__ = ["PolyMesh", "FvMesh", "faces_to_csr"]


def faces_to_csr(faces) -> tuple[np.ndarray, np.ndarray]:
    """(face_ptr int32 [n_faces + 1], face_pts int32) of a face list."""
    if isinstance(faces, tuple) and len(faces) == 2:
        ptr = np.ascontiguousarray(np.asarray(faces[0]), np.int64)
        pts = np.ascontiguousarray(np.asarray(faces[1]), np.int64)
    else:
        lens = np.fromiter((len(f) for f in faces), dtype=np.int64, count=len(faces))
        ptr = np.zeros(len(faces) + 1, np.int64)
        np.cumsum(lens, out=ptr[1:])
        pts = (np.concatenate([np.asarray(f.cpu() if isinstance(f, torch.Tensor) else f,
                                          np.int64).ravel() for f in faces])
               if len(faces) else np.zeros(0, np.int64))
    if ptr.shape[0] < 1 or ptr[0] != 0 or np.any(np.diff(ptr) < 0) or ptr[-1] != pts.shape[0]:
        raise ValueError("face_ptr must start at 0, be non-decreasing and end at len(face_pts)")
    if pts.shape[0] >= 2**31:
        raise ValueError("more than 2^31 face vertices")
    return ptr.astype(np.int32), pts.astype(np.int32)


def _i64(a) -> np.ndarray:
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(a), np.int64)


class PolyMesh:
    """Topology and points of a polyhedral mesh (reference
    ``PolyMesh(points, faces, owner, neighbour, boundary=None, *,
    validate=True, device=None, dtype=None)``)."""

    def __init__(self, points, faces, owner, neighbour, boundary: list[dict] | None = None, *,
                 validate: bool = True, device=None, dtype: torch.dtype | None = None) -> None:
        dev = resolve_device(device)
        dtype = dtype or torch.float64
        if dtype != torch.float64:
            raise TypeError(f"mesh geometry runs in float64, got {dtype}")
        pts = torch.as_tensor(points, dtype=torch.float64)
        if pts.dim() != 2 or pts.shape[1] != 3:
            raise ValueError(f"points must have shape (n_points, 3), got {tuple(pts.shape)}")
        self._points = pts.to(dev).contiguous()
        self._face_ptr_h, self._face_pts_h = faces_to_csr(faces)
        own, nei = _i64(owner), _i64(neighbour)
        self._n_points = int(pts.shape[0])
        self._n_faces = int(self._face_ptr_h.shape[0] - 1)
        self._n_internal_faces = int(nei.shape[0])
        self._n_cells = int(own.max()) + 1 if own.size else 0
        if own.shape[0] != self._n_faces:
            raise ValueError(f"owner has {own.shape[0]} entries for {self._n_faces} faces")
        if self._face_pts_h.size and (self._face_pts_h.min() < 0 or
                                      self._face_pts_h.max() >= self._n_points):
            raise ValueError(f"a face refers to a point outside [0, {self._n_points})")
        if validate:
            _validate_owner_neighbour(own, nei, self._n_cells, self._n_internal_faces)
        self._own_h, self._nei_h = own, nei
        self._owner = torch.from_numpy(own).to(dev)
        self._neighbour = torch.from_numpy(nei).to(dev)
        self._boundary = list(boundary) if boundary is not None else []
        self._device = dev
        self._faces_list: list[torch.Tensor] | None = None

    # ------------------------------------------------------------------
    @property
    def points(self) -> torch.Tensor:
        return self._points

    @property
    def faces(self) -> list[torch.Tensor]:
        if self._faces_list is None:
            p, q = self._face_ptr_h, torch.from_numpy(self._face_pts_h.astype(np.int64))
            self._faces_list = [q[p[i]:p[i + 1]].to(self._device) for i in range(self._n_faces)]
        return self._faces_list

    @property
    def owner(self) -> torch.Tensor:
        return self._owner

    @property
    def neighbour(self) -> torch.Tensor:
        return self._neighbour

    @property
    def boundary(self) -> list[dict]:
        return self._boundary

    @property
    def n_points(self) -> int:
        return self._n_points

    @property
    def n_faces(self) -> int:
        return self._n_faces

    @property
    def n_cells(self) -> int:
        return self._n_cells

    @property
    def n_internal_faces(self) -> int:
        return self._n_internal_faces

    @property
    def device(self) -> torch.device:
        return self._device

    @property
    def dtype(self) -> torch.dtype:
        return torch.float64

    def face_points(self, face_idx: int) -> torch.Tensor:
        a, b = self._face_ptr_h[face_idx], self._face_ptr_h[face_idx + 1]
        idx = torch.from_numpy(self._face_pts_h[a:b].astype(np.int64)).to(self._device)
        return self._points[idx]

    def is_boundary_face(self, face_idx: int) -> bool:
        return face_idx >= self._n_internal_faces

    def patch_faces(self, patch_idx: int) -> range:
        p = self._boundary[patch_idx]
        return range(p["startFace"], p["startFace"] + p["nFaces"])

    @classmethod
    def from_raw(cls, points: Sequence, faces: Sequence, owner: Sequence, neighbour: Sequence,
                 boundary: list[dict] | None = None, **kwargs):
        return cls(torch.tensor(points, dtype=torch.float64), [list(f) for f in faces],
                   owner, neighbour, boundary, **kwargs)

    def __repr__(self) -> str:
        return (f"{type(self).__name__}(n_points={self._n_points}, n_faces={self._n_faces}, "
                f"n_cells={self._n_cells}, n_internal_faces={self._n_internal_faces}, "
                f"device={self._device})")


def _validate_owner_neighbour(own: np.ndarray, nei: np.ndarray, n_cells: int,
                              n_internal: int) -> None:
    """The reference's checks (mesh/topology.py:35-88)."""
    if own.shape[0] < n_internal:
        raise ValueError(f"Total faces ({own.shape[0]}) < n_internal_faces ({n_internal})")
    if own.size and (own.min() < 0 or own.max() >= n_cells):
        raise ValueError(f"owner indices out of range [0, {n_cells})")
    if n_internal:
        if nei.min() < 0 or nei.max() >= n_cells:
            raise ValueError(f"neighbour indices out of range [0, {n_cells})")
        bad = int((own[:n_internal] >= nei).sum())
        if bad:
            raise ValueError(f"{bad} internal face(s) violate owner < neighbour convention")


class FvMesh(PolyMesh):
    """PolyMesh plus lazily computed finite-volume geometry, on the GPU."""

    def __init__(self, *args, **kwargs) -> None:
        super().__init__(*args, **kwargs)
        self._geo: dict[str, torch.Tensor] = {}
        self._dev_addr: dict[str, torch.Tensor] | None = None

    # ------------------------------------------------------------------
    def _addr(self) -> dict[str, torch.Tensor]:
        if self._dev_addr is None:
            dev = self._device
            n, nf, ni = self._n_cells, self._n_faces, self._n_internal_faces
            own32 = np.ascontiguousarray(self._own_h, np.int32)
            nei32 = np.ascontiguousarray(self._nei_h, np.int32)
            cptr = np.empty(n + 1, np.int32)
            cfaces = np.empty(max(nf + ni, 1), np.int32)
            _lib.check(_lib.lib().gbf_cell_faces(n, nf, ni, own32.ctypes.data,
                                                 nei32.ctypes.data, cptr.ctypes.data,
                                                 cfaces.ctypes.data), "gbf_cell_faces")
            to = lambda a: torch.from_numpy(a).to(dev)  # noqa: E731
            self._dev_addr = dict(face_ptr=to(self._face_ptr_h),
                                  face_pts=to(self._face_pts_h if self._face_pts_h.size
                                              else np.zeros(1, np.int32)),
                                  cell_ptr=to(cptr), cell_faces=to(cfaces),
                                  owner32=to(own32 if own32.size else np.zeros(1, np.int32)),
                                  neighbour32=to(nei32 if nei32.size else np.zeros(1, np.int32)))
        return self._dev_addr

    def _compute_face_geometry(self) -> None:
        if "face_centres" in self._geo:
            return
        a = self._addr()
        nf = self._n_faces
        fc = torch.empty(nf, 3, device=self._device, dtype=torch.float64)
        fa = torch.empty(nf, 3, device=self._device, dtype=torch.float64)
        _lib.check(_lib.lib().gbf_face_geometry_f64(nf, a["face_ptr"].data_ptr(),
                                                    a["face_pts"].data_ptr(),
                                                    self._points.data_ptr(), fc.data_ptr(),
                                                    fa.data_ptr(), _lib.stream_ptr(self._device)),
                   "gbf_face_geometry_f64")
        self._geo["face_centres"], self._geo["face_areas"] = fc, fa

    def _compute_cell_geometry(self) -> None:
        if "cell_volumes" in self._geo:
            return
        self._compute_face_geometry()
        a = self._addr()
        n = self._n_cells
        vol = torch.empty(n, device=self._device, dtype=torch.float64)
        cen = torch.empty(n, 3, device=self._device, dtype=torch.float64)
        status = torch.zeros(1, device=self._device, dtype=torch.int32)
        _lib.check(_lib.lib().gbf_cell_geometry_f64(
            n, a["cell_ptr"].data_ptr(), a["cell_faces"].data_ptr(), a["face_ptr"].data_ptr(),
            a["face_pts"].data_ptr(), self._points.data_ptr(),
            self._geo["face_centres"].data_ptr(), vol.data_ptr(), cen.data_ptr(),
            status.data_ptr(), _lib.stream_ptr(self._device)), "gbf_cell_geometry_f64")
        if int(status.item()):
            raise ValueError("a cell has more than 64 distinct vertices; the GPU cell-geometry "
                             "kernel supports up to 64")
        self._geo["cell_volumes"], self._geo["cell_centres"] = vol, cen

    def _compute_interpolation_geometry(self) -> None:
        if "face_weights" in self._geo:
            return
        self._compute_cell_geometry()
        a = self._addr()
        nf = self._n_faces
        w = torch.empty(nf, device=self._device, dtype=torch.float64)
        d = torch.empty(nf, device=self._device, dtype=torch.float64)
        _lib.check(_lib.lib().gbf_face_interp_f64(
            nf, self._n_internal_faces, a["owner32"].data_ptr(), a["neighbour32"].data_ptr(),
            self._geo["cell_centres"].data_ptr(), self._geo["face_centres"].data_ptr(),
            self._geo["face_areas"].data_ptr(), w.data_ptr(), d.data_ptr(),
            _lib.stream_ptr(self._device)), "gbf_face_interp_f64")
        self._geo["face_weights"], self._geo["delta_coefficients"] = w, d

    def compute_geometry(self) -> None:
        """Compute every geometric quantity (reference ``compute_geometry``)."""
        self._compute_face_geometry()
        self._compute_cell_geometry()
        self._compute_interpolation_geometry()

    # ------------------------------------------------------------------
    @property
    def face_centres(self) -> torch.Tensor:
        self._compute_face_geometry()
        return self._geo["face_centres"]

    @property
    def face_areas(self) -> torch.Tensor:
        self._compute_face_geometry()
        return self._geo["face_areas"]

    @property
    def cell_centres(self) -> torch.Tensor:
        self._compute_cell_geometry()
        return self._geo["cell_centres"]

    @property
    def cell_volumes(self) -> torch.Tensor:
        self._compute_cell_geometry()
        return self._geo["cell_volumes"]

    @property
    def face_weights(self) -> torch.Tensor:
        self._compute_interpolation_geometry()
        return self._geo["face_weights"]

    @property
    def delta_coefficients(self) -> torch.Tensor:
        self._compute_interpolation_geometry()
        return self._geo["delta_coefficients"]

    @property
    def face_areas_magnitude(self) -> torch.Tensor:
        return torch.linalg.vector_norm(self.face_areas, dim=1)

    @property
    def face_normals(self) -> torch.Tensor:
        a = self.face_areas
        mag = torch.linalg.vector_norm(a, dim=1, keepdim=True)
        return a / torch.where(mag > 1e-30, mag, torch.ones_like(mag))

    @property
    def total_volume(self) -> torch.Tensor:
        return self.cell_volumes.sum()

    @classmethod
    def from_poly_mesh(cls, mesh: PolyMesh) -> "FvMesh":
        return cls(mesh.points, (mesh._face_ptr_h, mesh._face_pts_h), mesh._own_h, mesh._nei_h,
                   mesh.boundary, validate=False, device=mesh.device)
