"""Structured hex meshes of the unit cube stored as unstructured LDU meshes.

This module produces the mesh inputs of the linear-solve path: owner /
neighbour addressing, face area vectors, delta coefficients, cell volumes,
cell centres and linear-interpolation weights.  It is a vectorised
restatement of the reference geometry formulas in
``src/pyfoam/mesh/mesh_geometry.py``:

* face centre = arithmetic mean of the face vertices (``:35-63``);
* face area vector = 1/2 * sum_j v_j x v_{j+1} (``:66-108``);
* cell volume / centre = sum of |tet| volumes of (vertex mean, face centre,
  v_j, v_{j+1}) over the cell's faces, volume-weighted tet centroids
  (``:139-254``);
* weights w_f = |d_N| / (|d_P| + |d_N|) (``:262-327``);
* internal delta coefficients 1 / |d . n_hat| with d = C_N - C_P
  (``:330-395``).

Two deliberate differences from the reference mesh pipeline, which produces
wrong vertices for the y- and z-normal internal faces
(``src/pyfoam/mesh/generation/block_mesh.py:378-387``) and always zero
boundary delta coefficients (``mesh_geometry.py:352,377``):

* face vertices are generated correctly for all three directions;
* boundary faces on a *Dirichlet* patch get delta = 1 / |(C_f - C_P) . n_hat|
  so that ``fvm.laplacian`` sees a fixed-value boundary; all other boundary
  faces keep delta = 0 (zero gradient), as in the reference.

Cells are indexed ``c = i + j*nx + k*nx*ny``.  Internal faces are in
upper-triangular cell order: for each cell in ascending order its +x, +y, +z
faces (when the neighbour exists), so ``owner < neighbour`` and faces are
sorted by owner.  Boundary faces follow, grouped by patch
(x0, x1, y0, y1, z0, z1), each patch ordered by owner cell.

All randomness uses ``numpy.random.default_rng(seed)`` (PCG64), which gives
the same stream on every platform.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

__all__ = ["HexMesh", "PATCH_NAMES"]

PATCH_NAMES = ("x0", "x1", "y0", "y1", "z0", "z1")


def _cross(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    return np.stack(
        [
            a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
            a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
            a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0],
        ],
        axis=-1,
    )


@dataclass
class _Patch:
    name: str
    start: int
    size: int


class HexMesh:
    """Hex mesh of the unit cube with optional interior jitter.

    Parameters
    ----------
    nx, ny, nz : int
        Cells per direction (``ny``/``nz`` default to ``nx``).
    jitter : float
        Interior points move by i.i.d. U[-jitter, jitter] * h per coordinate.
    seed : int
        Seed of the jitter stream.
    dirichlet : tuple of str
        Patches that get a non-zero boundary delta coefficient.
    device, dtype :
        Where the torch tensors of the mesh live.
    geometry : bool
        Compute the geometry with the vectorised numpy restatement (default).
        ``False`` keeps only points and addressing, e.g. for ``polymesh()``
        whose geometry the GPU ``FvMesh`` computes.
    """

    def __init__(
        self,
        nx: int,
        ny: int | None = None,
        nz: int | None = None,
        *,
        jitter: float = 0.0,
        seed: int = 1,
        dirichlet: tuple[str, ...] = ("x0",),
        device: torch.device | str = "cpu",
        dtype: torch.dtype = torch.float64,
        geometry: bool = True,
    ) -> None:
        ny = nx if ny is None else ny
        nz = nx if nz is None else nz
        if min(nx, ny, nz) < 1:
            raise ValueError("mesh needs at least one cell per direction")
        self.nx, self.ny, self.nz = nx, ny, nz
        self.jitter = float(jitter)
        self.seed = seed
        self.dirichlet = tuple(dirichlet)
        self.device = torch.device(device)
        self.dtype = dtype

        n = nx * ny * nz
        self.n_cells = n
        c = np.arange(n, dtype=np.int64)
        i = c % nx
        j = (c // nx) % ny
        k = c // (nx * ny)

        # ---- internal faces, upper-triangular cell order (+x, +y, +z) ----
        has = np.stack([i < nx - 1, j < ny - 1, k < nz - 1], axis=1)
        flat = np.flatnonzero(has.ravel())
        fcell = flat // 3
        fdir = flat % 3
        step = np.array([1, nx, nx * ny], dtype=np.int64)
        self._int_cell = fcell
        self._int_dir = fdir
        owner_int = fcell
        neigh = fcell + step[fdir]
        self.n_internal_faces = int(owner_int.shape[0])

        # ---- boundary faces grouped by patch ----
        bcells, bkind = [], []
        self.patches: dict[str, _Patch] = {}
        start = self.n_internal_faces
        masks = [i == 0, i == nx - 1, j == 0, j == ny - 1, k == 0, k == nz - 1]
        for p, (name, m) in enumerate(zip(PATCH_NAMES, masks)):
            cells = c[m]
            bcells.append(cells)
            bkind.append(np.full(cells.shape[0], p, dtype=np.int64))
            self.patches[name] = _Patch(name, start, int(cells.shape[0]))
            start += int(cells.shape[0])
        self._bnd_cell = np.concatenate(bcells)
        self._bnd_kind = np.concatenate(bkind)
        self.n_faces = start
        owner_all = np.concatenate([owner_int, self._bnd_cell])

        # ---- points ----
        self._points = self._make_points()

        self._owner_np = owner_all
        self._neigh_np = neigh
        if geometry:
            self._geometry()

    # ------------------------------------------------------------------
    def _make_points(self) -> np.ndarray:
        nx, ny, nz = self.nx, self.ny, self.nz
        gx = np.linspace(0.0, 1.0, nx + 1)
        gy = np.linspace(0.0, 1.0, ny + 1)
        gz = np.linspace(0.0, 1.0, nz + 1)
        Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
        pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        if self.jitter > 0.0:
            rng = np.random.default_rng(self.seed)
            h = np.array([1.0 / nx, 1.0 / ny, 1.0 / nz])
            d = rng.uniform(-self.jitter, self.jitter, size=pts.shape) * h
            pi = np.arange(pts.shape[0])
            ii = pi % (nx + 1)
            jj = (pi // (nx + 1)) % (ny + 1)
            kk = pi // ((nx + 1) * (ny + 1))
            interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)
            pts[interior] += d[interior]
        return pts

    def _pid(self, i, j, k):
        return i + j * (self.nx + 1) + k * (self.nx + 1) * (self.ny + 1)

    def _face_points(self, cells: np.ndarray, kind: np.ndarray) -> np.ndarray:
        """Point indices (F, 4) of faces; kind 0..2 = +x,+y,+z internal faces
        of the cell, 3..8 = boundary patches x0..z1 with outward normals."""
        nx, ny = self.nx, self.ny
        i = cells % nx
        j = (cells // nx) % ny
        k = cells // (nx * ny)
        P = self._pid
        out = np.empty((cells.shape[0], 4), dtype=np.int64)

        def put(m, a, b, c_, d):
            out[m, 0], out[m, 1], out[m, 2], out[m, 3] = a[m], b[m], c_[m], d[m]

        i1, j1, k1 = i + 1, j + 1, k + 1
        # +x face at plane i+1 (normal +x): (y,z) = (0,0)(1,0)(1,1)(0,1)
        m = (kind == 0) | (kind == 4)
        put(m, P(i1, j, k), P(i1, j1, k), P(i1, j1, k1), P(i1, j, k1))
        m = kind == 3  # x0: plane i, normal -x
        put(m, P(i, j, k), P(i, j, k1), P(i, j1, k1), P(i, j1, k))
        # +y face at plane j+1 (normal +y): (z,x) = (0,0)(1,0)(1,1)(0,1)
        m = (kind == 1) | (kind == 6)
        put(m, P(i, j1, k), P(i, j1, k1), P(i1, j1, k1), P(i1, j1, k))
        m = kind == 5  # y0: plane j, normal -y
        put(m, P(i, j, k), P(i1, j, k), P(i1, j, k1), P(i, j, k1))
        # +z face at plane k+1 (normal +z): (x,y) = (0,0)(1,0)(1,1)(0,1)
        m = (kind == 2) | (kind == 8)
        put(m, P(i, j, k1), P(i1, j, k1), P(i1, j1, k1), P(i, j1, k1))
        m = kind == 7  # z0: plane k, normal -z
        put(m, P(i, j, k), P(i, j1, k), P(i1, j1, k), P(i1, j, k))
        return out

    def _face_geometry(self, cells, kind, chunk=1 << 21):
        n = cells.shape[0]
        centres = np.empty((n, 3))
        areas = np.empty((n, 3))
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            v = self._points[self._face_points(cells[s:e], kind[s:e])]
            centres[s:e] = v.mean(axis=1)
            a = np.zeros((e - s, 3))
            for q in range(4):
                a += _cross(v[:, q], v[:, (q + 1) % 4])
            areas[s:e] = 0.5 * a
        return centres, areas

    def _uniform_face_geometry(self, cells, kind):
        """Closed form of the face centres / area vectors of an unjittered
        mesh (the same values the vertex formulas give, up to rounding)."""
        hx, hy, hz = 1.0 / self.nx, 1.0 / self.ny, 1.0 / self.nz
        i = cells % self.nx
        j = (cells // self.nx) % self.ny
        k = cells // (self.nx * self.ny)
        # offset of the face plane from the cell's low corner, per kind
        ox = np.array([1.0, 0.5, 0.5, 0.0, 1.0, 0.5, 0.5, 0.5, 0.5])
        oy = np.array([0.5, 1.0, 0.5, 0.5, 0.5, 0.0, 1.0, 0.5, 0.5])
        oz = np.array([0.5, 0.5, 1.0, 0.5, 0.5, 0.5, 0.5, 0.0, 1.0])
        fc = np.stack([(i + ox[kind]) * hx, (j + oy[kind]) * hy, (k + oz[kind]) * hz], axis=1)
        ax = np.array([1, 0, 0, -1, 1, 0, 0, 0, 0], dtype=np.float64) * (hy * hz)
        ay = np.array([0, 1, 0, 0, 0, -1, 1, 0, 0], dtype=np.float64) * (hz * hx)
        az = np.array([0, 0, 1, 0, 0, 0, 0, -1, 1], dtype=np.float64) * (hx * hy)
        fa = np.stack([ax[kind], ay[kind], az[kind]], axis=1)
        return fc, fa

    def _cell_geometry(self, chunk=1 << 18):
        """Volumes and centres from the tet decomposition of each hex."""
        n = self.n_cells
        vol = np.empty(n)
        cen = np.empty((n, 3))
        kinds = np.array([3, 4, 5, 6, 7, 8])  # the six faces of a cell, outward
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            cells = np.arange(s, e, dtype=np.int64)
            m = e - s
            fp = np.stack(
                [self._face_points(cells, np.full(m, kd)) for kd in kinds], axis=1
            )  # (m, 6, 4)
            v = self._points[fp]  # (m, 6, 4, 3)
            corners = np.concatenate([fp[:, 0], fp[:, 1]], axis=1)  # x0 + x1 faces = 8 corners
            ref = self._points[corners].mean(axis=1)  # (m, 3)
            fc = v.mean(axis=2)  # (m, 6, 3)
            a = v
            b = np.roll(v, -1, axis=2)
            r = ref[:, None, None, :]
            f = fc[:, :, None, :]
            tv = np.abs(np.einsum("...i,...i->...", f - r, _cross(a - r, b - r))) / 6.0
            tc = (r + f + a + b) / 4.0
            tot = tv.sum(axis=(1, 2))
            vol[s:e] = tot
            cen[s:e] = (tv[..., None] * tc).sum(axis=(1, 2)) / tot[:, None]
        return vol, cen

    def _geometry(self) -> None:
        nint = self.n_internal_faces
        uniform = self.jitter == 0.0
        all_cells = np.concatenate([self._int_cell, self._bnd_cell])
        all_kind = np.concatenate([self._int_dir, self._bnd_kind + 3])
        if uniform:
            fc, fa = self._uniform_face_geometry(all_cells, all_kind)
        else:
            fc, fa = self._face_geometry(all_cells, all_kind)
        if uniform:
            hx, hy, hz = 1.0 / self.nx, 1.0 / self.ny, 1.0 / self.nz
            c = np.arange(self.n_cells, dtype=np.int64)
            i = c % self.nx
            j = (c // self.nx) % self.ny
            k = c // (self.nx * self.ny)
            cen = np.stack([(i + 0.5) * hx, (j + 0.5) * hy, (k + 0.5) * hz], axis=1)
            vol = np.full(self.n_cells, hx * hy * hz)
        else:
            vol, cen = self._cell_geometry()
        own = self._owner_np
        nei = self._neigh_np
        # weights (internal faces), boundary weight 1
        w = np.ones(self.n_faces)
        dP = np.linalg.norm(fc[:nint] - cen[own[:nint]], axis=1)
        dN = np.linalg.norm(fc[:nint] - cen[nei], axis=1)
        den = dP + dN
        w[:nint] = dN / np.where(den > 1e-30, den, 1.0)
        # delta coefficients
        delta = np.zeros(self.n_faces)
        smag = np.linalg.norm(fa, axis=1)
        nhat = fa / np.where(smag > 1e-30, smag, 1.0)[:, None]
        d = cen[nei] - cen[own[:nint]]
        ddn = np.abs((d * nhat[:nint]).sum(axis=1))
        delta[:nint] = 1.0 / np.where(ddn > 1e-30, ddn, 1.0)
        for name in self.dirichlet:
            p = self.patches[name]
            sl = slice(p.start, p.start + p.size)
            db = np.abs(((fc[sl] - cen[own[sl]]) * nhat[sl]).sum(axis=1))
            delta[sl] = 1.0 / np.where(db > 1e-30, db, 1.0)
        self._np = dict(
            face_centres=fc, face_areas=fa, cell_volumes=vol, cell_centres=cen,
            weights=w, delta_coefficients=delta,
        )
        self._t: dict[str, torch.Tensor] = {}

    # ------------------------------------------------------------------
    # Duck-typed FvMesh surface used by fvm.laplacian / fvm.div
    # ------------------------------------------------------------------
    def _tensor(self, key: str, arr: np.ndarray, dtype) -> torch.Tensor:
        t = self._t.get(key)
        if t is None:
            t = torch.from_numpy(np.ascontiguousarray(arr)).to(device=self.device, dtype=dtype)
            self._t[key] = t
        return t

    @property
    def owner(self) -> torch.Tensor:
        """Owner cell of every face (internal then boundary), int64."""
        return self._tensor("owner", self._owner_np, torch.int64)

    @property
    def neighbour(self) -> torch.Tensor:
        """Neighbour cell of every internal face, int64."""
        return self._tensor("neighbour", self._neigh_np, torch.int64)

    @property
    def internal_owner(self) -> torch.Tensor:
        return self.owner[: self.n_internal_faces]

    def __getattr__(self, name: str):
        np_store = self.__dict__.get("_np")
        if np_store is not None and name in np_store:
            return self._tensor(name, np_store[name], self.dtype)
        raise AttributeError(name)

    @property
    def points(self) -> torch.Tensor:
        return self._tensor("points", self._points, self.dtype)

    def polymesh(self) -> dict:
        """The mesh as polyMesh arrays: points (n_points, 3), faces as CSR
        (face_ptr, face_pts; four vertices each, normal out of the owner),
        owner (all faces), neighbour (internal faces) and the boundary
        patches (name, type, startFace, nFaces)."""
        cells = np.concatenate([self._int_cell, self._bnd_cell])
        kind = np.concatenate([self._int_dir, self._bnd_kind + 3])
        faces = self._face_points(cells, kind)
        return dict(points=self._points, face_ptr=np.arange(0, 4 * faces.shape[0] + 1, 4),
                    face_pts=faces.ravel(), owner=self._owner_np, neighbour=self._neigh_np,
                    boundary=[{"name": p.name, "type": "patch", "startFace": p.start,
                               "nFaces": p.size} for p in self.patches.values()])

    def to(self, device=None, dtype=None) -> "HexMesh":
        """Return a shallow copy whose tensors live on ``device``/``dtype``."""
        m = object.__new__(HexMesh)
        m.__dict__.update(self.__dict__)
        m.device = torch.device(device) if device is not None else self.device
        m.dtype = dtype or self.dtype
        m._t = {}
        return m

    def numpy(self, name: str) -> np.ndarray:
        """Host copy of a geometry array (``owner``/``neighbour`` included)."""
        if name == "owner":
            return self._owner_np
        if name == "neighbour":
            return self._neigh_np
        return self._np[name]

    def __repr__(self) -> str:
        return (
            f"HexMesh({self.nx}x{self.ny}x{self.nz}, jitter={self.jitter}, "
            f"n_cells={self.n_cells}, n_internal_faces={self.n_internal_faces}, "
            f"device={self.device})"
        )
