"""LDU matrix on the GPU, drop-in for ``pyfoam.core.ldu_matrix.LduMatrix``
(``src/pyfoam/core/ldu_matrix.py:27-392``).

Storage is the reference's: ``diag`` (n_cells), ``lower`` / ``upper``
(n_internal_faces) in face order and int64 ``owner`` / ``neighbour``, all on
one CUDA device.  Derived per-matrix data -- the cell-sliced packed copy of
the off-diagonals used by the gather kernels -- is cached and keyed by the
coefficient tensors' in-place version counters, so it also follows in-place
edits (the reference needs ``invalidate_cache()`` after those).

``Ax`` / ``Ax_T`` run libgbfoam's cell-centred gather, which reproduces the
reference's face-ordered ``scatter_add`` summation bit for bit.
"""

from __future__ import annotations

import torch

from .. import _lib
from .device import resolve_device, to_device
from .dtype import CFD_DTYPE, INDEX_DTYPE, assert_floating
from .topology import Topology, get_topology

__all__ = ["LduMatrix"]


class LduMatrix:
    """LDU-format sparse matrix for finite-volume systems.

    Parameters
    ----------
    n_cells : int
        Matrix dimension.
    owner, neighbour : torch.Tensor
        ``(n_internal_faces,)`` owner / neighbour cell of each internal face.
    device : torch.device or str, optional
        A CUDA device (default: the current one).  CPU is rejected.
    dtype : torch.dtype, optional
        float64 (default) or float32.
    """

    def __init__(
        self,
        n_cells: int,
        owner: torch.Tensor,
        neighbour: torch.Tensor,
        *,
        device: torch.device | str | None = None,
        dtype: torch.dtype | None = None,
    ) -> None:
        self._device = resolve_device(device)
        self._dtype = dtype or CFD_DTYPE
        if self._dtype not in (torch.float64, torch.float32):
            raise TypeError(f"LduMatrix dtype must be float64 or float32, got {self._dtype}")
        self._n_cells = int(n_cells)
        self._n_internal_faces = int(neighbour.shape[0])
        if int(owner.shape[0]) != self._n_internal_faces:
            raise ValueError(
                f"owner has {owner.shape[0]} entries, neighbour has {neighbour.shape[0]}"
            )
        self._owner = owner.to(device=self._device, dtype=INDEX_DTYPE).contiguous()
        self._neighbour = neighbour.to(device=self._device, dtype=INDEX_DTYPE).contiguous()
        self._diag = torch.zeros(self._n_cells, device=self._device, dtype=self._dtype)
        self._lower = torch.zeros(self._n_internal_faces, device=self._device, dtype=self._dtype)
        self._upper = torch.zeros(self._n_internal_faces, device=self._device, dtype=self._dtype)
        self._csr_cache: dict = {}
        self._topology: Topology | None = None

    # ------------------------------------------------------------------
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
        return self._dtype

    @property
    def owner(self) -> torch.Tensor:
        return self._owner

    @property
    def neighbour(self) -> torch.Tensor:
        return self._neighbour

    def _coerce(self, value: torch.Tensor, size: int, name: str) -> torch.Tensor:
        if not isinstance(value, torch.Tensor):
            value = torch.as_tensor(value)
        v = to_device(value, self._device, self._dtype)
        if v.dim() != 1 or v.shape[0] != size:
            raise ValueError(f"{name} must have shape ({size},), got {tuple(v.shape)}")
        return v

    @property
    def diag(self) -> torch.Tensor:
        return self._diag

    @diag.setter
    def diag(self, value: torch.Tensor) -> None:
        self._diag = self._coerce(value, self._n_cells, "diag")
        self.invalidate_cache()

    @property
    def lower(self) -> torch.Tensor:
        return self._lower

    @lower.setter
    def lower(self, value: torch.Tensor) -> None:
        self._lower = self._coerce(value, self._n_internal_faces, "lower")
        self.invalidate_cache()

    @property
    def upper(self) -> torch.Tensor:
        return self._upper

    @upper.setter
    def upper(self, value: torch.Tensor) -> None:
        self._upper = self._coerce(value, self._n_internal_faces, "upper")
        self.invalidate_cache()

    # ------------------------------------------------------------------
    # derived data
    # ------------------------------------------------------------------
    def topology(self) -> Topology:
        if self._topology is None:
            self._topology = get_topology(self._n_cells, self._owner, self._neighbour)
        return self._topology

    def _stream(self) -> int:
        return _lib.stream_ptr(self._device)

    def packed(self, transposed: bool = False, dtype: torch.dtype | None = None) -> torch.Tensor:
        """Cell-sliced copy of the off-diagonals: (lower, upper) packing, or
        (upper, lower) for the transpose.  ``dtype=float32`` on a float64
        matrix gives the rounded FP32 copy used by the mixed solver."""
        dt = dtype or self._dtype
        lo, up = self._diag_free_sources(transposed)
        key = ("packed", transposed, dt, lo.data_ptr(), lo._version, up.data_ptr(), up._version)
        hit = self._csr_cache.get(key)
        if hit is not None:
            return hit
        topo = self.topology()
        out = torch.empty(max(topo.n_slots, 1), device=self._device, dtype=dt)
        L = _lib.lib()
        if self._dtype == torch.float64 and dt == torch.float64:
            fn, name = L.gbf_pack_f64, "gbf_pack_f64"
        elif self._dtype == torch.float32 and dt == torch.float32:
            fn, name = L.gbf_pack_f32, "gbf_pack_f32"
        elif self._dtype == torch.float64 and dt == torch.float32:
            fn, name = L.gbf_pack_f64_to_f32, "gbf_pack_f64_to_f32"
        else:
            raise TypeError(f"cannot pack a {self._dtype} matrix as {dt}")
        _lib.check(fn(topo.layout_ref, lo.data_ptr(), up.data_ptr(), out.data_ptr(),
                      self._stream()), name)
        # drop stale packings of the same kind
        for k in [k for k in self._csr_cache if k[:3] == key[:3]]:
            del self._csr_cache[k]
        self._csr_cache[key] = out
        return out

    def packed_sym32(self) -> torch.Tensor | None:
        """FP32 owner-side half of a symmetric float64 matrix (lower == upper
        bit for bit) on a layout that supports it, else None.  The mixed
        solver's inner Amul then streams half the coefficient bytes and gives
        the same bits as with the full packing."""
        if self._dtype != torch.float64 or self._n_internal_faces == 0:
            return None
        topo = self.topology()
        if not topo.symmetric_storage:
            return None
        lo, up = self._lower, self._upper
        key = ("packed_sym32", lo.data_ptr(), lo._version, up.data_ptr(), up._version)
        if key in self._csr_cache:
            return self._csr_cache[key]
        out = torch.empty(max(topo.n_slots // 2, 1), device=self._device, dtype=torch.float32)
        flag = torch.zeros(1, device=self._device, dtype=torch.int32)
        _lib.check(_lib.lib().gbf_pack_sym_f64_to_f32(topo.layout_ref, lo.data_ptr(),
                                                      up.data_ptr(), out.data_ptr(),
                                                      flag.data_ptr(), self._stream()),
                   "gbf_pack_sym_f64_to_f32")
        res = None if int(flag.item()) else out
        for k in [k for k in self._csr_cache if k[0] == "packed_sym32"]:
            del self._csr_cache[k]
        self._csr_cache[key] = res
        return res

    def _diag_free_sources(self, transposed: bool):
        return (self._upper, self._lower) if transposed else (self._lower, self._upper)

    # ------------------------------------------------------------------
    # Matrix-vector products
    # ------------------------------------------------------------------
    def _check_x(self, x: torch.Tensor) -> torch.Tensor:
        assert_floating(x, "x")
        if x.shape[0] != self._n_cells:
            raise ValueError(f"x has {x.shape[0]} elements, expected {self._n_cells}")
        return x.to(device=self._device, dtype=self._dtype).contiguous()

    def _amul(self, x: torch.Tensor, transposed: bool) -> torch.Tensor:
        x = self._check_x(x)
        topo = self.topology()
        coef = self.packed(transposed)
        L = _lib.lib()
        if self._dtype == torch.float64:
            y = torch.empty(self._n_cells, device=self._device, dtype=torch.float64)
            _lib.check(L.gbf_amul_f64(topo.layout_ref, coef.data_ptr(), self._diag.data_ptr(),
                                      x.data_ptr(), y.data_ptr(), int(transposed), self._stream()),
                       "gbf_amul_f64")
        else:
            # reference semantics: float32 products, float64 sums and result
            # (core/backend.py:58-63 allocates the scatter output in float64)
            y = torch.empty(self._n_cells, device=self._device, dtype=torch.float64)
            _lib.check(L.gbf_amul_f32_f64out(topo.layout_ref, coef.data_ptr(),
                                             self._diag.data_ptr(), x.data_ptr(), y.data_ptr(),
                                             int(transposed), self._stream()),
                       "gbf_amul_f32_f64out")
        return y

    def Ax(self, x: torch.Tensor) -> torch.Tensor:
        """y = A x  (core/ldu_matrix.py:172-217).

        Raises ``TypeError`` for a non-floating x and ``ValueError`` for a
        wrong length, as the reference does."""
        return self._amul(x, transposed=False)

    def Ax_T(self, x: torch.Tensor) -> torch.Tensor:
        """y = A^T x  (core/ldu_matrix.py:219-258)."""
        return self._amul(x, transposed=True)

    def add_to_diag(self, values: torch.Tensor) -> None:
        """diag += values (scalar or (n_cells,)), core/ldu_matrix.py:260-273."""
        if not isinstance(values, torch.Tensor):
            values = torch.as_tensor(values, dtype=self._dtype)
        if values.dim() == 0:
            self._diag = (self._diag + values.to(self._device)).contiguous()
        else:
            self._diag = (self._diag + values.to(device=self._device, dtype=self._dtype)).contiguous()
        self.invalidate_cache()

    # ------------------------------------------------------------------
    # COO / CSR views (format conversion only; products use the kernels)
    # ------------------------------------------------------------------
    def to_sparse_coo(self) -> torch.Tensor:
        n = self._n_cells
        ar = torch.arange(n, device=self._device, dtype=INDEX_DTYPE)
        rows = torch.cat([ar, self._owner, self._neighbour])
        cols = torch.cat([ar, self._neighbour, self._owner])
        vals = torch.cat([self._diag, self._lower, self._upper])
        return torch.sparse_coo_tensor(torch.stack([rows, cols]), vals, (n, n),
                                       device=self._device).coalesce()

    def to_sparse_csr(self) -> torch.Tensor:
        return self.to_sparse_coo().to_sparse_csr()

    def to_sparse_csr_cached(self) -> torch.Tensor:
        key = ("csr", self._diag._version, self._lower._version, self._upper._version)
        hit = self._csr_cache.get(key)
        if hit is None:
            hit = self.to_sparse_csr()
            self._csr_cache[key] = hit
        return hit

    def Ax_sparse(self, x: torch.Tensor) -> torch.Tensor:
        """y = A x for (n_cells,) or (n_cells, k) x, column by column through
        the Amul kernel (the reference's CSR product,
        core/ldu_matrix.py:349-366)."""
        assert_floating(x, "x")
        if x.dim() == 1:
            return self.Ax(x)
        return torch.stack([self.Ax(x[:, j]) for j in range(x.shape[1])], dim=1)

    def Ax_batched(self, x: torch.Tensor) -> torch.Tensor:
        return self.Ax_sparse(x)

    def invalidate_cache(self) -> None:
        """Drop every derived array cached on this matrix: the packed
        FP64/FP32 coefficients and the factorised DIC/DILU diagonals all live
        in ``_csr_cache``, so the next solve re-packs and re-factorises.  The
        setters and in-place edits already invalidate entries through the
        coefficients' version counters; a caller calls this to force that
        work (a benchmark timing the whole solve, or a matrix whose storage
        was overwritten through another alias)."""
        self._csr_cache.clear()

    def __repr__(self) -> str:
        return (
            f"LduMatrix(n_cells={self._n_cells}, n_internal_faces={self._n_internal_faces}, "
            f"device={self._device}, dtype={self._dtype})"
        )
