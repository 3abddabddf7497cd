"""DIC and DILU preconditioners on the GPU, drop-in for
``pyfoam.solvers.preconditioners`` (``src/pyfoam/solvers/preconditioners.py``).

The factorised diagonal is built by libgbfoam's wavefront kernels, which
apply the reference's sequential updates in the reference's order, so the
diagonal is bitwise identical:

* DIC (``preconditioners.py:88-133``): cells ascending, for each face into
  the cell (face order) ``d[i] -= a*a / d[j]`` with ``a = upper[f]``;
* DILU (``preconditioners.py:228-272``): faces ascending, both ends updated
  from the values before the face.

By default the wavefront runs as a dataflow walk (``FACTOR_FORMS``): one
cooperative launch in which every step waits only on the values it reads,
with no barrier between levels.

``apply`` is the reference's diagonal-only ``r / d``; ``apply_full`` is the
forward / diagonal / backward sweep pair (``:153-201``, ``:290-337``).
The factorised diagonal is cached on the matrix, keyed by the coefficient
tensors' version counters (the reference rebuilds it on every solve; the
result is the same).
"""

from __future__ import annotations

from typing import Protocol

import torch

from .. import _lib
from ..core.dtype import assert_floating
from ..core.ldu_matrix import LduMatrix

__all__ = ["Preconditioner", "DICPreconditioner", "DILUPreconditioner", "FACTOR_FORMS",
           "factor_dic", "factor_dilu"]

#: How a factorisation walks its level schedule, all giving the same bits:
#: "flow" -- one cooperative launch, every step waiting only on the values it
#: reads (gbf_dic_build_flow_f64 / gbf_dilu_build_flow_f64); "levels" -- one
#: cooperative launch with a grid barrier between levels; "per_level" -- one
#: launch per level.
FACTOR_FORMS = ("flow", "levels", "per_level")


def _check_form(form: str) -> None:
    if form not in FACTOR_FORMS:
        raise ValueError(f"factorisation form must be one of {FACTOR_FORMS}, got {form!r}")


def factor_dic(topo, coef: torch.Tensor, diag: torch.Tensor, d: torch.Tensor, device,
               form: str = "flow") -> None:
    """DIC factorised diagonal of the FP64 matrix (coef = packed slots) into d;
    raises if a bounded wait of a cooperative form ran out."""
    _check_form(form)
    sched = topo.dic_schedule()
    L, st = _lib.lib(), _lib.stream_ptr(device)
    bar = None if form == "per_level" else _lib.wavefront_barrier(device)
    if form == "flow":
        _lib.check(L.gbf_dic_build_flow_f64(topo.layout_ref, coef.data_ptr(), diag.data_ptr(),
                                            sched.items.data_ptr(), d.data_ptr(),
                                            bar.data_ptr(), st), "gbf_dic_build_flow_f64")
    else:
        _lib.check(L.gbf_dic_build_f64(topo.layout_ref, coef.data_ptr(), diag.data_ptr(),
                                       sched.ptr.data_ptr(), sched.items.data_ptr(),
                                       sched.n_levels, sched.max_level_size, d.data_ptr(),
                                       None if bar is None else bar.data_ptr(), st),
                   "gbf_dic_build_f64")
    if bar is not None:
        _lib.check_wavefront(bar, "DIC factorisation", device)


def factor_dilu(topo, lower: torch.Tensor, upper: torch.Tensor, diag: torch.Tensor,
                d: torch.Tensor, device, form: str = "flow") -> None:
    """DILU factorised diagonal of the FP64 matrix into d; raises if a
    bounded wait of a cooperative form ran out."""
    _check_form(form)
    sched = topo.dilu_schedule()
    L, st = _lib.lib(), _lib.stream_ptr(device)
    bar = None if form == "per_level" else _lib.wavefront_barrier(device)
    if form == "flow":
        links = topo.dilu_flow_links()
        slots = torch.empty(max(2 * topo.n_faces, 1), dtype=torch.float64, device=device)
        _lib.check(L.gbf_dilu_build_flow_f64(topo.layout_ref, lower.data_ptr(), upper.data_ptr(),
                                             diag.data_ptr(), sched.items.data_ptr(),
                                             links.prev.data_ptr(), links.cell_last.data_ptr(),
                                             slots.data_ptr(), d.data_ptr(), bar.data_ptr(), st),
                   "gbf_dilu_build_flow_f64")
    else:
        _lib.check(L.gbf_dilu_build_f64(topo.layout_ref, lower.data_ptr(), upper.data_ptr(),
                                        diag.data_ptr(), sched.ptr.data_ptr(),
                                        sched.items.data_ptr(), sched.n_levels,
                                        sched.max_level_size, d.data_ptr(),
                                        None if bar is None else bar.data_ptr(), st),
                   "gbf_dilu_build_f64")
    if bar is not None:
        _lib.check_wavefront(bar, "DILU factorisation", device)


class Preconditioner(Protocol):
    def apply(self, r: torch.Tensor) -> torch.Tensor: ...


def _as_f64_matrix(matrix: LduMatrix):
    """FP64 views of the coefficients (float32 matrices factorise in FP64 and
    round the factorised diagonal once at the end)."""
    if matrix.dtype == torch.float64:
        return matrix, matrix.diag, matrix.lower, matrix.upper
    m64 = LduMatrix(matrix.n_cells, matrix.owner, matrix.neighbour, device=matrix.device,
                    dtype=torch.float64)
    m64._topology = matrix.topology()
    m64.diag, m64.lower, m64.upper = matrix.diag, matrix.lower, matrix.upper
    return m64, m64.diag, m64.lower, m64.upper


class _DiagonalFactor:
    kind = ""
    #: walk of the factorisation (one of FACTOR_FORMS; the same bits)
    factor_form = "flow"

    def __init__(self, matrix: LduMatrix) -> None:
        self._matrix = matrix
        self._device = matrix.device
        self._dtype = matrix.dtype
        key = (self.kind, matrix.diag.data_ptr(), matrix.diag._version, matrix.lower.data_ptr(),
               matrix.lower._version, matrix.upper.data_ptr(), matrix.upper._version)
        hit = matrix._csr_cache.get(key)
        if hit is None:
            hit = self._build()
            for k in [k for k in matrix._csr_cache if k[0] == self.kind]:
                del matrix._csr_cache[k]
            matrix._csr_cache[key] = hit
        self._precond_diag = hit

    @property
    def precond_diag(self) -> torch.Tensor:
        return self._precond_diag

    def _build(self) -> torch.Tensor:  # pragma: no cover - abstract
        raise NotImplementedError

    def apply(self, r: torch.Tensor) -> torch.Tensor:
        """z = r / d_factored (preconditioners.py:135-151, :274-288)."""
        assert_floating(r, "r")
        r = r.to(device=self._device, dtype=self._dtype).contiguous()
        if self._dtype == torch.float64:
            z = torch.empty_like(r)
            _lib.check(_lib.lib().gbf_diag_apply_f64(r.shape[0], r.data_ptr(),
                                                     self._precond_diag.data_ptr(), z.data_ptr(),
                                                     _lib.stream_ptr(self._device)),
                       "gbf_diag_apply_f64")
            return z
        return r / self._precond_diag


class DICPreconditioner(_DiagonalFactor):
    """Diagonal incomplete Cholesky (preconditioners.py:62-201)."""

    kind = "DIC"

    def _build(self) -> torch.Tensor:
        m64, diag, _, _ = _as_f64_matrix(self._matrix)
        topo = self._matrix.topology()
        d = torch.empty(self._matrix.n_cells, device=self._device, dtype=torch.float64)
        if self._matrix.n_cells == 0:
            return d.to(self._dtype)
        factor_dic(topo, m64.packed(), diag, d, self._device, self.factor_form)
        return d.to(self._dtype)

    def apply_full(self, r: torch.Tensor) -> torch.Tensor:
        """Forward (D+L) sweep, diagonal scaling, backward (D+U) sweep
        (preconditioners.py:153-201)."""
        from .sweeps import dic_apply_full

        return dic_apply_full(self, r)


class DILUPreconditioner(_DiagonalFactor):
    """Diagonal incomplete LU (preconditioners.py:204-337)."""

    kind = "DILU"

    def _build(self) -> torch.Tensor:
        m64, diag, lower, upper = _as_f64_matrix(self._matrix)
        topo = self._matrix.topology()
        d = torch.empty(self._matrix.n_cells, device=self._device, dtype=torch.float64)
        if self._matrix.n_cells == 0:
            return d.to(self._dtype)
        factor_dilu(topo, lower, upper, diag, d, self._device, self.factor_form)
        return d.to(self._dtype)

    def apply_full(self, r: torch.Tensor) -> torch.Tensor:
        """Forward sweep with upper, diagonal scaling, backward sweep with
        lower (preconditioners.py:290-337)."""
        from .sweeps import dilu_apply_full

        return dilu_apply_full(self, r)
