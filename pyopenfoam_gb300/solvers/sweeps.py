"""Full DIC / DILU solves M z = r (forward sweep, diagonal scaling, backward
sweep) on the GPU: ``DICPreconditioner.apply_full``
(solvers/preconditioners.py:153-201) and ``DILUPreconditioner.apply_full``
(:290-337), each sweep a wavefront walk (by default a dataflow walk,
``SWEEP_FORMS``) that is bitwise equal to the reference's sequential face
loop."""

from __future__ import annotations

import torch

from .. import _lib
from ..core.dtype import assert_floating

__all__ = ["dic_apply_full", "dilu_apply_full", "SWEEP_FORMS"]

#: How a triangular sweep walks its level schedule (the same bits): "flow" --
#: one cooperative launch in which a face waits only on the values it reads
#: (gbf_sweep_flow_f64); "levels" -- one cooperative launch with a grid
#: barrier per level; "per_level" -- a launch per level.
SWEEP_FORMS = ("flow", "levels", "per_level")


def _sweep(topo, coef: torch.Tensor, d: torch.Tensor, z: torch.Tensor, reverse: bool,
           lower_only: bool, form: str) -> None:
    L, dev = _lib.lib(), z.device
    st = _lib.stream_ptr(dev)
    sch = topo.sweep_schedule(reverse, lower_only)
    if form == "flow":
        n_items, links = topo.sweep_flow_links(reverse, lower_only)
        if n_items == 0:
            return
        slots = torch.empty(n_items, dtype=torch.float64, device=dev)
        _lib.check(L.gbf_sweep_flow_f64(topo.layout_ref, coef.data_ptr(), d.data_ptr(),
                                        sch.items.data_ptr(), n_items, links.prev.data_ptr(),
                                        links.cell_last.data_ptr(), int(reverse), z.data_ptr(),
                                        slots.data_ptr(), _lib.wavefront_barrier(dev).data_ptr(),
                                        st), "gbf_sweep_flow_f64")
        return
    # one barrier buffer per sweep: the two sweeps are stream-ordered, but a
    # buffer is never shared between calls that could be in flight together
    bar = _lib.wavefront_barrier(dev) if form == "levels" else None
    _lib.check(L.gbf_sweep_f64(topo.layout_ref, coef.data_ptr(), d.data_ptr(), sch.ptr.data_ptr(),
                               sch.items.data_ptr(), sch.n_levels, sch.max_level_size,
                               int(reverse), z.data_ptr(), None if bar is None else bar.data_ptr(),
                               st), "gbf_sweep_f64")


def _apply_full(pre, r: torch.Tensor, lower_only: bool, back_coef: torch.Tensor,
                form: str = "flow"):
    if form not in SWEEP_FORMS:
        raise ValueError(f"form must be one of {SWEEP_FORMS}, got {form!r}")
    assert_floating(r, "r")
    m = pre._matrix
    if m.dtype != torch.float64:
        raise TypeError("apply_full runs on float64 matrices")
    dev = m.device
    z = r.to(device=dev, dtype=torch.float64).clone().contiguous()
    if z.shape[0] != m.n_cells:
        raise ValueError(f"r has {z.shape[0]} elements, expected {m.n_cells}")
    topo = m.topology()
    d = pre.precond_diag.contiguous()
    if m.n_cells == 0:
        return z
    _sweep(topo, m.upper, d, z, False, lower_only, form)
    _lib.check(_lib.lib().gbf_diag_apply_f64(m.n_cells, z.data_ptr(), d.data_ptr(), z.data_ptr(),
                                             _lib.stream_ptr(dev)), "gbf_diag_apply_f64")
    _sweep(topo, back_coef, d, z, True, lower_only, form)
    return z


def dic_apply_full(pre, r: torch.Tensor, form: str = "flow") -> torch.Tensor:
    return _apply_full(pre, r, True, pre._matrix.upper, form)


def dilu_apply_full(pre, r: torch.Tensor, form: str = "flow") -> torch.Tensor:
    return _apply_full(pre, r, False, pre._matrix.lower, form)
