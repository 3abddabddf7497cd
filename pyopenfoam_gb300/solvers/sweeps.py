"""Full DIC / DILU solves M z = r (forward sweep, diagonal scaling, backward
sweep) on the GPU: ``DICPreconditioner.apply_full``
(solvers/preconditioners.py:153-201) and ``DILUPreconditioner.apply_full``
(:290-337), each sweep a level-scheduled wavefront that is bitwise equal to
the reference's sequential face loop."""

from __future__ import annotations

import torch

from .. import _lib
from ..core.dtype import assert_floating

__all__ = ["dic_apply_full", "dilu_apply_full"]


def _apply_full(pre, r: torch.Tensor, lower_only: bool, back_coef: torch.Tensor):
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
    L = _lib.lib()
    st = _lib.stream_ptr(dev)
    if m.n_cells == 0:
        return z
    fwd = topo.sweep_schedule(False, lower_only)
    # one barrier buffer per sweep: the two sweeps are stream-ordered, but a
    # buffer is never shared between calls that could be in flight together
    _lib.check(L.gbf_sweep_f64(topo.layout_ref, m.upper.data_ptr(), d.data_ptr(),
                               fwd.ptr.data_ptr(), fwd.items.data_ptr(), fwd.n_levels,
                               fwd.max_level_size, 0, z.data_ptr(),
                               _lib.wavefront_barrier(m.device).data_ptr(), st), "gbf_sweep_f64")
    _lib.check(L.gbf_diag_apply_f64(m.n_cells, z.data_ptr(), d.data_ptr(), z.data_ptr(), st),
               "gbf_diag_apply_f64")
    bwd = topo.sweep_schedule(True, lower_only)
    _lib.check(L.gbf_sweep_f64(topo.layout_ref, back_coef.data_ptr(), d.data_ptr(),
                               bwd.ptr.data_ptr(), bwd.items.data_ptr(), bwd.n_levels,
                               bwd.max_level_size, 1, z.data_ptr(),
                               _lib.wavefront_barrier(m.device).data_ptr(), st), "gbf_sweep_f64")
    return z


def dic_apply_full(pre, r: torch.Tensor) -> torch.Tensor:
    return _apply_full(pre, r, True, pre._matrix.upper)


def dilu_apply_full(pre, r: torch.Tensor) -> torch.Tensor:
    return _apply_full(pre, r, False, pre._matrix.lower)
