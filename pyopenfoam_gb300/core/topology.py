"""Mesh-topology data shared by every matrix on the same owner/neighbour
addressing: the cell-sliced slot layout and the DIC / DILU wavefront
schedules.

Built once on the host (libgbfoam ``gbf_layout_*``, ``gbf_*_schedule``) and
kept on the device.  The reference rebuilds its per-cell face lists on every
preconditioner construction (``solvers/preconditioners.py:116-122``) and
caches a CSR copy per matrix (``core/ldu_matrix.py:101-102``); here one
topology object is cached per addressing and shared by all matrices on it.
"""

from __future__ import annotations

import ctypes
from collections import OrderedDict
from dataclasses import dataclass

import numpy as np
import torch

from .._lib import Layout, check, lib

__all__ = ["Topology", "get_topology", "Schedule", "FlowLinks"]


@dataclass
class Schedule:
    """Wavefront levels: items of level l are items[ptr[l]:ptr[l+1]]."""

    ptr: torch.Tensor
    items: torch.Tensor
    n_levels: int
    max_level_size: int


@dataclass
class FlowLinks:
    """Dataflow DILU links: prev[2i], prev[2i+1] = slots holding face item
    i's owner / neighbour value before it (-1: the diagonal); cell_last[c] =
    slot of cell c's last face (-1: none)."""

    prev: torch.Tensor
    cell_last: torch.Tensor


def _i32_host(t: torch.Tensor, n_cells: int, name: str) -> np.ndarray:
    a = t.detach().to("cpu", torch.int64).numpy()
    if a.size and (a.min() < 0 or a.max() >= n_cells):
        raise ValueError(f"{name} holds a cell index outside [0, {n_cells})")
    return np.ascontiguousarray(a, dtype=np.int32)


class Topology:
    """Device-resident slot layout of one owner/neighbour addressing."""

    #: use the per-slice column-offset compression in the gather kernels
    compress = True
    #: pad all slices to one width when that costs at most this many percent
    #: more slots (-1: never)
    uniform_pad_pct = 5

    def __init__(self, n_cells: int, owner: torch.Tensor, neighbour: torch.Tensor) -> None:
        if n_cells < 0 or n_cells >= 2**31:
            raise ValueError(f"n_cells={n_cells} outside [0, 2^31)")
        if owner.shape[0] != neighbour.shape[0]:
            raise ValueError(
                f"owner has {owner.shape[0]} faces, neighbour has {neighbour.shape[0]}"
            )
        dev = owner.device
        self.device = dev
        self.n_cells = int(n_cells)
        self.n_faces = int(neighbour.shape[0])
        self._own_h = _i32_host(owner, n_cells, "owner")
        self._nei_h = _i32_host(neighbour, n_cells, "neighbour")
        L = lib()
        ns, nslots, mw, uni = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
        check(
            L.gbf_layout_plan(self.n_cells, self.n_faces, self._own_h.ctypes.data,
                              self._nei_h.ctypes.data, self.uniform_pad_pct, ctypes.byref(ns),
                              ctypes.byref(nslots), ctypes.byref(mw), ctypes.byref(uni)),
            "gbf_layout_plan",
        )
        self.uniform = bool(uni.value)
        self.n_slices, self.n_slots, self.max_width = ns.value, nslots.value, mw.value
        off = np.empty(self.n_slices + 1, np.int32)
        w = np.empty(max(self.n_slices, 1), np.int32)
        col = np.empty(max(self.n_slots, 1), np.int32)
        face = np.empty(max(self.n_slots, 1), np.int32)
        check(
            L.gbf_layout_fill(self.n_cells, self.n_faces, self._own_h.ctypes.data,
                              self._nei_h.ctypes.data, self.uniform_pad_pct, off.ctypes.data,
                              w.ctypes.data, col.ctypes.data, face.ctypes.data),
            "gbf_layout_fill",
        )
        to = lambda a: torch.from_numpy(a).to(dev)  # noqa: E731
        self.slice_off = to(off)
        self.slice_w = to(w)
        self.slot_col = to(col)
        self.slot_face = to(face)
        self.owner32 = to(self._own_h) if self.n_faces else torch.zeros(1, dtype=torch.int32, device=dev)
        self.neighbour32 = to(self._nei_h) if self.n_faces else torch.zeros(1, dtype=torch.int32, device=dev)
        # offset compression of the columns (identical results, less index traffic)
        nent = max(self.n_slots // 32, 1)
        dm = np.empty(2 * nent, np.int32)
        nu = ctypes.c_int64()
        check(L.gbf_layout_compress(self.n_slices, off.ctypes.data, w.ctypes.data,
                                    col.ctypes.data, dm.ctypes.data, ctypes.byref(nu)),
              "gbf_layout_compress")
        self.n_uniform_entries = nu.value
        self.slot_dm = to(dm)
        uwo = int(w[0] & 0xFFFF) if self.uniform and self.n_slices else 0
        uwn = int(w[0] >> 16) if self.uniform and self.n_slices else 0
        all_uni = int(self.compress and self.n_uniform_entries == self.n_slots // 32)
        # mirror table: lets a symmetric matrix be stored as its owner-side half
        self.slot_mirror = None
        if all_uni and uwo > 0 and self.n_faces > 0:
            mir = np.empty(nent, np.int8)
            ok = ctypes.c_int32()
            check(L.gbf_layout_mirror(self.n_faces, self.n_slices, uwo, uwn, face.ctypes.data,
                                      self._own_h.ctypes.data, dm.ctypes.data, mir.ctypes.data,
                                      ctypes.byref(ok)), "gbf_layout_mirror")
            if ok.value:
                self.slot_mirror = to(mir)
        self.layout = Layout(
            self.n_cells, self.n_faces, self.n_slices, self.max_width, uwo, uwn, all_uni, 0,
            self.n_slots,
            self.slice_off.data_ptr(), self.slice_w.data_ptr(), self.slot_col.data_ptr(),
            self.slot_face.data_ptr(), self.owner32.data_ptr(), self.neighbour32.data_ptr(),
            self.slot_dm.data_ptr() if self.compress else None,
            self.slot_mirror.data_ptr() if self.slot_mirror is not None else None,
        )
        self._dic: Schedule | None = None
        self._dilu: Schedule | None = None
        self._dilu_flow: FlowLinks | None = None
        self._sweeps: dict = {}
        self._sweeps_h: dict = {}
        self._sweep_links: dict = {}

    @property
    def layout_ref(self):
        return ctypes.byref(self.layout)

    def uncompressed_layout(self) -> Layout:
        """The same layout without the offset compression (slot_col only)."""
        L = Layout()
        ctypes.pointer(L)[0] = self.layout
        L.slot_dm = None
        L.all_uniform = 0
        L.slot_mirror = None
        return L

    def variable_width_layout(self) -> Layout:
        """The same layout read through slice_off/slice_w (no fixed-width
        address arithmetic)."""
        L = Layout()
        ctypes.pointer(L)[0] = self.layout
        L.uniform_wo = 0
        L.uniform_wn = 0
        L.all_uniform = 0
        L.slot_mirror = None
        return L

    @property
    def symmetric_storage(self) -> bool:
        """True when the hex 3+3 kernels can read a symmetric matrix from
        its owner-side half (uniform 3+3 compressed layout with a mirror
        table)."""
        return (self.slot_mirror is not None and self.layout.uniform_wo == 3
                and self.layout.uniform_wn == 3 and self.layout.all_uniform == 1)

    def dic_schedule(self) -> Schedule:
        if self._dic is None:
            n = self.n_cells
            ptr = np.empty(n + 1, np.int32)
            cells = np.empty(max(n, 1), np.int32)
            nl, mx = ctypes.c_int32(), ctypes.c_int32()
            check(
                lib().gbf_dic_schedule(n, self.n_faces, self._own_h.ctypes.data,
                                       self._nei_h.ctypes.data, ptr.ctypes.data,
                                       cells.ctypes.data, ctypes.byref(nl), ctypes.byref(mx)),
                "gbf_dic_schedule",
            )
            self._dic = Schedule(torch.from_numpy(ptr[: nl.value + 1].copy()).to(self.device),
                                 torch.from_numpy(cells).to(self.device), nl.value, mx.value)
        return self._dic

    def dilu_schedule(self) -> Schedule:
        if self._dilu is None:
            nf = self.n_faces
            ptr = np.empty(nf + 1, np.int32)
            faces = np.empty(max(nf, 1), np.int32)
            nl, mx = ctypes.c_int32(), ctypes.c_int32()
            check(
                lib().gbf_dilu_schedule(self.n_cells, nf, self._own_h.ctypes.data,
                                        self._nei_h.ctypes.data, ptr.ctypes.data,
                                        faces.ctypes.data, ctypes.byref(nl), ctypes.byref(mx)),
                "gbf_dilu_schedule",
            )
            self._dilu = Schedule(torch.from_numpy(ptr[: nl.value + 1].copy()).to(self.device),
                                  torch.from_numpy(faces).to(self.device), nl.value, mx.value)
            self._dilu_faces_h = faces
        return self._dilu

    def dilu_flow_links(self) -> FlowLinks:
        """Slot links of the dataflow DILU factorisation over
        ``dilu_schedule()`` (see ``gbf_dilu_flow_links``)."""
        if self._dilu_flow is None:
            self.dilu_schedule()
            nf, n = self.n_faces, self.n_cells
            prev = np.empty(max(2 * nf, 1), np.int32)
            last = np.empty(max(n, 1), np.int32)
            check(
                lib().gbf_dilu_flow_links(n, nf, self._own_h.ctypes.data, self._nei_h.ctypes.data,
                                          self._dilu_faces_h.ctypes.data, prev.ctypes.data,
                                          last.ctypes.data),
                "gbf_dilu_flow_links",
            )
            self._dilu_flow = FlowLinks(torch.from_numpy(prev).to(self.device),
                                        torch.from_numpy(last).to(self.device))
        return self._dilu_flow

    def sweep_schedule(self, reverse: bool, lower_only: bool) -> Schedule:
        """Level schedule of one triangular sweep of the full DIC/DILU solve
        (see ``gbf_sweep_schedule``)."""
        key = (bool(reverse), bool(lower_only))
        hit = self._sweeps.get(key)
        if hit is None:
            nf = self.n_faces
            ptr = np.empty(nf + 1, np.int32)
            faces = np.empty(max(nf, 1), np.int32)
            nl, mx = ctypes.c_int32(), ctypes.c_int32()
            check(lib().gbf_sweep_schedule(self.n_cells, nf, self._own_h.ctypes.data,
                                           self._nei_h.ctypes.data, int(reverse),
                                           int(lower_only), ptr.ctypes.data, faces.ctypes.data,
                                           ctypes.byref(nl), ctypes.byref(mx)),
                  "gbf_sweep_schedule")
            hit = Schedule(torch.from_numpy(ptr[: nl.value + 1].copy()).to(self.device),
                           torch.from_numpy(faces).to(self.device), nl.value, mx.value)
            self._sweeps[key] = hit
            self._sweeps_h[key] = (int(ptr[nl.value]) if nl.value > 0 else 0, faces)
        return hit

    def sweep_flow_links(self, reverse: bool, lower_only: bool) -> tuple[int, FlowLinks]:
        """(item count, slot links) of the dataflow form of
        ``sweep_schedule(reverse, lower_only)`` (see ``gbf_sweep_flow_links``)."""
        key = (bool(reverse), bool(lower_only))
        hit = self._sweep_links.get(key)
        if hit is None:
            self.sweep_schedule(reverse, lower_only)
            n_items, faces = self._sweeps_h[key]
            prev = np.empty(max(2 * n_items, 1), np.int32)
            last = np.empty(max(self.n_cells, 1), np.int32)
            check(lib().gbf_sweep_flow_links(self.n_cells, self.n_faces, self._own_h.ctypes.data,
                                             self._nei_h.ctypes.data, int(reverse), n_items,
                                             faces.ctypes.data, prev.ctypes.data,
                                             last.ctypes.data), "gbf_sweep_flow_links")
            hit = (n_items, FlowLinks(torch.from_numpy(prev).to(self.device),
                                      torch.from_numpy(last).to(self.device)))
            self._sweep_links[key] = hit
        return hit


_CACHE: "OrderedDict[tuple, tuple]" = OrderedDict()
_CACHE_SIZE = 8


def get_topology(n_cells: int, owner: torch.Tensor, neighbour: torch.Tensor) -> Topology:
    """Cached Topology of (n_cells, owner, neighbour).

    The key holds the tensors' pointers and in-place version counters; the
    cache entry keeps the tensors alive, so a pointer cannot be recycled
    while its entry exists.
    """
    key = (
        str(owner.device), int(n_cells), owner.data_ptr(), owner.numel(), owner._version,
        neighbour.data_ptr(), neighbour.numel(), neighbour._version,
    )
    hit = _CACHE.get(key)
    if hit is not None:
        _CACHE.move_to_end(key)
        return hit[0]
    topo = Topology(n_cells, owner, neighbour)
    _CACHE[key] = (topo, owner, neighbour)
    while len(_CACHE) > _CACHE_SIZE:
        _CACHE.popitem(last=False)
    return topo
