"""Algebraic multigrid on the GPU, drop-in for ``pyfoam.solvers.gamg.
GAMGSolver`` (``src/pyfoam/solvers/gamg.py:104-585``).

The reference's method, step for step:

* hierarchy: greedy aggregation in cell order (target half the cells,
  at least ``min_cells_coarse``), coarse diagonal = aggregate sums of the
  fine diagonal, coarse lower/upper = sums over the fine faces between two
  aggregates (faces inside an aggregate are dropped), until
  ``max_levels`` levels or ``min_cells_coarse`` cells or no reduction;
* V-cycle: ``n_pre_smooth`` Jacobi sweeps x += D^-1 (b - A x), residual,
  restriction by aggregate sums, recursive coarse correction from zero,
  prolongation by injection, ``n_post_smooth`` sweeps; 50 Jacobi sweeps on
  the coarsest level;
* outer loop: V-cycles from the given x, the residual checked after each
  (the first check is after the first cycle, as in the reference).

The aggregation and the coarse face lists depend only on the mesh topology:
they are built once on the host (``gbf_gamg_aggregate``,
``gbf_gamg_coarse_faces``) and cached.  Everything that touches
coefficients or vectors -- coarse coefficients, residuals, smoothing,
restriction, prolongation, norms -- runs as libgbfoam kernels with the
reference's summation orders, so x is bitwise the reference's for the same
number of cycles.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from .. import _lib
from ..core.ldu_matrix import LduMatrix
from .linear_solver import LinearSolverBase
from .residual import ConvergenceInfo, ResidualMonitor
from .smoothers import relax, residual

__all__ = ["GAMGSolver", "GAMGLevel", "AggregationData"]


@dataclass
class AggregationData:
    """Fine -> coarse map of one level (reference ``AggregationData``) plus
    the device lists the transfer kernels use."""

    n_coarse: int
    fine_to_coarse: torch.Tensor      # int64 [n_fine] (reference dtype)
    f2c32: torch.Tensor               # int32 [n_fine]
    agg_ptr: torch.Tensor             # int32 [n_coarse + 1]
    agg_cells: torch.Tensor           # int32 [n_fine], fine cells per aggregate ascending
    cf_ptr: torch.Tensor              # int32 [n_cfaces + 1]
    cf_faces: torch.Tensor            # int32, fine faces per coarse face ascending
    coarse_owner: np.ndarray          # int64 [n_cfaces]
    coarse_neighbour: np.ndarray      # int64 [n_cfaces]


@dataclass
class GAMGLevel:
    """One level's matrix (reference ``GAMGLevel`` fields via ``matrix``)."""

    matrix: LduMatrix

    @property
    def n_cells(self) -> int:
        return self.matrix.n_cells

    @property
    def diag(self) -> torch.Tensor:
        return self.matrix.diag

    @property
    def lower(self) -> torch.Tensor:
        return self.matrix.lower

    @property
    def upper(self) -> torch.Tensor:
        return self.matrix.upper

    @property
    def owner(self) -> torch.Tensor:
        return self.matrix.owner

    @property
    def neighbour(self) -> torch.Tensor:
        return self.matrix.neighbour


def _csr(keys: np.ndarray, n_keys: int) -> tuple[np.ndarray, np.ndarray]:
    """(ptr, members): members of each key in ascending member order."""
    valid = keys >= 0
    idx = np.flatnonzero(valid).astype(np.int64)
    k = keys[valid].astype(np.int64)
    order = np.argsort(k, kind="stable")
    ptr = np.zeros(n_keys + 1, np.int64)
    np.add.at(ptr, k + 1, 1)
    np.cumsum(ptr, out=ptr)
    return ptr.astype(np.int32), idx[order].astype(np.int32)


def _aggregate(topo, n_target: int, dev) -> AggregationData | None:
    n, nf = topo.n_cells, topo.n_faces
    L = _lib.lib()
    f2c = np.empty(max(n, 1), np.int32)
    nc = ctypes.c_int32()
    _lib.check(L.gbf_gamg_aggregate(n, nf, topo._own_h.ctypes.data, topo._nei_h.ctypes.data,
                                    int(n_target), f2c.ctypes.data, ctypes.byref(nc)),
               "gbf_gamg_aggregate")
    f2c = f2c[:n]
    if nc.value >= n:
        return None
    co = np.empty(max(nf, 1), np.int32)
    cn = np.empty(max(nf, 1), np.int32)
    f2cf = np.empty(max(nf, 1), np.int32)
    ncf = ctypes.c_int32()
    _lib.check(L.gbf_gamg_coarse_faces(nf, topo._own_h.ctypes.data, topo._nei_h.ctypes.data,
                                       f2c.ctypes.data, co.ctypes.data, cn.ctypes.data,
                                       f2cf.ctypes.data, ctypes.byref(ncf)),
               "gbf_gamg_coarse_faces")
    agg_ptr, agg_cells = _csr(f2c, nc.value)
    cf_ptr, cf_faces = _csr(f2cf[:nf], ncf.value)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a) if a.size  # noqa: E731
                                    else np.zeros(1, a.dtype)).to(dev)
    return AggregationData(
        n_coarse=nc.value, fine_to_coarse=torch.from_numpy(f2c.astype(np.int64)).to(dev),
        f2c32=to(f2c), agg_ptr=to(agg_ptr), agg_cells=to(agg_cells), cf_ptr=to(cf_ptr),
        cf_faces=to(cf_faces), coarse_owner=co[: ncf.value].astype(np.int64),
        coarse_neighbour=cn[: ncf.value].astype(np.int64))


class GAMGSolver(LinearSolverBase):
    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, max_iter: int = 100,
                 min_iter: int = 0, verbose: bool = False, n_pre_smooth: int = 2,
                 n_post_smooth: int = 2, max_levels: int = 10, min_cells_coarse: int = 10,
                 smoother: str = "PCG", *, use_graph: bool = True) -> None:
        super().__init__(tolerance=tolerance, rel_tol=rel_tol, max_iter=max_iter,
                         min_iter=min_iter, verbose=verbose)
        self._n_pre_smooth = n_pre_smooth
        self._n_post_smooth = n_post_smooth
        self._max_levels = max_levels
        self._min_cells_coarse = min_cells_coarse
        self._smoother_type = smoother.upper()  # stored; the reference smooths with Jacobi
        self._use_graph = bool(use_graph)
        self.last_levels: list[GAMGLevel] = []

    # ------------------------------------------------------------------
    def _hierarchy(self, matrix: LduMatrix):
        """Levels (fine first) and aggregations; the topology part is cached
        on the fine topology, the coefficients on the matrix."""
        dev = matrix.device
        key = ("gamg", self._max_levels, self._min_cells_coarse, matrix.diag.data_ptr(),
               matrix.diag._version, matrix.lower.data_ptr(), matrix.lower._version,
               matrix.upper.data_ptr(), matrix.upper._version)
        hit = matrix._csr_cache.get(key)
        if hit is not None:
            return hit
        topo_cache = matrix.topology().__dict__.setdefault("_gamg", {})
        tkey = (self._max_levels, self._min_cells_coarse)
        aggs_topo = topo_cache.get(tkey)
        levels = [GAMGLevel(matrix)]
        aggs: list[AggregationData] = []
        build_topo = aggs_topo is None
        if build_topo:
            aggs_topo = []
        L = _lib.lib()
        st = _lib.stream_ptr(dev)
        cur = matrix
        for lvl in range(self._max_levels):
            if cur.n_cells <= self._min_cells_coarse:
                break
            if build_topo:
                agg = _aggregate(cur.topology(), max(cur.n_cells // 2, self._min_cells_coarse),
                                 dev)
                if agg is None:
                    break
                aggs_topo.append(agg)
            else:
                if lvl >= len(aggs_topo):
                    break
                agg = aggs_topo[lvl]
            nc, ncf = agg.n_coarse, agg.coarse_owner.shape[0]
            coarse = LduMatrix(nc, torch.from_numpy(agg.coarse_owner),
                               torch.from_numpy(agg.coarse_neighbour), device=dev)
            d = torch.empty(max(nc, 1), device=dev, dtype=torch.float64)
            lo = torch.empty(max(ncf, 1), device=dev, dtype=torch.float64)
            up = torch.empty(max(ncf, 1), device=dev, dtype=torch.float64)
            _lib.check(L.gbf_gamg_restrict_f64(nc, agg.agg_ptr.data_ptr(),
                                               agg.agg_cells.data_ptr(), cur.diag.data_ptr(),
                                               d.data_ptr(), st), "gbf_gamg_restrict_f64")
            _lib.check(L.gbf_gamg_coarse_coeffs_f64(ncf, agg.cf_ptr.data_ptr(),
                                                    agg.cf_faces.data_ptr(),
                                                    cur.lower.data_ptr(), cur.upper.data_ptr(),
                                                    lo.data_ptr(), up.data_ptr(), st),
                       "gbf_gamg_coarse_coeffs_f64")
            coarse._diag, coarse._lower, coarse._upper = d[:nc], lo[:ncf], up[:ncf]
            aggs.append(agg)
            levels.append(GAMGLevel(coarse))
            cur = coarse
        if build_topo:
            topo_cache[tkey] = aggs_topo
        out = (levels, aggs)
        # one hierarchy (and its captured cycle) per matrix: drop stale ones
        for k in [k for k in matrix._csr_cache if k[0] in ("gamg", "gamg_cycle")]:
            del matrix._csr_cache[k]
        matrix._csr_cache[key] = out
        return out

    @staticmethod
    def _jacobi(m: LduMatrix, x: torch.Tensor, b: torch.Tensor, n_it: int,
                r: torch.Tensor) -> None:
        for _ in range(n_it):
            residual(m, b, x, r)
            relax(x, r, 1.0, m.diag)

    def _v_cycle(self, levels, aggs, i: int, x: torch.Tensor, b: torch.Tensor) -> None:
        m = levels[i].matrix
        r = torch.empty_like(x)
        if i == len(levels) - 1:
            self._jacobi(m, x, b, 50, r)
            return
        self._jacobi(m, x, b, self._n_pre_smooth, r)
        residual(m, b, x, r)
        agg = aggs[i]
        st = _lib.stream_ptr(m.device)
        L = _lib.lib()
        rc = torch.empty(agg.n_coarse, device=m.device, dtype=torch.float64)
        _lib.check(L.gbf_gamg_restrict_f64(agg.n_coarse, agg.agg_ptr.data_ptr(),
                                           agg.agg_cells.data_ptr(), r.data_ptr(), rc.data_ptr(),
                                           st), "gbf_gamg_restrict_f64")
        ec = torch.zeros_like(rc)
        self._v_cycle(levels, aggs, i + 1, ec, rc)
        _lib.check(L.gbf_gamg_prolong_add_f64(m.n_cells, agg.f2c32.data_ptr(), ec.data_ptr(),
                                              x.data_ptr(), st), "gbf_gamg_prolong_add_f64")
        self._jacobi(m, x, b, self._n_post_smooth, r)

    def _solve(self, matrix: LduMatrix, source: torch.Tensor, x0: torch.Tensor,
               monitor: ResidualMonitor, max_iter: int) -> tuple[torch.Tensor, ConvergenceInfo]:
        if matrix.dtype != torch.float64:
            raise TypeError("GAMGSolver runs on float64 matrices")
        dev, n = matrix.device, matrix.n_cells
        b = source.to(device=dev, dtype=torch.float64).contiguous()
        x = x0.to(device=dev, dtype=torch.float64).clone().contiguous()
        if b.shape[0] != n or x.shape[0] != n:
            raise ValueError(f"source/x0 have {b.shape[0]}/{x.shape[0]} elements, expected {n}")
        levels, aggs = self._hierarchy(matrix)
        self.last_levels = levels
        cyc = self._cycle(matrix, levels, aggs)
        cyc["x"].copy_(x)
        cyc["b"].copy_(b)
        converged = False
        for i in range(1, max_iter + 1):
            cyc["run"]()
            if monitor.check(float(cyc["nrm"].item()), i):
                converged = True
                break
        return cyc["x"].clone(), monitor.build_info(converged=converged)

    def _cycle(self, matrix: LduMatrix, levels, aggs) -> dict:
        """One V-cycle plus the residual norm on static buffers, captured
        once into a CUDA graph per hierarchy (the cycle is a few hundred
        small launches, so replaying the graph removes the per-launch host
        cost); eager launches if capture is off or fails."""
        key = ("gamg_cycle", id(levels))
        hit = matrix._csr_cache.get(key)
        if hit is not None:
            return hit
        dev, n = matrix.device, matrix.n_cells
        L = _lib.lib()
        buf = {"x": torch.zeros(n, device=dev, dtype=torch.float64),
               "b": torch.zeros(n, device=dev, dtype=torch.float64),
               "r": torch.empty(n, device=dev, dtype=torch.float64),
               "ws": torch.empty(int(L.gbf_norm2_workspace_bytes()), device=dev,
                                 dtype=torch.uint8),
               "nrm": torch.empty(1, device=dev, dtype=torch.float64), "levels": levels}

        def body():
            self._v_cycle(levels, aggs, 0, buf["x"], buf["b"])
            residual(matrix, buf["b"], buf["x"], buf["r"])
            _lib.check(L.gbf_norm2_f64(n, buf["r"].data_ptr(), buf["nrm"].data_ptr(),
                                       buf["ws"].data_ptr(), _lib.stream_ptr(dev)),
                       "gbf_norm2_f64")

        buf["run"] = body
        if self._use_graph and n > 0:
            try:
                side = torch.cuda.Stream(device=dev)
                side.wait_stream(torch.cuda.current_stream(dev))
                with torch.cuda.stream(side):
                    body()  # warm-up: module load, occupancy queries, allocator pool
                torch.cuda.current_stream(dev).wait_stream(side)
                torch.cuda.synchronize(dev)
                graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(graph):
                    body()
                buf["graph"] = graph
                buf["run"] = graph.replay
            except RuntimeError:
                buf["run"] = body
        matrix._csr_cache[key] = buf
        return buf
