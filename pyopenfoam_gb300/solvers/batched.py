"""Batched mixed-precision PCG: many independent LDU systems of uneven sizes
solved together, with an autotuner for the launch shape.

No reference counterpart (the reference solves one system per call).  The
systems are concatenated into one block-diagonal matrix -- each system's
cells padded to a multiple of 32 with isolated unit-diagonal cells that stay
zero -- so one topology, one DIC factorisation (all systems' wavefront level
l in one launch) and one packed coefficient copy serve the whole batch.  The
solve is ``gbf_batched_mixed_pcg_solve``: per-system scalars and convergence
masks, a chunk of iterations captured in a CUDA graph and replayed.

The autotuner times a short fixed-iteration solve for each (block size,
tile size) candidate and keeps the fastest, caching the choice per
(GPU, total cells, systems, faces) in a JSON file
(``$GBFOAM_AUTOTUNE_CACHE``, default ``~/.cache/pyopenfoam_gb300/autotune.json``).
"""

from __future__ import annotations

import ctypes
import json
import os
import time
from dataclasses import dataclass

import numpy as np
import torch

from .. import _lib
from ..core.ldu_matrix import LduMatrix
from .preconditioners import factor_dic, factor_dilu
from .residual import ConvergenceInfo

__all__ = ["BatchedPCGSolver", "BatchLayout", "autotune_cache_path"]

BLOCK_SIZES = (128, 256, 512)
TILE_CELLS = (1024, 2048, 4096, 8192)
FORMS = {"plain": 0, "graph": 1, "persistent": 2, "persistent_graph": 3}
TUNED_FORMS = ("graph", "persistent")
THREADS_PER_CELL = (1, 2)
#: wavefront grouping of the factorisation -> preconditioners.FACTOR_FORMS:
#: a dataflow walk, one cooperative launch with a grid barrier per level, or
#: one launch per level (the same bits)
WAVEFRONTS = {"flow": "flow", "cooperative": "levels", "per_level": "per_level"}


def autotune_cache_path() -> str:
    return os.environ.get(
        "GBFOAM_AUTOTUNE_CACHE",
        os.path.join(os.path.expanduser("~"), ".cache", "pyopenfoam_gb300", "autotune.json"))


@dataclass
class _Tiles:
    cells: int
    tensors: tuple
    struct: _lib.Batch


class BatchLayout:
    """Block-diagonal concatenation of systems sharing one device."""

    def __init__(self, matrices: list[LduMatrix]) -> None:
        if not matrices:
            raise ValueError("empty batch")
        dev = matrices[0].device
        for m in matrices:
            if m.device != dev or m.dtype != torch.float64:
                raise ValueError("batched systems must be float64 on one device")
        self.device = dev
        self.sizes = [m.n_cells for m in matrices]
        self.padded = [(n + 31) // 32 * 32 for n in self.sizes]
        self.offsets = np.concatenate([[0], np.cumsum(self.padded)]).astype(np.int64)
        self.n_cells = int(self.offsets[-1])
        own = [m.owner + int(o) for m, o in zip(matrices, self.offsets[:-1])]
        nei = [m.neighbour + int(o) for m, o in zip(matrices, self.offsets[:-1])]
        self.owner = torch.cat(own).contiguous()
        self.neighbour = torch.cat(nei).contiguous()
        self.matrix = LduMatrix(self.n_cells, self.owner, self.neighbour, device=dev)
        self.matrix.topology()
        self._tiles: dict[int, _Tiles] = {}
        pad = torch.zeros(self.n_cells, dtype=torch.bool, device=dev)
        for n, o, p in zip(self.sizes, self.offsets[:-1], self.padded):
            pad[int(o) + n:int(o) + p] = True
        self.pad_mask = pad

    def tiles(self, tile_cells: int) -> _Tiles:
        hit = self._tiles.get(tile_cells)
        if hit is None:
            sys_, beg, end, t0 = [], [], [], [0]
            for s, (o, p) in enumerate(zip(self.offsets[:-1], self.padded)):
                for b0 in range(int(o), int(o) + p, tile_cells):
                    sys_.append(s)
                    beg.append(b0)
                    end.append(min(b0 + tile_cells, int(o) + p))
                t0.append(len(sys_))
            to = lambda a: torch.tensor(a, dtype=torch.int32, device=self.device)  # noqa: E731
            ts = (to(sys_), to(beg), to(end), to(t0))
            st = _lib.Batch(len(self.sizes), len(sys_), *(t.data_ptr() for t in ts))
            hit = _Tiles(tile_cells, ts, st)
            self._tiles[tile_cells] = hit
        return hit

    def set_coefficients(self, matrices: list[LduMatrix]) -> None:
        dev = self.device
        diags, lows, ups = [], [], []
        for m, n, p in zip(matrices, self.sizes, self.padded):
            diags.append(m.diag)
            if p > n:
                diags.append(torch.ones(p - n, dtype=torch.float64, device=dev))
            lows.append(m.lower)
            ups.append(m.upper)
        self.matrix.diag = torch.cat(diags)
        self.matrix.lower = torch.cat(lows)
        self.matrix.upper = torch.cat(ups)

    def gather(self, vectors: list[torch.Tensor]) -> torch.Tensor:
        out = torch.zeros(self.n_cells, dtype=torch.float64, device=self.device)
        for v, n, o in zip(vectors, self.sizes, self.offsets[:-1]):
            out[int(o):int(o) + n] = v.to(device=self.device, dtype=torch.float64)
        return out

    def scatter(self, x: torch.Tensor) -> list[torch.Tensor]:
        return [x[int(o):int(o) + n] for n, o in zip(self.sizes, self.offsets[:-1])]


class BatchedPCGSolver:
    """PCG + DIC (or DILU / none) on a batch of independent systems, FP32
    inner iterations with FP64 reliable updates, all systems per launch.

    ``solve(matrices, sources, x0s=None)`` returns a list of
    ``(x, iterations, final_residual)``, one per system, with the same
    conventions as the single-system solvers; ``last_infos`` holds the
    per-system ConvergenceInfo.  ``form`` is one of ``FORMS`` or None (the
    autotuner chooses; ``use_graph=False`` means ``"plain"``)."""

    def __init__(self, tolerance: float = 1e-6, rel_tol: float = 0.01, max_iter: int = 1000,
                 min_iter: int = 0, preconditioner: str = "DIC", *, delta: float = 0.1,
                 block_size: int | None = None, tile_cells: int | None = None,
                 use_graph: bool = True, autotune: bool = True, check_every: int = 16,
                 form: str | None = None, wavefront: str | None = None,
                 threads_per_cell: int | None = None) -> None:
        self.tolerance, self.rel_tol = float(tolerance), float(rel_tol)
        self.max_iter, self.min_iter = int(max_iter), int(min_iter)
        self.precond = preconditioner.upper()
        if self.precond not in ("DIC", "DILU", "NONE"):
            raise ValueError(f"Unknown preconditioner '{preconditioner}'. Use 'DIC', 'DILU', "
                             "or 'none'.")
        if form is not None and form not in FORMS:
            raise ValueError(f"form must be one of {sorted(FORMS)}, got {form!r}")
        if wavefront is not None and wavefront not in WAVEFRONTS:
            raise ValueError(f"wavefront must be one of {tuple(WAVEFRONTS)} or None")
        if threads_per_cell not in (None, 1, 2):
            raise ValueError("threads_per_cell must be 1, 2 or None")
        self.threads_per_cell = threads_per_cell
        self.delta = float(delta)
        self.block_size, self.tile_cells = block_size, tile_cells
        self.form = form if form is not None else (None if use_graph else "plain")
        self.wavefront = wavefront
        self.autotune = bool(autotune)
        self.check_every = int(check_every)
        self._layouts: dict = {}
        self.last_infos: list[ConvergenceInfo] = []
        self.last_results: list = []
        self.last_config: dict = {}

    # ------------------------------------------------------------------
    def layout(self, matrices: list[LduMatrix]) -> BatchLayout:
        key = tuple((m.n_cells, m.owner.data_ptr(), m.owner._version, m.neighbour.data_ptr(),
                     m.neighbour._version) for m in matrices)
        hit = self._layouts.get(key)
        if hit is None:
            hit = BatchLayout(matrices)
            self._layouts = {key: hit}
        return hit

    def _factor(self, bl: BatchLayout, wavefront: str) -> torch.Tensor | None:
        """The FP64 DIC/DILU diagonal of the batch matrix, cached on it; its
        wavefront runs as a dataflow walk, as one cooperative launch with a
        grid barrier per level, or as one launch per level (same bits)."""
        if self.precond == "NONE":
            return None
        m = bl.matrix
        key = ("batched_factor", self.precond)
        hit = m._csr_cache.get(key)
        if hit is not None and hit[0] == (m.diag._version, m.lower._version, m.upper._version,
                                          m.diag.data_ptr(), m.lower.data_ptr(),
                                          m.upper.data_ptr()):
            return hit[1]
        d = self._build_factor(bl, wavefront)
        m._csr_cache[key] = ((m.diag._version, m.lower._version, m.upper._version,
                              m.diag.data_ptr(), m.lower.data_ptr(), m.upper.data_ptr()), d)
        return d

    def _build_factor(self, bl: BatchLayout, wavefront: str) -> torch.Tensor:
        m = bl.matrix
        topo = m.topology()
        d = torch.empty(m.n_cells, device=bl.device, dtype=torch.float64)
        if self.precond == "DIC":
            factor_dic(topo, m.packed(), m.diag, d, bl.device, WAVEFRONTS[wavefront])
        else:
            factor_dilu(topo, m.lower, m.upper, m.diag, d, bl.device, WAVEFRONTS[wavefront])
        return d

    def _run(self, bl: BatchLayout, b: torch.Tensor, x: torch.Tensor, block: int, tile: int,
             max_iter: int, tol: float, rel: float, form: str, wavefront: str, tpc: int = 1):
        m = bl.matrix
        topo = m.topology()
        pre = self._factor(bl, wavefront)
        coef64 = m.packed()
        coef32 = m.packed(dtype=torch.float32)
        T = bl.tiles(tile)
        L = _lib.lib()
        S = len(bl.sizes)
        ws = torch.empty(int(L.gbf_batched_mixed_pcg_workspace_bytes(m.n_cells, S,
                                                                     T.struct.n_tiles)),
                         dtype=torch.uint8, device=bl.device)
        P = _lib.SolveParams(tol, rel, int(max_iter), self.min_iter, self.check_every, 0)
        R = (_lib.SolveResult * S)()
        _lib.check(L.gbf_batched_mixed_pcg_solve(
            topo.layout_ref, ctypes.byref(T.struct), coef64.data_ptr(), m.diag.data_ptr(),
            coef32.data_ptr(), None if pre is None else pre.data_ptr(), b.data_ptr(),
            x.data_ptr(), self.delta, ctypes.byref(P), int(block),
            FORMS[form] | (4 if tpc == 2 else 0), R,
            ws.data_ptr(), ws.numel(), _lib.stream_ptr(bl.device)), "gbf_batched_mixed_pcg_solve")
        return list(R)

    def _timed(self, fn, reps: int = 2) -> float:
        times = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        return min(times)

    def _tune(self, bl: BatchLayout, b: torch.Tensor) -> dict:
        fixed = {"block": self.block_size, "tile": self.tile_cells, "form": self.form,
                 "wavefront": self.wavefront, "tpc": self.threads_per_cell}
        if all(v is not None for v in fixed.values()):
            return fixed
        name = torch.cuda.get_device_name(bl.device)
        key = (f"{name}|{bl.n_cells}|{len(bl.sizes)}|{bl.matrix.n_internal_faces}|"
               f"{self.precond}")
        path = autotune_cache_path()
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
        hit = cache.get(key)
        if hit is not None and all(k in hit for k in fixed):
            return {k: (fixed[k] if fixed[k] is not None else hit[k]) for k in fixed}
        if not self.autotune:
            return {"block": self.block_size or 256, "tile": self.tile_cells or 4096,
                    "form": self.form or "graph", "wavefront": self.wavefront or "flow",
                    "tpc": self.threads_per_cell or 1}
        timings: dict = {}
        # wavefront of the factorisation: both ways once (same bits)
        if self.precond == "NONE":
            wf = self.wavefront or "flow"
        elif self.wavefront is None:
            for w in WAVEFRONTS:
                timings[f"factor_{w}"] = self._timed(lambda w=w: self._build_factor(bl, w))
            wf = min(WAVEFRONTS, key=lambda w: timings[f"factor_{w}"])
        else:
            wf = self.wavefront
        forms = [self.form] if self.form else list(TUNED_FORMS)
        blocks = [self.block_size] if self.block_size else list(BLOCK_SIZES)
        tiles = [self.tile_cells] if self.tile_cells else list(TILE_CELLS)
        tpcs = [self.threads_per_cell] if self.threads_per_cell else list(THREADS_PER_CELL)
        x = torch.zeros_like(b)
        best_per_form = {}
        for fm in forms:
            best = None
            for tpc in tpcs:
                for blk in blocks:
                    for tl in tiles:
                        t = self._timed(lambda: (x.zero_(), self._run(bl, b, x, blk, tl, 24, 0.0,
                                                                      0.0, fm, wf, tpc)))
                        timings[f"{fm}:{blk}x{tl}x{tpc}"] = t
                        if best is None or t < best[0]:
                            best = (t, blk, tl, tpc)
            best_per_form[fm] = best
        # the forms differ most once systems finish unevenly: one full solve each
        choice = None
        for fm, (_, blk, tl, tpc) in best_per_form.items():
            if len(best_per_form) > 1:
                t = self._timed(lambda: (x.zero_(), self._run(bl, b, x, blk, tl, self.max_iter,
                                                              self.tolerance, self.rel_tol, fm,
                                                              wf, tpc)), reps=1)
                timings[f"full_solve:{fm}"] = t
            else:
                t = 0.0
            if choice is None or t < choice[0]:
                choice = (t, fm, blk, tl, tpc)
        cfg = {"block": choice[2], "tile": choice[3], "form": choice[1], "wavefront": wf,
               "tpc": choice[4]}
        cache[key] = dict(cfg, timings=timings)
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
        self.last_config["timings"] = timings
        return cfg

    def solve(self, matrices: list[LduMatrix], sources: list[torch.Tensor],
              x0s: list[torch.Tensor] | None = None, tolerance: float | None = None,
              max_iter: int | None = None):
        if len(sources) != len(matrices) or (x0s is not None and len(x0s) != len(matrices)):
            raise ValueError("matrices, sources and x0s must have the same length")
        for m, s in zip(matrices, sources):
            if s.shape[0] != m.n_cells:
                raise ValueError(f"source has {s.shape[0]} elements, expected {m.n_cells}")
        bl = self.layout(matrices)
        bl.set_coefficients(matrices)
        b = bl.gather(sources)
        x = bl.gather(x0s) if x0s is not None else torch.zeros_like(b)
        cfg = self._tune(bl, b)
        self.last_config.update(cfg)
        self.last_config["tiles"] = bl.tiles(cfg["tile"]).struct.n_tiles
        tol = self.tolerance if tolerance is None else float(tolerance)
        mi = self.max_iter if max_iter is None else int(max_iter)
        res = self._run(bl, b, x, cfg["block"], cfg["tile"], mi, tol, self.rel_tol, cfg["form"],
                        cfg["wavefront"], cfg["tpc"])
        self.last_results = res
        self.last_infos = []
        out = []
        for xs, r in zip(bl.scatter(x), res):
            info = ConvergenceInfo(
                converged=r.status == _lib.GBF_CONVERGED, iterations=r.iterations,
                final_residual=r.final_residual, initial_residual=r.initial_residual,
                residual_ratio=(r.final_residual / r.initial_residual
                                if r.initial_residual > 0 else 0.0),
                tolerance=tol, residual_history=[r.initial_residual, r.final_residual])
            self.last_infos.append(info)
            out.append((xs, r.iterations, r.final_residual))
        return out
