"""Batched mixed-precision PCG: every system of a batch reaches its
tolerance on its true FP64 residual, agrees with the FP64 oracle, converges
independently (per-system masks), and the CUDA-graph and plain launch paths
give identical bits."""

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyopenfoam_gb300.mesh.batch import poisson_batch
from pyopenfoam_gb300.solvers.batched import BatchedPCGSolver

pytestmark = pytest.mark.gpu


def _np(m):
    return (m.owner.cpu().numpy(), m.neighbour.cpu().numpy(), m.diag.cpu().numpy(),
            m.lower.cpu().numpy(), m.upper.cpu().numpy())


def test_batched_systems_converge_independently(tmp_path, monkeypatch):
    monkeypatch.setenv("GBFOAM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    mats, rhs, sides = poisson_batch(6, lo=6, hi=20, seed=11)
    s = BatchedPCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=3000)
    out = s.solve(mats, rhs)
    assert (tmp_path / "tune.json").exists()  # the autotuner cached its choice
    its = []
    for (x, it, res), m, b, info in zip(out, mats, rhs, s.last_infos):
        assert info.converged
        own, nei, d, lo, up = _np(m)
        bb = b.cpu().numpy()
        xh = x.cpu().numpy()
        r = bb - O.amul(own, nei, d, lo, up, xh)
        tr = np.linalg.norm(r) / np.linalg.norm(bb)
        assert tr < 1e-8
        pd = O.dic_build(own, nei, d, up)
        o = O.pcg(own, nei, d, lo, up, bb, np.zeros_like(bb), pd, 0.0, 1e-12, 20000)
        # |x - x*|/|x*| <= kappa * |r|/|b|: the error is bounded by the system's
        # own true residual (measured on GB300: at most 23x it over these six
        # systems, 1.8e-7 at the largest)
        assert np.linalg.norm(xh - o.x) / np.linalg.norm(o.x) < 50 * tr
        its.append(it)
    assert len(set(its)) > 1  # uneven systems stop at different iterations


@pytest.mark.parametrize("tpc", [1, 2])
@pytest.mark.parametrize("block,tile", [(256, 1024), (128, 2048), (512, 4096)])
def test_batched_forms_give_identical_bits(block, tile, tpc):
    """Graph replay, plain launches, the persistent cooperative launch and the
    persistent launch captured in a graph: the same per-element arithmetic
    and the same per-tile reductions in tile order, so x, the iteration and
    update counts and the residuals agree bit for bit -- also for systems
    that stop at very different iterations (sides 6..24)."""
    mats, rhs, _ = poisson_batch(7, lo=6, hi=24, seed=5)
    ref = None
    for form in ("graph", "plain", "persistent", "persistent_graph"):
        s = BatchedPCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=2000, block_size=block,
                             tile_cells=tile, form=form, wavefront="cooperative",
                             threads_per_cell=tpc)
        xs = [x.cpu().numpy() for x, _, _ in s.solve(mats, rhs)]
        got = (xs, [(r.iterations, r.outer_updates, r.status, r.final_residual)
                    for r in s.last_results])
        assert all(i.converged for i in s.last_infos), form
        if ref is None:
            ref = got
            assert len({r[0] for r in got[1]}) > 1  # uneven stops
            continue
        for u, v in zip(got[0], ref[0]):
            np.testing.assert_array_equal(u, v)
        assert got[1] == ref[1], form


def test_batched_two_threads_per_cell():
    """Two threads per cell split a cell's Amul by side and give its bits;
    the p.Ap partial sums run over other threads, so the solve agrees with
    one thread per cell to rounding -- both reach the tolerance on their
    true residuals, same iteration counts within one or two."""
    mats, rhs, _ = poisson_batch(4, lo=8, hi=20, seed=8)
    out = {}
    for tpc in (1, 2):
        s = BatchedPCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=2000, block_size=256,
                             tile_cells=1024, form="graph", wavefront="cooperative",
                             threads_per_cell=tpc)
        xs = s.solve(mats, rhs)
        assert all(i.converged for i in s.last_infos)
        out[tpc] = (xs, [r.iterations for r in s.last_results])
    for (x1, _, _), (x2, _, _), m, b in zip(out[1][0], out[2][0], mats, rhs):
        own, nei, d, lo, up = _np(m)
        bb = b.cpu().numpy()
        for x in (x1, x2):
            r = bb - O.amul(own, nei, d, lo, up, x.cpu().numpy())
            assert np.linalg.norm(r) / np.linalg.norm(bb) < 1e-8
        assert float(torch.linalg.vector_norm(x1 - x2) / torch.linalg.vector_norm(x1)) < 1e-6
    assert all(abs(a - b) <= 2 for a, b in zip(out[1][1], out[2][1]))
    with pytest.raises(ValueError, match="threads_per_cell"):
        BatchedPCGSolver(threads_per_cell=3)


def test_batched_factor_wavefront_forms_match():
    mats, rhs, _ = poisson_batch(3, lo=8, hi=12, seed=6)
    out = []
    for wf in ("flow", "cooperative", "per_level"):
        s = BatchedPCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=2000, block_size=256,
                             tile_cells=1024, form="graph", wavefront=wf)
        out.append([x.cpu().numpy() for x, _, _ in s.solve(mats, rhs)])
    for u, v, w in zip(*out):
        np.testing.assert_array_equal(u, v)
        np.testing.assert_array_equal(u, w)


def test_batched_persistent_form_against_oracle(tmp_path, monkeypatch):
    monkeypatch.setenv("GBFOAM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    mats, rhs, _ = poisson_batch(5, lo=6, hi=18, seed=12)
    s = BatchedPCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=3000, form="persistent")
    out = s.solve(mats, rhs)
    assert s.last_config["form"] == "persistent"
    for (x, it, res), m, b, info in zip(out, mats, rhs, s.last_infos):
        assert info.converged
        own, nei, d, lo, up = _np(m)
        bb, xh = b.cpu().numpy(), x.cpu().numpy()
        tr = np.linalg.norm(bb - O.amul(own, nei, d, lo, up, xh)) / np.linalg.norm(bb)
        assert tr < 1e-8
        o = O.pcg(own, nei, d, lo, up, bb, np.zeros_like(bb), O.dic_build(own, nei, d, up), 0.0,
                  1e-12, 20000)
        assert np.linalg.norm(xh - o.x) / np.linalg.norm(o.x) < 50 * tr


def test_batched_autotuner_considers_both_forms(tmp_path, monkeypatch):
    monkeypatch.setenv("GBFOAM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    mats, rhs, _ = poisson_batch(3, lo=6, hi=10, seed=7)
    s = BatchedPCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=2000, block_size=256)
    s.solve(mats, rhs)
    t = s.last_config["timings"]
    assert any(k.startswith("graph:") for k in t) and any(k.startswith("persistent:") for k in t)
    assert any(k.endswith("x1") for k in t if ":" in k and not k.startswith("full"))
    assert any(k.endswith("x2") for k in t if ":" in k and not k.startswith("full"))
    assert s.last_config["tpc"] in (1, 2)
    assert "full_solve:graph" in t and "full_solve:persistent" in t
    assert "factor_flow" in t and "factor_cooperative" in t and "factor_per_level" in t
    assert s.last_config["form"] in ("graph", "persistent")


def test_batched_matches_single_system_solver_closely():
    from pyopenfoam_gb300 import MixedPrecisionPCGSolver

    mats, rhs, _ = poisson_batch(3, lo=10, hi=14, seed=2)
    bs = BatchedPCGSolver(tolerance=0.0, rel_tol=1e-10, max_iter=3000, block_size=128,
                          tile_cells=2048)
    out = bs.solve(mats, rhs)
    single = MixedPrecisionPCGSolver(tolerance=0.0, rel_tol=1e-10, max_iter=3000)
    for (x, it, _), m, b in zip(out, mats, rhs):
        xs, its, _ = single(m, b, torch.zeros_like(b))
        assert abs(it - its) <= 0.1 * its + 3
        assert torch.linalg.vector_norm(x - xs) / torch.linalg.vector_norm(xs) < 1e-7
