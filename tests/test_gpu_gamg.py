"""GAMGSolver on the GPU against the reference's own GAMGSolver
(tests/golden/reference_gamg.npz, make_golden.py --gamg): the aggregation
maps and coarse matrices of every level bitwise, and x bitwise after four
V-cycles (the same iteration count; the residual norm to 1e-13 relative)."""

import os

import numpy as np
import pytest
import torch

from pyopenfoam_gb300 import LduMatrix, create_solver
from pyopenfoam_gb300.solvers import GAMGSolver
from tests.golden.cases import c1_poisson, hex_poisson, random_ldu

pytestmark = pytest.mark.gpu
GM = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_gamg.npz"))


def _case(tag):
    c = c1_poisson(6, seed=4) if tag == "poi" else random_ldu(5, seed=41, permute_faces=True)
    if tag == "rnd":
        c["b"] = c["r"]
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(c[k]) for k in ("diag", "lower", "upper"))
    return m, torch.as_tensor(c["b"])


def _eq(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and (a.view(np.int64) == b.view(np.int64)).all()


@pytest.mark.parametrize("tag", ["poi", "rnd"])
def test_gamg_matches_reference(tag):
    m, b = _case(tag)
    s = GAMGSolver(tolerance=0.0, rel_tol=0.0, max_iter=4, min_cells_coarse=10)
    x, it, res = s(m, b, torch.zeros_like(b))
    sizes = GM[f"{tag}_sizes"].tolist()
    assert [lv.n_cells for lv in s.last_levels][: len(sizes)] == sizes
    for lvl in range(len(sizes) - 1):
        cl = s.last_levels[lvl + 1].matrix
        assert np.array_equal(cl.owner.cpu().numpy(), GM[f"{tag}_L{lvl + 1}_owner"])
        assert np.array_equal(cl.neighbour.cpu().numpy(), GM[f"{tag}_L{lvl + 1}_neighbour"])
        for k in ("diag", "lower", "upper"):
            assert _eq(getattr(cl, k).cpu().numpy(), GM[f"{tag}_L{lvl + 1}_{k}"]), (lvl, k)
    assert it == int(GM[f"{tag}_it"])
    assert _eq(x.cpu().numpy(), GM[f"{tag}_x"])
    assert abs(res - float(GM[f"{tag}_res"])) <= 1e-13 * float(GM[f"{tag}_res"])


def test_gamg_reduces_the_residual_and_reuses_its_hierarchy():
    d = hex_poisson(16, seed=2)
    m = LduMatrix(d["n"], torch.as_tensor(d["owner"]), torch.as_tensor(d["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(d[k]) for k in ("diag", "lower", "upper"))
    b = torch.as_tensor(d["b"])
    s = create_solver("GAMG", tolerance=0.0, rel_tol=0.0, max_iter=6)
    assert isinstance(s, GAMGSolver)
    x, it, res = s(m, b, torch.zeros_like(b))
    h = s.last_info.residual_history
    assert it == 6 and all(h[i + 1] < h[i] for i in range(len(h) - 1))
    levels = s.last_levels
    x2, _, res2 = s(m, b, torch.zeros_like(b))  # cached hierarchy: same result
    assert s.last_levels is levels or [l.n_cells for l in s.last_levels] == [l.n_cells
                                                                               for l in levels]
    assert torch.equal(x, x2) and res2 == res
