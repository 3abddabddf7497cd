"""PBiCGSolver and DiagonalSolver on the GPU against the reference's own
solvers (tests/golden/reference_pbicg.npz, make_golden.py --pbicg).

The reference PBiCG's recurrence is reproduced step for step; only its dot
products are summed in another order, so x agrees to 1e-12 relative over the
first iterations (the reference recurrence itself diverges on this system,
which is why the comparison stops at six iterations).  DiagonalSolver is
bitwise."""

import os

import numpy as np
import pytest
import torch

from pyopenfoam_gb300 import LduMatrix, create_solver
from pyopenfoam_gb300.solvers import DiagonalSolver, PBiCGSolver
from tests.golden.cases import random_ldu

pytestmark = pytest.mark.gpu
PB = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_pbicg.npz"))


def _m(diag=None):
    c = random_ldu(5, seed=51, permute_faces=False)
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag = torch.as_tensor(c["diag"] if diag is None else diag)
    m.lower, m.upper = torch.as_tensor(c["lower"]), torch.as_tensor(c["upper"])
    return m, torch.as_tensor(c["r"])


@pytest.mark.parametrize("pc", ["DILU", "DIC", "none"])
@pytest.mark.parametrize("k", [1, 3, 6])
def test_pbicg_matches_reference(pc, k):
    m, b = _m()
    s = PBiCGSolver(tolerance=0.0, rel_tol=0.0, max_iter=k, preconditioner=pc)
    x, it, res = s(m, b, torch.zeros_like(b))
    ref = PB[f"pbicg_{pc}_{k}_x"]
    assert it == int(PB[f"pbicg_{pc}_{k}_it"])
    assert np.abs(x.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
    assert abs(res - float(PB[f"pbicg_{pc}_{k}_res"])) <= 1e-11 * float(PB[f"pbicg_{pc}_{k}_res"])


def test_diagonal_solver_bitwise():
    m, b = _m(PB["diag_d"])
    s = create_solver("diagonal")
    assert isinstance(s, DiagonalSolver)
    x, it, res = s(m, b, torch.zeros_like(b))
    assert (x.cpu().numpy().view(np.int64) == PB["diag_x"].view(np.int64)).all()
    assert it == int(PB["diag_it"]) and abs(res - float(PB["diag_res"])) <= 1e-14 * abs(
        float(PB["diag_res"]))
    with pytest.raises(ValueError):
        PBiCGSolver(preconditioner="ILU")(m, b, torch.zeros_like(b))
