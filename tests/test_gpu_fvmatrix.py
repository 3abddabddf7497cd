"""FvMatrix on the GPU (core/fv_matrix.py:66-317): relax, set_reference,
residual, add_explicit_source and solve, against the reference formulas
evaluated in numpy with the same order of operations (bitwise), and the
relaxation-factor range error."""

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyopenfoam_gb300 import FvMatrix, PCGSolver
from tests.golden.cases import random_ldu

pytestmark = pytest.mark.gpu


def _fv(c):
    m = FvMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                 device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(c[k]) for k in ("diag", "lower", "upper"))
    m.source = torch.as_tensor(c["r"])
    return m


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.int64)


def test_relax_set_reference_residual_bitwise():
    c = random_ldu(6, seed=61)
    m = _fv(c)
    old = np.random.default_rng(2).uniform(-1, 1, c["n"])
    a = 0.7
    m.relax(torch.as_tensor(old), a)
    d = c["diag"] / a
    s = c["r"] + (1.0 - a) * d * old
    assert (_bits(m.diag.cpu().numpy()) == _bits(d)).all()
    assert (_bits(m.source.cpu().numpy()) == _bits(s)).all()
    assert m.relaxation_factor == a
    m.set_reference(5, value=2.5)
    large = max(abs(d[5]), 1.0) * 1e10
    d[5] += large
    s[5] += large * 2.5
    assert (_bits(m.diag.cpu().numpy()) == _bits(d)).all()
    assert (_bits(m.source.cpu().numpy()) == _bits(s)).all()
    x = np.random.default_rng(3).uniform(-1, 1, c["n"])
    r = m.residual(torch.as_tensor(x)).cpu().numpy()
    ref = s - O.amul(c["owner"], c["neighbour"], d, c["lower"], c["upper"], x)
    assert (_bits(r) == _bits(ref)).all()
    m.add_explicit_source(torch.full((c["n"],), 0.25, dtype=torch.float64))
    assert (_bits(m.source.cpu().numpy()) == _bits(s + 0.25)).all()
    with pytest.raises(ValueError):
        m.relax(torch.as_tensor(old), 1.5)
    with pytest.raises(ValueError):
        m.set_reference(c["n"])


def test_fvmatrix_solve_uses_gpu_solver():
    c = random_ldu(6, seed=62)
    c["upper"] = c["lower"]  # symmetric, for PCG
    m = _fv(c)
    # FvMatrix.solve passes its own tolerance (default 1e-6, absolute) to the
    # solver, as the reference does (core/fv_matrix.py:265-290)
    x, it, res = m.solve(PCGSolver(rel_tol=1e-10, max_iter=500, preconditioner="none"),
                         torch.zeros(c["n"], dtype=torch.float64), tolerance=0.0)
    assert x.device.type == "cuda" and it > 1
    r = c["r"] - O.amul(c["owner"], c["neighbour"], c["diag"], c["lower"], c["upper"],
                        x.cpu().numpy())
    assert np.linalg.norm(r) / np.linalg.norm(c["r"]) < 1e-9
