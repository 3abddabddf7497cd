"""128^3 hex topology (2,097,152 cells, 6,242,304 faces)
against the reference's own outputs (tests/golden/reference_ldu128.npz,
made by running the reference on the same seeded system): Amul, Ax_T and
FP32 Amul bitwise, the DIC and DILU factorised diagonals bitwise, and
PBiCGStab+DILU against the reference's residual checks, check count and
solution."""

import numpy as np
import pytest
import torch

from pyopenfoam_gb300 import (DICPreconditioner, DILUPreconditioner, LduMatrix,
                              PBiCGSTABSolver)
from tests.golden.cases import LDU128_FIXTURE, random_ldu, sha
from tests.test_oracle_pins import check_ldu128_bicgstab

pytestmark = pytest.mark.gpu
R = np.load(LDU128_FIXTURE)


@pytest.fixture(scope="module")
def case():
    c = random_ldu(128, seed=5)
    # the seeded inputs are the ones the reference ran on
    assert sha(np.concatenate([c["diag"], c["lower"], c["upper"], c["x"], c["r"]])) == str(
        R["coeff_sha"])
    return c


def mat(c, dtype=torch.float64):
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda", dtype=dtype)
    m.diag, m.lower, m.upper = (torch.as_tensor(c[k]) for k in ("diag", "lower", "upper"))
    return m


def test_amul_and_factorisations_bitwise(case):
    m = mat(case)
    x = torch.as_tensor(case["x"])
    assert sha(m.Ax(x).cpu().numpy()) == str(R["Ax_sha"])
    assert sha(m.Ax_T(x).cpu().numpy()) == str(R["AxT_sha"])
    m32 = mat(case, torch.float32)
    assert sha(m32.Ax(x.float()).cpu().numpy()) == str(R["Ax_f32_sha"])
    assert sha(DICPreconditioner(m).precond_diag.cpu().numpy()) == str(R["dic_sha"])
    assert sha(DILUPreconditioner(m).precond_diag.cpu().numpy()) == str(R["dilu_sha"])


def test_pbicgstab_dilu_against_reference(case):
    m = mat(case)
    s = PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-10, max_iter=200, preconditioner="DILU")
    x, it, res = s(m, torch.as_tensor(case["r"]), torch.zeros(case["n"], dtype=torch.float64))
    # the bar and why it is not bitwise: check_ldu128_bicgstab's docstring
    check_ldu128_bicgstab(s.last_info.converged, it, s.last_info.residual_history,
                          x.cpu().numpy(), R)
