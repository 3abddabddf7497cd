"""The reference's own hot-path unit tests, restated against this package on
CUDA tensors.

One test here per reference test of the drop-in surface -- LduMatrix
(tests/unit/core/test_ldu_matrix.py), PCGSolver (tests/unit/solvers/
test_pcg.py), PBiCGSTABSolver (tests/unit/solvers/test_pbicgstab.py), the DIC
and DILU preconditioners (tests/unit/solvers/test_preconditioners.py:17-137),
DifferentiableLinearSolve (tests/unit/differentiable/test_linear_solver.py)
and DifferentiableLaplacian (tests/unit/differentiable/test_operators.py:
171-257) -- with the same inputs and the same assertions, each test naming
the reference test it restates.  Where the reference asserts on the CPU
device, the restated test asserts the CUDA device instead (a CPU device is
refused here: there is no CPU fallback).
"""

from __future__ import annotations

import pytest
import torch

from pyopenfoam_gb300 import (DICPreconditioner, DILUPreconditioner, LduMatrix,
                              PBiCGSTABSolver, PCGSolver, create_solver)
from pyopenfoam_gb300.differentiable import DifferentiableLaplacian, DifferentiableLinearSolve
from pyopenfoam_gb300.mesh import FvMesh

pytestmark = pytest.mark.gpu

f64 = torch.float64
i64 = torch.int64
DEV = torch.device("cuda", 0)


def T(v, dtype=f64):
    return torch.tensor(v, dtype=dtype)


def two_cell():
    return 2, T([0], i64), T([1], i64)


def chain3():
    return 3, T([0, 1], i64), T([1, 2], i64)


def no_faces(n):
    return LduMatrix(n, T([], i64), T([], i64))


def symmetric(n, owner, neighbour, coeff=1.0):
    """The reference's make_symmetric_matrix (tests/unit/solvers/conftest.py:
    10-33): lower = upper = -coeff, diag = sum of |off-diagonals| + 0.1."""
    m = LduMatrix(n, owner, neighbour)
    nf = int(neighbour.shape[0])
    m.lower = torch.full((nf,), -coeff, dtype=f64)
    m.upper = torch.full((nf,), -coeff, dtype=f64)
    d = torch.zeros(n, dtype=f64)
    d.index_add_(0, owner, torch.full((nf,), coeff, dtype=f64))
    d.index_add_(0, neighbour, torch.full((nf,), coeff, dtype=f64))
    m.diag = d + 0.1
    return m


def asymmetric(n, owner, neighbour):
    """make_asymmetric_matrix (conftest.py:36-60): lower = -1, upper = -1.5,
    diag_P += 1 per owned face, diag_N += 1.5 per neighbour face, + 0.5."""
    m = LduMatrix(n, owner, neighbour)
    nf = int(neighbour.shape[0])
    m.lower = torch.full((nf,), -1.0, dtype=f64)
    m.upper = torch.full((nf,), -1.5, dtype=f64)
    d = torch.zeros(n, dtype=f64)
    d.index_add_(0, owner, torch.full((nf,), 1.0, dtype=f64))
    d.index_add_(0, neighbour, torch.full((nf,), 1.5, dtype=f64))
    m.diag = d + 0.5
    return m


def chain10():
    return 10, torch.arange(9), torch.arange(1, 10)


# ---------------------------------------------------------------------------
# LduMatrix: tests/unit/core/test_ldu_matrix.py
# ---------------------------------------------------------------------------
def test_ldu_construction():
    """test_basic_creation, test_{diag,lower,upper}_zeros_initially,
    test_default_dtype_is_float64, test_owner_neighbour_stored (:59-92) and
    test_device_cpu (:94-98, here: the CUDA device)."""
    n, own, nei = two_cell()
    m = LduMatrix(n, own, nei)
    assert m.n_cells == 2 and m.n_internal_faces == 1
    assert torch.equal(m.diag.cpu(), torch.zeros(2, dtype=f64))
    assert torch.equal(m.lower.cpu(), torch.zeros(1, dtype=f64))
    assert torch.equal(m.upper.cpu(), torch.zeros(1, dtype=f64))
    assert m.dtype == f64 and m.diag.dtype == m.lower.dtype == m.upper.dtype == f64
    assert torch.equal(m.owner.cpu(), own) and torch.equal(m.neighbour.cpu(), nei)
    assert m.device.type == "cuda" and m.diag.device.type == "cuda"
    with pytest.raises(ValueError):
        LduMatrix(n, own, nei, device="cpu")


def test_ldu_repr():
    """test_repr (:100-107)."""
    r = repr(LduMatrix(*two_cell()))
    assert "LduMatrix" in r and "n_cells=2" in r and "n_internal_faces=1" in r


def test_ldu_setters_and_add_to_diag():
    """test_set_diag / lower / upper, test_add_to_diag_scalar / vector
    (:115-144)."""
    m = LduMatrix(*two_cell())
    m.diag = T([4.0, 4.0])
    m.lower = T([-1.0])
    m.upper = T([-1.0])
    assert torch.equal(m.diag.cpu(), T([4.0, 4.0]))
    assert torch.equal(m.lower.cpu(), T([-1.0])) and torch.equal(m.upper.cpu(), T([-1.0]))
    m = LduMatrix(*two_cell())
    m.add_to_diag(torch.tensor(3.0))
    assert torch.equal(m.diag.cpu(), T([3.0, 3.0]))
    m = LduMatrix(*two_cell())
    m.add_to_diag(T([1.0, 2.0]))
    assert torch.equal(m.diag.cpu(), T([1.0, 2.0]))


@pytest.mark.parametrize("case", ["identity", "symmetric", "asymmetric", "chain", "zero"])
def test_ldu_ax(case):
    """test_identity_matrix, test_symmetric_off_diagonal,
    test_asymmetric_off_diagonal, test_3cell_chain, test_zero_matrix
    (:152-210): the same matrices and vectors, exact answers."""
    if case == "chain":
        m = LduMatrix(*chain3())
        m.diag, m.lower, m.upper = T([4.0, 6.0, 4.0]), T([-1.0, -1.0]), T([-1.0, -1.0])
        x, want = T([1.0, 2.0, 3.0]), T([2.0, 8.0, 10.0])
    else:
        m = LduMatrix(*two_cell())
        if case == "identity":
            m.diag = T([3.0, 5.0])
            x, want = T([2.0, 4.0]), T([6.0, 20.0])
        elif case == "symmetric":
            m.diag, m.lower, m.upper = T([2.0, 2.0]), T([-1.0]), T([-1.0])
            x, want = T([1.0, 1.0]), T([1.0, 1.0])
        elif case == "asymmetric":
            m.diag, m.lower, m.upper = T([4.0, 4.0]), T([-1.0]), T([-2.0])
            x, want = T([1.0, 3.0]), T([1.0, 10.0])
        else:
            x, want = T([5.0, 7.0]), T([0.0, 0.0])
    y = m.Ax(x.to(DEV))
    assert y.device.type == "cuda"
    assert torch.equal(y.cpu(), want)


def test_ldu_ax_errors():
    """test_wrong_size_raises (:212-218) and test_non_floating_raises
    (:220-226): ValueError naming the size, TypeError for integers."""
    m = LduMatrix(*two_cell())
    with pytest.raises(ValueError, match="3 elements"):
        m.Ax(T([1.0, 2.0, 3.0]).to(DEV))
    with pytest.raises(TypeError, match="floating-point"):
        m.Ax(torch.tensor([1, 2], dtype=i64).to(DEV))


def test_ldu_sparse_views():
    """test_to_sparse_coo_shape / values, test_to_sparse_csr,
    test_sparse_matvec_matches_ldu (:235-287) and
    test_to_sparse_coo_matches_original (:296-311)."""
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([4.0, 4.0]), T([-1.0]), T([-1.0])
    coo = m.to_sparse_coo()
    assert coo.shape == (2, 2)
    dense = coo.to_dense().cpu()
    assert dense[0, 0] == 4.0 and dense[1, 1] == 4.0
    assert dense[0, 1] == -1.0 and dense[1, 0] == -1.0
    m.diag, m.lower, m.upper = T([2.0, 3.0]), T([-1.0]), T([-2.0])
    assert m.to_sparse_csr().layout == torch.sparse_csr
    c = LduMatrix(*chain3())
    c.diag, c.lower, c.upper = T([4.0, 6.0, 4.0]), T([-1.0, -1.0]), T([-1.0, -1.0])
    x = T([1.0, 2.0, 3.0]).to(DEV)
    y_sparse = torch.sparse.mm(c.to_sparse_coo(), x.unsqueeze(1)).squeeze(1)
    assert torch.allclose(c.Ax(x), y_sparse, atol=1e-12)
    c.upper = T([-2.0, -2.0])
    d = c.to_sparse_coo().to_dense().cpu()
    # as in the reference's view: lower[f] at (owner, neighbour), upper[f] at
    # (neighbour, owner)
    assert d[0, 0] == 4.0 and d[1, 1] == 6.0 and d[0, 1] == -1.0 and d[1, 0] == -2.0


def test_ldu_csr_cache_and_invalidation():
    """test_to_sparse_csr_cached, test_cache_invalidation_on_{diag,lower,
    upper}_set, test_cache_invalidation_on_add_to_diag and
    test_invalidate_cache_explicit (:313-389)."""

    def fresh():
        m = LduMatrix(*two_cell())
        m.diag, m.lower, m.upper = T([2.0, 3.0]), T([-1.0]), T([-2.0])
        return m

    m = fresh()
    assert m.to_sparse_csr_cached() is m.to_sparse_csr_cached()
    for edit in (lambda m: setattr(m, "diag", T([5.0, 6.0])),
                 lambda m: setattr(m, "lower", T([-3.0])),
                 lambda m: setattr(m, "upper", T([-4.0])),
                 lambda m: m.add_to_diag(T([1.0, 1.0]))):
        m = fresh()
        c1 = m.to_sparse_csr_cached()
        edit(m)
        assert m.to_sparse_csr_cached() is not c1
    m = fresh()
    m.to_sparse_csr_cached()
    m.invalidate_cache()
    assert "csr" not in m._csr_cache


def test_ldu_ax_sparse_and_batched():
    """test_ax_sparse_matches_ax, test_ax_sparse_asymmetric, test_ax_batched,
    test_ax_sparse_zero_off_diagonal (:391-458): Ax_sparse / Ax_batched
    against Ax and against the CSR product at 1e-12."""
    c = LduMatrix(*chain3())
    c.diag, c.lower, c.upper = T([4.0, 6.0, 4.0]), T([-1.0, -1.0]), T([-1.0, -1.0])
    x = T([1.0, 2.0, 3.0]).to(DEV)
    assert torch.allclose(c.Ax(x), c.Ax_sparse(x), atol=1e-12)
    csr = c.to_sparse_csr_cached()
    assert torch.allclose(c.Ax_sparse(x), (csr @ x.unsqueeze(1)).squeeze(1), atol=1e-12)
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([4.0, 4.0]), T([-1.0]), T([-2.0])
    x2 = T([1.0, 3.0]).to(DEV)
    assert torch.allclose(m.Ax(x2), m.Ax_sparse(x2), atol=1e-12)
    X = T([[1.0, 10.0], [2.0, 20.0], [3.0, 30.0]]).to(DEV)
    Y = c.Ax_batched(X)
    assert torch.allclose(Y[:, 0], c.Ax(X[:, 0]), atol=1e-12)
    assert torch.allclose(Y[:, 1], c.Ax(X[:, 1]), atol=1e-12)
    z = LduMatrix(*two_cell())
    z.diag, z.lower, z.upper = T([3.0, 5.0]), T([0.0]), T([0.0])
    assert torch.equal(z.Ax_sparse(T([2.0, 4.0]).to(DEV)).cpu(), T([6.0, 20.0]))


def test_ldu_diffusion_matrix_3cell():
    """test_diffusion_matrix_3cell (:462-486)."""
    m = LduMatrix(*chain3())
    coeff = T([1.0, 1.0])
    m.lower, m.upper, m.diag = -coeff, -coeff, T([1.0, 2.0, 1.0])
    assert torch.allclose(m.Ax(torch.ones(3, dtype=f64, device=DEV)).cpu(),
                          torch.zeros(3, dtype=f64), atol=1e-12)
    assert torch.allclose(m.Ax(T([1.0, 2.0, 3.0]).to(DEV)).cpu(), T([-1.0, 0.0, 1.0]),
                          atol=1e-12)


# ---------------------------------------------------------------------------
# PCGSolver: tests/unit/solvers/test_pcg.py
# ---------------------------------------------------------------------------
def _solve(solver, m, b, x0=None):
    b = b.to(DEV)
    x0 = torch.zeros_like(b) if x0 is None else x0.to(DEV)
    x, it, res = solver(m, b, x0)
    assert x.device.type == "cuda"
    return x, it, res


def test_pcg_identity_and_scaled_identity():
    """test_identity_system (:15-29) and test_scaled_identity (:31-43)."""
    m = no_faces(3)
    m.diag = T([1.0, 1.0, 1.0])
    x, it, _ = _solve(PCGSolver(tolerance=1e-10, max_iter=100, preconditioner="none"), m,
                      T([2.0, 3.0, 4.0]))
    assert torch.allclose(x.cpu(), T([2.0, 3.0, 4.0]), atol=1e-8) and it <= 2
    m = no_faces(2)
    m.diag = T([2.0, 2.0])
    x, _, _ = _solve(PCGSolver(tolerance=1e-10, max_iter=100, preconditioner="none"), m,
                     T([4.0, 6.0]))
    assert torch.allclose(x.cpu(), T([2.0, 3.0]), atol=1e-8)


def test_pcg_symmetric_2cell():
    """test_symmetric_2cell (:45-64): x = [1, 2] in fewer than 20 checks."""
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([4.0, 4.0]), T([-1.0]), T([-1.0])
    x, it, _ = _solve(PCGSolver(tolerance=1e-10, max_iter=100, preconditioner="none"), m,
                      T([2.0, 7.0]))
    assert torch.allclose(x.cpu(), T([1.0, 2.0]), atol=1e-6) and it < 20


@pytest.mark.parametrize("pre", ["none", "DIC", "DILU"])
def test_pcg_3cell_chain(pre):
    """test_symmetric_3cell_chain, test_with_dic_preconditioner,
    test_with_dilu_preconditioner (:66-116): |b - A x| < 1e-6."""
    m = symmetric(*chain3())
    b = T([1.0, 2.0, 1.0])
    x, _, _ = _solve(PCGSolver(tolerance=1e-10, max_iter=1000, preconditioner=pre), m, b)
    assert torch.linalg.vector_norm(b.to(DEV) - m.Ax(x)) < 1e-6


def test_pcg_convergence_info():
    """test_convergence_info (:121-133)."""
    m = symmetric(*chain3())
    x, it, res = _solve(PCGSolver(tolerance=1e-6, max_iter=100), m, T([1.0, 2.0, 1.0]))
    assert isinstance(it, int) and isinstance(res, float) and it > 0 and res < 1e-6


def test_pcg_max_iterations_stops():
    """test_max_iterations_stops (:135-150): an ill-conditioned system with
    max_iter = 5 stops within 5 checks... and returns the current x."""
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([1.0, 1e8]), T([-1.0]), T([-1.0])
    s = PCGSolver(tolerance=1e-15, max_iter=5, preconditioner="none")
    x, it, _ = _solve(s, m, T([1.0, 1.0]))
    assert it <= 5 and torch.isfinite(x).all()


def test_pcg_10cell_convergence():
    """test_10cell_convergence (:152-166)."""
    m = symmetric(*chain10())
    b = torch.ones(10, dtype=f64)
    x, _, _ = _solve(PCGSolver(tolerance=1e-8, max_iter=500, preconditioner="DIC"), m, b)
    assert torch.linalg.vector_norm(b.to(DEV) - m.Ax(x)) < 1e-4


def test_pcg_zero_rhs():
    """test_zero_rhs (:168-182): a zero right-hand side gives x = 0."""
    m = LduMatrix(*chain3())
    m.diag, m.lower, m.upper = T([4.0, 6.0, 4.0]), T([-1.0, -1.0]), T([-1.0, -1.0])
    x, _, _ = _solve(PCGSolver(tolerance=1e-10, max_iter=100), m, torch.zeros(3, dtype=f64))
    assert torch.allclose(x.cpu(), torch.zeros(3, dtype=f64), atol=1e-10)


def test_solver_factory_and_repr():
    """test_create_pcg, test_create_pcg_case_insensitive,
    test_unknown_solver_raises, test_repr (test_pcg.py:188-209) and
    test_create_pbicgstab, test_create_case_insensitive, test_repr
    (test_pbicgstab.py:162-170, 185-189)."""
    s = create_solver("PCG", tolerance=1e-8)
    assert isinstance(s, PCGSolver) and s.tolerance == 1e-8
    assert isinstance(create_solver("pcg"), PCGSolver)
    with pytest.raises(ValueError, match="Unknown solver"):
        create_solver("FOOBAR")
    r = repr(PCGSolver(tolerance=1e-8, max_iter=500))
    assert "PCGSolver" in r and "1e-08" in r
    assert isinstance(create_solver("PBiCGSTAB", tolerance=1e-8), PBiCGSTABSolver)
    assert isinstance(create_solver("pbicgstab"), PBiCGSTABSolver)
    assert "PBiCGSTABSolver" in repr(PBiCGSTABSolver(tolerance=1e-8, max_iter=500))


# ---------------------------------------------------------------------------
# PBiCGSTABSolver: tests/unit/solvers/test_pbicgstab.py
# ---------------------------------------------------------------------------
def test_pbicgstab_small_systems():
    """test_identity_system (:15-27), test_symmetric_2cell (:29-45),
    test_asymmetric_2cell (:47-65)."""
    m = no_faces(3)
    m.diag = T([1.0, 1.0, 1.0])
    s = PBiCGSTABSolver(tolerance=1e-10, max_iter=100, preconditioner="none")
    x, _, _ = _solve(s, m, T([2.0, 3.0, 4.0]))
    assert torch.allclose(x.cpu(), T([2.0, 3.0, 4.0]), atol=1e-8)
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([4.0, 4.0]), T([-1.0]), T([-1.0])
    x, _, _ = _solve(s, m, T([2.0, 7.0]))
    assert torch.allclose(x.cpu(), T([1.0, 2.0]), atol=1e-6)
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([4.0, 5.0]), T([-1.0]), T([-2.0])
    x, _, _ = _solve(s, m, T([3.0, 3.0]))
    assert torch.allclose(x.cpu(), T([1.0, 1.0]), atol=1e-4)


@pytest.mark.parametrize("pre,bar", [("none", 1e-4), ("DILU", 0.1), ("DIC", 1e-4)])
def test_pbicgstab_asymmetric_3cell(pre, bar):
    """test_asymmetric_3cell (:67-79), test_with_dilu_preconditioner
    (:81-94), test_with_dic_preconditioner (:96-109), each with its bar."""
    m = asymmetric(*chain3())
    b = T([1.0, 2.0, 1.0])
    x, _, _ = _solve(PBiCGSTABSolver(tolerance=1e-8, max_iter=500, preconditioner=pre), m, b)
    assert torch.linalg.vector_norm(b.to(DEV) - m.Ax(x)) < bar


def test_pbicgstab_convergence_info_and_factory_solve():
    """test_convergence_info (:114-125) and test_solve_via_factory
    (:172-183)."""
    m = asymmetric(*chain3())
    b = T([1.0, 2.0, 1.0])
    x, it, res = _solve(PBiCGSTABSolver(tolerance=1e-6, max_iter=200), m, b)
    assert isinstance(it, int) and isinstance(res, float) and it > 0
    x, _, _ = _solve(create_solver("PBiCGSTAB", tolerance=1e-6, max_iter=200), m, b)
    assert torch.linalg.vector_norm(b.to(DEV) - m.Ax(x)) < 0.1


def test_pbicgstab_10cell_and_zero_rhs():
    """test_10cell_convergence (:127-140) and test_zero_rhs (:142-157)."""
    m = asymmetric(*chain10())
    b = torch.ones(10, dtype=f64)
    x, _, _ = _solve(PBiCGSTABSolver(tolerance=1e-8, max_iter=500, preconditioner="DILU"), m, b)
    assert torch.linalg.vector_norm(b.to(DEV) - m.Ax(x)) < 0.1
    z = LduMatrix(*chain3())
    z.diag, z.lower, z.upper = T([4.0, 6.0, 4.0]), T([-1.0, -1.0]), T([-2.0, -2.0])
    x, _, _ = _solve(PBiCGSTABSolver(tolerance=1e-10, max_iter=100), z, torch.zeros(3, dtype=f64))
    assert torch.allclose(x.cpu(), torch.zeros(3, dtype=f64), atol=1e-10)


# ---------------------------------------------------------------------------
# DIC / DILU: tests/unit/solvers/test_preconditioners.py:17-137
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("cls", [DICPreconditioner, DILUPreconditioner])
def test_preconditioner_diagonal_only(cls):
    """TestDICPreconditioner / TestDILUPreconditioner.test_diagonal_only_matrix
    (:20-30, :82-91): r / diag."""
    m = no_faces(3)
    m.diag = T([4.0, 2.0, 8.0])
    z = cls(m).apply(T([4.0, 2.0, 8.0]).to(DEV))
    assert torch.allclose(z.cpu(), T([1.0, 1.0, 1.0]), atol=1e-10)


def test_dic_symmetric_identity_and_device():
    """test_symmetric_matrix (:32-46), test_identity_preconditioner (:48-61),
    test_output_device_dtype (:63-77, here: CUDA)."""
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([2.0, 2.0]), T([-1.0]), T([-1.0])
    z = DICPreconditioner(m).apply(T([1.0, 1.0]).to(DEV))
    assert z.shape == (2,) and bool((z > 0).all())
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([100.0, 100.0]), T([-0.001]), T([-0.001])
    r = T([1.0, 1.0]).to(DEV)
    assert torch.allclose(DICPreconditioner(m).apply(r), r / 100.0, atol=1e-6)
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([4.0, 4.0]), T([-1.0]), T([-1.0])
    z = DICPreconditioner(m).apply(T([1.0, 1.0]).to(DEV))
    assert z.device == m.device and z.dtype == m.dtype


def test_dilu_asymmetric_matches_dic_and_shape():
    """test_asymmetric_matrix (:93-106), test_symmetric_matches_dic
    (:108-126), test_output_shape (:128-137)."""
    m = LduMatrix(*two_cell())
    m.diag, m.lower, m.upper = T([4.0, 4.0]), T([-1.0]), T([-2.0])
    z = DILUPreconditioner(m).apply(T([1.0, 1.0]).to(DEV))
    assert z.shape == (2,) and bool((z > 0).all())
    c = LduMatrix(*chain3())
    c.diag, c.lower, c.upper = T([4.0, 6.0, 4.0]), T([-1.0, -1.0]), T([-1.0, -1.0])
    r = T([1.0, 2.0, 3.0]).to(DEV)
    assert torch.allclose(DICPreconditioner(c).apply(r), DILUPreconditioner(c).apply(r), atol=0.1)
    m5 = no_faces(5)
    m5.diag = torch.ones(5, dtype=f64)
    assert DILUPreconditioner(m5).apply(torch.ones(5, dtype=f64, device=DEV)).shape == (5,)


# ---------------------------------------------------------------------------
# DifferentiableLinearSolve: tests/unit/differentiable/test_linear_solver.py
# ---------------------------------------------------------------------------
def _dls_system():
    """The simple_system fixture (:14-33): 3 cells, faces (0,1), (1,2), (0,2)."""
    diag = T([4.0, 5.0, 4.0]).to(DEV).requires_grad_(True)
    lower = T([-1.0, -1.0, -0.5]).to(DEV).requires_grad_(True)
    upper = T([-1.0, -1.0, -0.5]).to(DEV).requires_grad_(True)
    b = T([1.0, 2.0, 3.0]).to(DEV).requires_grad_(True)
    own, nei = T([0, 1, 0], i64).to(DEV), T([1, 2, 2], i64).to(DEV)
    return diag, lower, upper, b, own, nei, torch.zeros(3, dtype=f64, device=DEV)


def _dls(diag, lower, upper, b, own, nei, x0):
    return DifferentiableLinearSolve.apply(diag, lower, upper, b,
                                           PCGSolver(tolerance=1e-10, max_iter=1000), own, nei,
                                           x0, 1e-10, 1000)


def test_dls_forward():
    """test_forward_shape, test_forward_values, test_forward_satisfies_equation
    (:37-73)."""
    diag, lower, upper, b, own, nei, x0 = _dls_system()
    x = _dls(diag, lower, upper, b, own, nei, x0)
    assert x.shape == (3,) and torch.isfinite(x).all()
    m = LduMatrix(3, own, nei, dtype=f64)
    m.diag, m.lower, m.upper = diag.detach(), lower.detach(), upper.detach()
    assert torch.allclose(m.Ax(x.detach()), b.detach(), atol=1e-6)


def test_dls_backward():
    """test_backward_wrt_b, test_backward_wrt_diag,
    test_backward_wrt_offdiagonal (:75-120)."""
    diag, lower, upper, b, own, nei, x0 = _dls_system()
    _dls(diag, lower, upper, b, own, nei, x0).sum().backward()
    for g in (b.grad, diag.grad, lower.grad, upper.grad):
        assert g is not None and torch.isfinite(g).all()


def test_dls_gradient_consistency():
    """test_gradient_consistency (:122-156): d(sum x)/db against central
    differences (eps 1e-6) at the reference's bar, 1e-2: its solver keeps the
    default rel_tol = 0.01, so every solve stops at 1 % relative residual
    (test_gpu_differentiable.py holds 1e-7 with solves driven to 1e-14)."""
    diag, lower, upper, b, own, nei, x0 = _dls_system()
    _dls(diag, lower, upper, b, own, nei, x0).sum().backward()
    eps = 1e-6
    for i in range(3):
        bp, bm = b.detach().clone(), b.detach().clone()
        bp[i] += eps
        bm[i] -= eps
        fp = _dls(diag.detach(), lower.detach(), upper.detach(), bp, own, nei, x0).sum()
        fm = _dls(diag.detach(), lower.detach(), upper.detach(), bm, own, nei, x0).sum()
        assert abs(float((fp - fm) / (2 * eps)) - float(b.grad[i])) < 1e-2


def test_dls_optimisation_with_adam():
    """test_optimization_with_differentiable_solve (:165-194): 200 Adam
    steps (lr 0.05) on b drive x towards [1, 2, 3] within 0.3."""
    diag, lower, upper, b0, own, nei, x0 = _dls_system()
    target = T([1.0, 2.0, 3.0]).to(DEV)
    b = b0.detach().clone().requires_grad_(True)
    opt = torch.optim.Adam([b], lr=0.05)
    for _ in range(200):
        opt.zero_grad()
        x = _dls(diag.detach(), lower.detach(), upper.detach(), b, own, nei, x0)
        ((x - target) ** 2).sum().backward()
        opt.step()
    with torch.no_grad():
        x = _dls(diag.detach(), lower.detach(), upper.detach(), b, own, nei, x0)
    assert torch.allclose(x, target, atol=0.3)


# ---------------------------------------------------------------------------
# DifferentiableLaplacian: tests/unit/differentiable/test_operators.py:171-257
# ---------------------------------------------------------------------------
_PTS = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1],
        [0, 0, 2], [1, 0, 2], [1, 1, 2], [0, 1, 2]]
_FACES = [[4, 5, 6, 7], [0, 3, 2, 1], [0, 1, 5, 4], [3, 7, 6, 2], [0, 4, 7, 3], [1, 2, 6, 5],
          [8, 9, 10, 11], [4, 5, 9, 8], [7, 11, 10, 6], [4, 8, 11, 7], [5, 6, 10, 9]]
_OWNER = [0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1]


def _two_cell_mesh():
    """The mesh fixture of test_operators.py (:26-72): two stacked unit cubes."""
    return FvMesh(torch.tensor(_PTS, dtype=f64), [torch.tensor(f, dtype=i64) for f in _FACES],
                  torch.tensor(_OWNER, dtype=i64), torch.tensor([1], dtype=i64),
                  [{"name": "bottom", "type": "wall", "startFace": 1, "nFaces": 5},
                   {"name": "top", "type": "wall", "startFace": 6, "nFaces": 5}], device=DEV)


def test_dlaplacian_forward_backward():
    """test_forward_shape, test_forward_values, test_backward_shape,
    test_backward_values, test_constant_field_laplacian_zero,
    test_diffusion_coefficient_scaling (:172-212)."""
    mesh = _two_cell_mesh()
    phi = T([1.0, 2.0]).to(DEV).requires_grad_(True)
    lap = DifferentiableLaplacian.apply(phi, 1.0, mesh)
    assert lap.shape == (2,) and torch.isfinite(lap).all()
    lap.sum().backward()
    assert phi.grad is not None and phi.grad.shape == (2,) and torch.isfinite(phi.grad).all()
    const = DifferentiableLaplacian.apply(T([5.0, 5.0]).to(DEV), 1.0, mesh)
    assert torch.allclose(const, torch.zeros(2, dtype=f64, device=DEV), atol=1e-10)
    p = T([1.0, 2.0]).to(DEV)
    assert torch.allclose(DifferentiableLaplacian.apply(p, 2.0, mesh),
                          2.0 * DifferentiableLaplacian.apply(p, 1.0, mesh), atol=1e-10)


def test_dlaplacian_gradcheck():
    """test_gradcheck (:214-222) and test_gradcheck_with_tensor_D (:224-237):
    torch.autograd.gradcheck with eps 1e-6, atol 1e-4."""
    mesh = _two_cell_mesh()
    phi = T([1.0, 2.0]).to(DEV).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda p: DifferentiableLaplacian.apply(p, 1.0, mesh), (phi,),
                                    eps=1e-6, atol=1e-4)
    D = torch.tensor(1.5, dtype=f64, device=DEV, requires_grad=True)
    assert torch.autograd.gradcheck(lambda p, d: DifferentiableLaplacian.apply(p, d, mesh),
                                    (phi, D), eps=1e-6, atol=1e-4)


def test_dlaplacian_gradient_flow():
    """test_gradient_flow_through_laplacian (:241-257)."""
    mesh = _two_cell_mesh()
    phi = T([1.0, 2.0]).to(DEV).requires_grad_(True)
    lap = DifferentiableLaplacian.apply(phi, 1.0, mesh)
    ((lap - T([0.5, 0.5]).to(DEV)) ** 2).sum().backward()
    assert phi.grad is not None and not torch.allclose(phi.grad, torch.zeros_like(phi.grad))
