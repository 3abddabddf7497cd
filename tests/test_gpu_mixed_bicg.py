"""Mixed-precision PBiCGStab (FP32 inner iterations, FP64 reliable updates):
every result is stated against the FP64 oracle (the reference's PBiCGStab
restated on the CPU).

The inner recurrence runs in FP32 and its residual is re-anchored to the
true FP64 residual, so the bounds are on the true residual, on the distance
to a tightly converged FP64 solution and on the iteration count, with the
tolerances written in each test."""

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyopenfoam_gb300 import (LduMatrix, MixedPrecisionPBiCGSTABSolver, PBiCGSTABSolver,
                              create_solver)
from pyopenfoam_gb300.mesh.poisson import convection_diffusion
from tests.golden.cases import random_ldu

pytestmark = pytest.mark.gpu
f64 = torch.float64


def mat(d):
    m = LduMatrix(d["n"], torch.as_tensor(d["owner"]), torch.as_tensor(d["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(d[k]) for k in ("diag", "lower", "upper"))
    return m


def true_rel(d, x):
    r = d["b"] - O.amul(d["owner"], d["neighbour"], d["diag"], d["lower"], d["upper"], x)
    return np.linalg.norm(r) / np.linalg.norm(d["b"])


def oracle_solve(d, rel, omega="standard", max_iter=20000):
    pd = O.dilu_build(d["owner"], d["neighbour"], d["diag"], d["lower"], d["upper"])
    return O.pbicgstab(d["owner"], d["neighbour"], d["diag"], d["lower"], d["upper"], d["b"],
                       np.zeros(d["n"]), pd, 0.0, rel, max_iter, threads=8, omega=omega)


FORMS = ("persistent", "kernels", "gather", "fused")


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("N,rel", [(32, 1e-10), (48, 1e-8), (40, 1e-12)])
def test_mixed_bicgstab_reaches_fp64_accuracy(N, rel, form):
    d = convection_diffusion(N, seed=1)
    m = mat(d)
    s = MixedPrecisionPBiCGSTABSolver(tolerance=0.0, rel_tol=rel, max_iter=5000, form=form)
    x, it, res = s(m, torch.as_tensor(d["b"]), torch.zeros(d["n"], dtype=f64))
    assert s.last_info.converged
    xh = x.cpu().numpy()
    tr = true_rel(d, xh)
    # declared only on true FP64 residuals: the oracle's residual agrees
    assert tr < rel, tr
    assert abs(res / np.linalg.norm(d["b"]) - tr) <= 1e-3 * tr
    # against the FP64 oracle converged 100x tighter
    o = oracle_solve(d, rel * 1e-2)
    assert o.converged
    err = np.linalg.norm(xh - o.x) / np.linalg.norm(o.x)
    # measured on GB300: 2.7 rel (32^3, 1e-10), 1.25 rel (48^3, 1e-8), 0.29 rel (40^3, 1e-12)
    assert err < 10 * rel, err
    # the kept Krylov space: inner iterations stay close to FP64 BiCGStab's
    # (the oracle's count has two checks per iteration plus the first)
    o2 = oracle_solve(d, rel)
    fp64_iters = (o2.iterations - 1) / 2
    assert it - 1 <= 1.3 * fp64_iters + 10, (it, o2.iterations)
    assert s.last_result.outer_updates >= 1
    # the residual history holds |r0| and the true residual of every update
    h = s.last_info.residual_history
    assert len(h) == s.last_result.outer_updates + 1
    assert h[0] == pytest.approx(np.linalg.norm(d["b"]), rel=1e-12)


@pytest.mark.parametrize("pre", ["DILU", "DIC", "none"])
def test_mixed_bicgstab_matches_fp64_gpu_solver(pre):
    """Same system through the FP64 GPU PBiCGStab and the mixed solver: both
    converge to 1e-10 and the solutions agree to the conditioning bound."""
    d = convection_diffusion(24, seed=3, peclet=4.0)
    m = mat(d)
    b = torch.as_tensor(d["b"])
    x64, it64, _ = PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-11, max_iter=4000,
                                   preconditioner=pre, omega="standard")(
        m, b, torch.zeros(d["n"], dtype=f64))
    s = MixedPrecisionPBiCGSTABSolver(tolerance=0.0, rel_tol=1e-10, max_iter=4000,
                                      preconditioner=pre)
    x, it, _ = s(m, b, torch.zeros(d["n"], dtype=f64))
    assert s.last_info.converged
    assert true_rel(d, x.cpu().numpy()) < 1e-10
    err = torch.linalg.vector_norm(x - x64) / torch.linalg.vector_norm(x64)
    assert err < 1e-8, float(err)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("permute", [False, True])
def test_mixed_bicgstab_reference_omega_and_generic_layout(permute, form):
    """The reference's omega = (t.z)/(t.t) on a diagonally dominant system,
    on the hex layout and on shuffled, non-triangular addressing (generic
    gather)."""
    d = random_ldu(20, seed=9, permute_faces=permute)
    d["b"] = d["r"]
    m = mat(d)
    s = MixedPrecisionPBiCGSTABSolver(tolerance=0.0, rel_tol=1e-10, max_iter=500,
                                      omega="reference", form=form)
    x, it, _ = s(m, torch.as_tensor(d["b"]), torch.zeros(d["n"], dtype=f64))
    assert s.last_info.converged
    xh = x.cpu().numpy()
    assert true_rel(d, xh) < 1e-10
    o = oracle_solve(d, 1e-13, omega="reference", max_iter=2000)
    assert np.linalg.norm(xh - o.x) / np.linalg.norm(o.x) < 1e-9


@pytest.mark.parametrize("form", FORMS)
def test_mixed_bicgstab_edge_cases(form):
    from functools import partial

    MixedPrecisionPBiCGSTABSolver_ = partial(MixedPrecisionPBiCGSTABSolver, form=form)
    d = convection_diffusion(12, seed=5)
    m = mat(d)
    n = d["n"]
    b = torch.as_tensor(d["b"])
    # zero right-hand side: converged at the first check, x stays zero
    s = MixedPrecisionPBiCGSTABSolver_(tolerance=1e-12, rel_tol=0.0, max_iter=100)
    x, it, res = s(m, torch.zeros(n, dtype=f64), torch.zeros(n, dtype=f64))
    assert s.last_info.converged and it == 1 and res == 0.0
    assert torch.count_nonzero(x) == 0
    # max_iter = 0: x0 unchanged, not converged
    x0 = torch.as_tensor(np.random.default_rng(0).uniform(-1, 1, n))
    s = MixedPrecisionPBiCGSTABSolver_(tolerance=0.0, rel_tol=1e-10, max_iter=0)
    x, it, res = s(m, b, x0)
    assert not s.last_info.converged
    assert torch.equal(x.cpu(), x0)
    # iteration limit: the FP32 correction is folded into x and the last
    # reported residual is the true residual of that x
    s = MixedPrecisionPBiCGSTABSolver_(tolerance=0.0, rel_tol=1e-14, max_iter=7)
    x, it, res = s(m, b, torch.zeros(n, dtype=f64))
    assert not s.last_info.converged
    # the limit, plus the folding iteration unless a fold was already due
    assert s.last_result.inner_iterations in (7, 8)
    assert res / np.linalg.norm(d["b"]) == pytest.approx(true_rel(d, x.cpu().numpy()),
                                                         rel=1e-6)
    # an initial guess that already meets the absolute tolerance is returned
    o = oracle_solve(d, 1e-13)
    s = MixedPrecisionPBiCGSTABSolver_(tolerance=1e-8, rel_tol=0.0, max_iter=500)
    x, it, _ = s(m, b, torch.as_tensor(o.x))
    assert it == 1 and torch.equal(x.cpu(), torch.as_tensor(o.x))
    # breakdown on a zero matrix (r~.v = 0), as the reference reports it
    z = dict(d, diag=np.zeros(n), lower=np.zeros_like(d["lower"]),
             upper=np.zeros_like(d["upper"]))
    s = MixedPrecisionPBiCGSTABSolver_(tolerance=0.0, rel_tol=1e-8, max_iter=50,
                                      preconditioner="none")
    x, it, _ = s(mat(z), b, torch.zeros(n, dtype=f64))
    assert not s.last_info.converged
    assert torch.isfinite(x).all()


def test_mixed_bicgstab_by_name():
    s = create_solver("MixedPBiCGStab", tolerance=0.0, rel_tol=1e-9, max_iter=2000)
    assert isinstance(s, MixedPrecisionPBiCGSTABSolver)
    d = convection_diffusion(16, seed=2)
    x, it, _ = s(mat(d), torch.as_tensor(d["b"]), torch.zeros(d["n"], dtype=f64))
    assert s.last_info.converged and true_rel(d, x.cpu().numpy()) < 1e-9


def test_mixed_bicgstab_forms_agree():
    """The persistent form and the per-iteration kernels run the same
    iteration; their dot products sum over different grids, so x agrees to
    rounding amplified by the Krylov recurrence -- and both reach the same
    true residual bound.  An unknown form is refused."""
    d = convection_diffusion(40, seed=4)
    m = mat(d)
    b = torch.as_tensor(d["b"])
    xs = {}
    for form in FORMS:
        s = MixedPrecisionPBiCGSTABSolver(tolerance=0.0, rel_tol=1e-10, max_iter=3000, form=form)
        x, it, _ = s(m, b, torch.zeros(d["n"], dtype=f64))
        assert s.last_info.converged and true_rel(d, x.cpu().numpy()) < 1e-10
        xs[form] = x
    ref = xs["kernels"]
    for form in ("persistent", "gather", "fused"):
        assert float(torch.linalg.vector_norm(xs[form] - ref) / torch.linalg.vector_norm(ref)) < 1e-8
    with pytest.raises(ValueError, match="form"):
        MixedPrecisionPBiCGSTABSolver(form="fastest")
