"""Mixed-precision refined PCG: every result is stated against the FP64
oracle (the reference algorithm restated on the CPU).

The mixed solver's inner iterations run in FP32 and its residual is
re-anchored to the true FP64 residual, so the test bounds are on the true
residual and on the distance to a tightly converged FP64 solution, with the
tolerances written in each test."""

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyopenfoam_gb300 import LduMatrix, MixedPrecisionPCGSolver, PCGSolver, create_solver
from pyopenfoam_gb300.mesh.poisson import hex_poisson
from tests.golden.cases import FIXTURE, jitter_case

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


@pytest.mark.parametrize("N,rel", [(32, 1e-10), (48, 1e-8)])
def test_mixed_reaches_fp64_accuracy(N, rel):
    d = hex_poisson(N, seed=2)
    m = mat(d)
    s = MixedPrecisionPCGSolver(tolerance=0.0, rel_tol=rel, max_iter=5000)
    x, it, res = s(m, torch.as_tensor(d["b"]), torch.zeros(d["n"], dtype=f64))
    assert s.last_info.converged
    xh = x.cpu().numpy()
    tr = true_rel(d, xh)
    # declared only on true FP64 residuals: the oracle's residual agrees
    assert tr < rel, tr
    assert abs(res / np.linalg.norm(d["b"]) - tr) <= 1e-3 * tr
    # against the FP64 oracle converged 100x tighter
    pd = O.dic_build(d["owner"], d["neighbour"], d["diag"], d["upper"])
    o = O.pcg(d["owner"], d["neighbour"], d["diag"], d["lower"], d["upper"], d["b"],
              np.zeros(d["n"]), pd, 0.0, rel * 1e-2, 20000, threads=8)
    err = np.linalg.norm(xh - o.x) / np.linalg.norm(o.x)
    # |dx|/|x| <= kappa |dr|/|b|; measured on GB300: 11.7 rel (32^3) and 9.8 rel (48^3)
    assert err < 30 * rel, err
    # the kept Krylov space: inner iterations stay close to FP64 PCG's
    o2 = O.pcg(d["owner"], d["neighbour"], d["diag"], d["lower"], d["upper"], d["b"],
               np.zeros(d["n"]), pd, 0.0, rel, 20000, threads=8)
    assert it <= 1.25 * o2.iterations + 10, (it, o2.iterations)
    assert s.last_result.outer_updates >= 1


def test_mixed_on_jittered_lognormal_laplacian():
    G = np.load(FIXTURE)
    jc = jitter_case(6)
    nint = int(jc["n_internal"])
    d = dict(n=int(jc["n_cells"]), owner=jc["owner"][:nint], neighbour=jc["neighbour"],
             diag=G["j6_lap_diag"], lower=G["j6_lap_lower"], upper=G["j6_lap_upper"], b=jc["b"])
    s = MixedPrecisionPCGSolver(tolerance=0.0, rel_tol=1e-10, max_iter=2000)
    x, it, res = s(mat(d), torch.as_tensor(d["b"]), torch.zeros(d["n"], dtype=f64))
    assert s.last_info.converged
    assert true_rel(d, x.cpu().numpy()) < 1e-10
    ref = G["j6_pcg_x"]  # reference PCG+DIC to 1e-10
    assert np.abs(x.cpu().numpy() - ref).max() / np.abs(ref).max() < 1e-6


def test_mixed_iteration_limit_folds_correction():
    d = hex_poisson(16, seed=1)
    m = mat(d)
    s = MixedPrecisionPCGSolver(tolerance=0.0, rel_tol=1e-12, max_iter=7)
    x, it, res = s(m, torch.as_tensor(d["b"]), torch.zeros(d["n"], dtype=f64))
    assert not s.last_info.converged
    assert it <= 7 + 2
    # x holds the folded correction: its true residual is what was reported
    tr = true_rel(d, x.cpu().numpy())
    assert abs(res / np.linalg.norm(d["b"]) - tr) <= 1e-6 * tr + 1e-12
    assert isinstance(create_solver("mixedpcg"), MixedPrecisionPCGSolver)


def test_mixed_zero_rhs_and_float32_rejected():
    d = hex_poisson(8, seed=1)
    m = mat(d)
    x, it, res = MixedPrecisionPCGSolver(tolerance=1e-10)(m, torch.zeros(d["n"], dtype=f64),
                                                          torch.zeros(d["n"], dtype=f64))
    assert it == 1 and res == 0.0 and torch.count_nonzero(x) == 0
    m32 = LduMatrix(2, torch.tensor([0]), torch.tensor([1]), device="cuda", dtype=torch.float32)
    with pytest.raises(TypeError):
        MixedPrecisionPCGSolver()(m32, torch.ones(2), torch.zeros(2))
    with pytest.raises(TypeError):
        PCGSolver()(m32, torch.ones(2), torch.zeros(2))


@pytest.mark.parametrize("N", [20, 48, 64])
def test_mixed_symmetric_half_storage_gives_identical_solve(N):
    """The inner Amul on the owner-side half of a symmetric matrix gives the
    bits of the full-packing Amul, so the whole mixed solve -- iterations,
    FP64 updates, x -- is bit for bit the same with and without it."""
    d = hex_poisson(N, seed=5)
    m = mat(d)
    assert m.topology().symmetric_storage and m.packed_sym32() is not None
    out = []
    for sym in (True, False):
        s = MixedPrecisionPCGSolver(tolerance=0.0, rel_tol=1e-10, max_iter=5000,
                                    symmetric_storage=sym)
        x, it, res = s(m, torch.as_tensor(d["b"]), torch.zeros(d["n"], dtype=f64))
        assert s.last_info.converged
        out.append((x.cpu().numpy(), it, res, s.last_result.outer_updates))
    (xa, ia, ra, ua), (xb, ib, rb, ub) = out
    assert (ia, ra, ua) == (ib, rb, ub)
    assert (xa.view(np.int64) == xb.view(np.int64)).all()
