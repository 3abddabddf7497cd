"""Preconditioner and Krylov-solver parity on the GPU.

* DIC / DILU factorised diagonals: bitwise against the reference goldens and
  the oracle (including unsorted, non-triangular addressing).
* PCG / PBiCGStab: the reference's own unit-test answers; iteration counts
  and solutions against the reference's golden runs and the oracle.  The
  reference's dot products round in a thread-dependent order, so solver
  trajectories are compared to a tolerance stated in each test.
"""

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyopenfoam_gb300 import (DICPreconditioner, DILUPreconditioner, LduMatrix,
                              PBiCGSTABSolver, PCGSolver, create_solver)
from tests.golden.cases import FIXTURE, c1_poisson, jitter_case, random_ldu, sha

pytestmark = pytest.mark.gpu
G = np.load(FIXTURE)
DEV = "cuda"
f64 = torch.float64


def mat(n, own, nei, diag, lower, upper):
    m = LduMatrix(n, torch.as_tensor(np.asarray(own)), torch.as_tensor(np.asarray(nei)),
                  device=DEV)
    m.diag = torch.as_tensor(np.asarray(diag, np.float64))
    m.lower = torch.as_tensor(np.asarray(lower, np.float64))
    m.upper = torch.as_tensor(np.asarray(upper, np.float64))
    return m


def relerr(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


# --------------------------------------------------------------------------
# preconditioners
# --------------------------------------------------------------------------
@pytest.mark.parametrize("name,N,perm", [("ldu32", 32, False), ("ldu12p", 12, True)])
def test_factorised_diagonals_bitwise(name, N, perm):
    c = random_ldu(N, 5, perm)
    m = mat(c["n"], c["owner"], c["neighbour"], c["diag"], c["lower"], c["upper"])
    assert sha(DICPreconditioner(m).precond_diag.cpu().numpy()) == str(G[f"{name}_dic_sha"])
    assert sha(DILUPreconditioner(m).precond_diag.cpu().numpy()) == str(G[f"{name}_dilu_sha"])


def test_factorisation_full_size_against_oracle():
    from tests.golden.cases import hex_faces

    n, own, nei = hex_faces(96)
    rng = np.random.default_rng(2)
    F = own.shape[0]
    lo, up, dg = rng.uniform(-1, 0, F), rng.uniform(-1, 0, F), rng.uniform(6, 7, n)
    m = mat(n, own, nei, dg, lo, up)
    np.testing.assert_array_equal(DICPreconditioner(m).precond_diag.cpu().numpy(),
                                  O.dic_build(own, nei, dg, up))
    np.testing.assert_array_equal(DILUPreconditioner(m).precond_diag.cpu().numpy(),
                                  O.dilu_build(own, nei, dg, lo, up))


def test_preconditioner_known_answers():
    # tests/unit/solvers/test_preconditioners.py:20-30, :82-91
    m = LduMatrix(3, torch.tensor([], dtype=torch.int64), torch.tensor([], dtype=torch.int64),
                  device=DEV)
    m.diag = torch.tensor([4.0, 2.0, 8.0], dtype=f64)
    r = torch.tensor([4.0, 2.0, 8.0], dtype=f64)
    for P in (DICPreconditioner, DILUPreconditioner):
        z = P(m).apply(r)
        assert z.device.type == "cuda" and z.dtype == f64
        np.testing.assert_allclose(z.cpu().numpy(), [1.0, 1.0, 1.0], atol=1e-10)
    # :50-65 dominant diagonal: z ~ r / diag
    m2 = mat(2, [0], [1], [100.0, 100.0], [-0.001], [-0.001])
    z = DICPreconditioner(m2).apply(torch.ones(2, dtype=f64))
    np.testing.assert_allclose(z.cpu().numpy(), [0.01, 0.01], atol=1e-6)


# --------------------------------------------------------------------------
# PCG -- reference unit tests (tests/unit/solvers/test_pcg.py)
# --------------------------------------------------------------------------
def test_pcg_reference_unit_cases():
    e = LduMatrix(3, torch.tensor([], dtype=torch.int64), torch.tensor([], dtype=torch.int64),
                  device=DEV)
    e.diag = torch.ones(3, dtype=f64)
    b = torch.tensor([2.0, 3.0, 4.0], dtype=f64)
    x, it, _ = PCGSolver(tolerance=1e-10, max_iter=100, preconditioner="none")(e, b,
                                                                               torch.zeros(3, dtype=f64))
    np.testing.assert_allclose(x.cpu().numpy(), b.numpy(), atol=1e-8)
    assert it <= 2
    m = mat(2, [0], [1], [4.0, 4.0], [-1.0], [-1.0])
    x, it, _ = PCGSolver(tolerance=1e-10, max_iter=100, preconditioner="none")(
        m, torch.tensor([2.0, 7.0], dtype=f64), torch.zeros(2, dtype=f64))
    np.testing.assert_allclose(x.cpu().numpy(), [1.0, 2.0], atol=1e-6)
    assert it < 20
    # max-iteration stop (:135-150)
    m = mat(2, [0], [1], [1.0, 1e8], [-1.0], [-1.0])
    x, it, _ = PCGSolver(tolerance=1e-15, max_iter=5, preconditioner="none")(
        m, torch.tensor([1.0, 1.0], dtype=f64), torch.zeros(2, dtype=f64))
    assert it <= 5
    # zero RHS (:168-182)
    m = mat(3, [0, 1], [1, 2], [4.0, 6.0, 4.0], [-1.0, -1.0], [-1.0, -1.0])
    x, it, res = PCGSolver(tolerance=1e-10, max_iter=100)(m, torch.zeros(3, dtype=f64),
                                                          torch.zeros(3, dtype=f64))
    assert it == 1 and res == 0.0 and torch.count_nonzero(x) == 0
    # factory
    s = create_solver("PCG", tolerance=1e-8)
    assert isinstance(s, PCGSolver) and s.tolerance == 1e-8


@pytest.mark.parametrize("pre", ["DIC", "DILU", "none"])
def test_pcg_matches_oracle_iteration_counts(pre):
    jc = jitter_case(6)
    nint = int(jc["n_internal"])
    own, nei = jc["owner"][:nint], jc["neighbour"]
    dg, lo, up = G["j6_lap_diag"], G["j6_lap_lower"], G["j6_lap_upper"]
    m = mat(dg.shape[0], own, nei, dg, lo, up)
    s = PCGSolver(tolerance=0.0, rel_tol=1e-10, max_iter=500, preconditioner=pre)
    x, it, res = s(m, torch.as_tensor(jc["b"]), torch.zeros(dg.shape[0], dtype=f64))
    pd = {"DIC": O.dic_build(own, nei, dg, up), "DILU": O.dilu_build(own, nei, dg, lo, up),
          "none": None}[pre]
    o = O.pcg(own, nei, dg, lo, up, jc["b"], np.zeros(dg.shape[0]), pd, 0.0, 1e-10, 500)
    assert it == o.iterations
    assert relerr(x.cpu().numpy(), o.x) < 1e-9
    assert relerr(s.last_info.residual_history, o.history) < 1e-6
    if pre == "DIC":
        assert it == int(G["j6_pcg_iterations"])
        assert relerr(x.cpu().numpy(), G["j6_pcg_x"]) < 1e-9


def test_pcg_config1_against_reference():
    """32^3 Poisson, PCG+DIC to 1e-6 relative: same iteration count
    as the reference (198, counting the iteration-0 check); x within 2e-11 of
    the reference's x (measured on GB300: 2.4e-12; the dot products sum in a
    different order than the reference's, so the two trajectories drift apart
    by rounding), and within 1e-12 after 50 iterations (measured 1.4e-13)."""
    c1 = c1_poisson(32)
    m = mat(c1["n"], c1["owner"], c1["neighbour"], c1["diag"], c1["lower"], c1["upper"])
    b = torch.as_tensor(c1["b"])
    s = PCGSolver(tolerance=0.0, rel_tol=1e-6, max_iter=1000, preconditioner="DIC")
    x, it, res = s(m, b, torch.zeros(c1["n"], dtype=f64))
    assert it == int(G["c1_pcg_iterations"]) == 198
    assert relerr(x.cpu().numpy(), G["c1_pcg_x"]) < 2e-11
    assert res / s.last_info.initial_residual < 1e-6
    s50 = PCGSolver(tolerance=0.0, rel_tol=0.0, max_iter=50, preconditioner="DIC")
    x50, it50, _ = s50(m, b, torch.zeros(c1["n"], dtype=f64))
    assert it50 == 51
    assert relerr(x50.cpu().numpy(), G["c1_pcg50_x"]) < 1e-12


# --------------------------------------------------------------------------
# PBiCGStab -- reference unit tests (tests/unit/solvers/test_pbicgstab.py)
# --------------------------------------------------------------------------
def test_pbicgstab_reference_unit_cases():
    m = mat(2, [0], [1], [4.0, 5.0], [-1.0], [-2.0])
    x, it, _ = PBiCGSTABSolver(tolerance=1e-10, max_iter=100, preconditioner="none")(
        m, torch.tensor([3.0, 3.0], dtype=f64), torch.zeros(2, dtype=f64))
    np.testing.assert_allclose(x.cpu().numpy(), [1.0, 1.0], atol=1e-4)
    m = mat(2, [0], [1], [4.0, 4.0], [-1.0], [-1.0])
    x, it, _ = PBiCGSTABSolver(tolerance=1e-10, max_iter=100, preconditioner="none")(
        m, torch.tensor([2.0, 7.0], dtype=f64), torch.zeros(2, dtype=f64))
    np.testing.assert_allclose(x.cpu().numpy(), [1.0, 2.0], atol=1e-6)
    own, nei = np.arange(9), np.arange(1, 10)
    dg = np.zeros(10)
    np.add.at(dg, own, 1.0)
    np.add.at(dg, nei, 1.5)
    m = mat(10, own, nei, dg + 0.5, -np.ones(9), -1.5 * np.ones(9))
    b = torch.ones(10, dtype=f64)
    x, it, _ = PBiCGSTABSolver(tolerance=1e-8, max_iter=500, preconditioner="DILU")(
        m, b, torch.zeros(10, dtype=f64))
    assert torch.linalg.vector_norm(b.cuda() - m.Ax(x)) < 0.1
    m = mat(3, [0, 1], [1, 2], [4.0, 6.0, 4.0], [-1.0, -1.0], [-2.0, -2.0])
    x, it, _ = PBiCGSTABSolver(tolerance=1e-10, max_iter=100)(m, torch.zeros(3, dtype=f64),
                                                             torch.zeros(3, dtype=f64))
    assert torch.count_nonzero(x) == 0


@pytest.mark.parametrize("omega", ["reference", "standard"])
def test_pbicgstab_against_oracle(omega):
    """Chain systems where BiCGStab is well conditioned: iteration counts equal
    and x within 1e-10 of the oracle running the same algorithm."""
    rng = np.random.default_rng(1)
    n = 40
    own, nei = np.arange(n - 1), np.arange(1, n)
    lo, up = -rng.uniform(0.5, 1.5, n - 1), -rng.uniform(0.5, 1.5, n - 1)
    dg = rng.uniform(3.0, 4.0, n)
    b = rng.uniform(-1, 1, n)
    m = mat(n, own, nei, dg, lo, up)
    s = PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-10, max_iter=200, omega=omega)
    x, it, _ = s(m, torch.as_tensor(b), torch.zeros(n, dtype=f64))
    o = O.pbicgstab(own, nei, dg, lo, up, b, np.zeros(n), O.dilu_build(own, nei, dg, lo, up),
                    0.0, 1e-10, 200, omega=omega)
    assert it == o.iterations
    assert relerr(x.cpu().numpy(), o.x) < 1e-10


def test_pbicgstab_first_iterations_on_jittered_mesh():
    """On this system rho = rt.r cancels to ~1e-3 of |r|^2 in the second
    iteration (the reference's omega = t.z/t.t barely reduces r), so the
    fixed-order GPU dots and the oracle's serial dots already give x that
    differ at ~2e-10 after two iterations (observed on GB300); the residual
    checks agree more tightly."""
    jc = jitter_case(6)
    nint = int(jc["n_internal"])
    own, nei = jc["owner"][:nint], jc["neighbour"]
    dg = G["j6_lap_diag"] - G["j6_div_diag"]
    lo = G["j6_lap_lower"] - G["j6_div_lower"]
    up = G["j6_lap_upper"] - G["j6_div_upper"]
    m = mat(dg.shape[0], own, nei, dg, lo, up)
    s = PBiCGSTABSolver(tolerance=0.0, rel_tol=0.0, max_iter=2)
    x, it, _ = s(m, torch.as_tensor(jc["b"]), torch.zeros(dg.shape[0], dtype=f64))
    o = O.pbicgstab(own, nei, dg, lo, up, jc["b"], np.zeros(dg.shape[0]),
                    O.dilu_build(own, nei, dg, lo, up), 0.0, 0.0, 2)
    assert it == o.iterations == 5
    assert relerr(x.cpu().numpy(), o.x) < 1e-8
    assert relerr(s.last_info.residual_history, o.history) < 1e-9


@pytest.mark.parametrize("N,prec", [(32, "DIC"), (20, "none"), (7, "DILU")])
def test_pcg_single_launch_and_kernel_forms_agree(N, prec):
    """The single cooperative launch (grid barriers) and the three-kernel
    form run the same iteration: same iteration count and status, x and the
    residual history within 1e-12 (their dot products sum in different
    block orders), both within 1e-8 of the oracle."""
    from pyopenfoam_gb300.mesh.poisson import hex_poisson

    d = hex_poisson(N, seed=7)
    m = LduMatrix(d["n"], torch.as_tensor(d["owner"]), torch.as_tensor(d["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(d[k]) for k in ("diag", "lower", "upper"))
    b = torch.as_tensor(d["b"])
    out = {}
    for launch in ("single", "kernels"):
        s = PCGSolver(tolerance=0.0, rel_tol=1e-9, max_iter=2000, preconditioner=prec,
                      launch=launch)
        x, it, res = s(m, b, torch.zeros_like(b))
        assert s.last_result.launches == (1 if launch == "single" else s.last_result.launches)
        out[launch] = (x.cpu().numpy(), it, s.last_info.converged,
                       np.array(s.last_info.residual_history))
    (xs, its, cs, hs), (xk, itk, ck, hk) = out["single"], out["kernels"]
    assert its == itk and cs and ck
    assert np.abs(xs - xk).max() <= 1e-12 * np.abs(xk).max()
    assert np.abs(hs - hk).max() <= 1e-12 * hk[0]
    pd = (None if prec == "none" else
          (O.dic_build if prec == "DIC" else lambda o, n_, dg, up: O.dilu_build(
              o, n_, dg, d["lower"], up))(d["owner"], d["neighbour"], d["diag"], d["upper"]))
    o = O.pcg(d["owner"], d["neighbour"], d["diag"], d["lower"], d["upper"], d["b"],
              np.zeros(d["n"]), pd, 0.0, 1e-9, 2000)
    assert o.iterations == its
    assert np.abs(xs - o.x).max() <= 1e-8 * np.abs(o.x).max()
    with pytest.raises(ValueError):
        PCGSolver(launch="graph")


def test_bounded_waits_give_up_instead_of_hanging():
    """Failure detection without a GPU fault: a grid-barrier wait whose
    partner block never arrives and an mbarrier wait that nothing completes
    both run out after their poll limits and report it; the context stays
    usable (a solve afterwards still works)."""
    import ctypes

    from pyopenfoam_gb300 import _lib

    out = (ctypes.c_int32 * 3)()
    _lib.check(_lib.lib().gbf_selftest_bounded_waits(out))
    assert list(out) == [1, 1, 1]
    c = c1_poisson(8)
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(c[k]) for k in ("diag", "lower", "upper"))
    x, it, res = PCGSolver(tolerance=0.0, rel_tol=1e-8, launch="single")(
        m, torch.as_tensor(c["b"]), torch.zeros(c["n"], dtype=torch.float64))
    assert it > 1 and torch.isfinite(x).all()


def test_wavefront_barrier_timeout_poisons_the_output():
    """The cooperative wavefronts' failure path, without a GPU fault: a
    barrier that can never complete runs out after its poll limit, sets the
    fault word and the output becomes NaN; the context stays usable (a DIC
    factorisation and a Gauss-Seidel sweep afterwards still work)."""
    import ctypes

    from pyopenfoam_gb300 import _lib
    from pyopenfoam_gb300.solvers.smoothers import gs_sweep

    out = (ctypes.c_int32 * 2)()
    _lib.check(_lib.lib().gbf_selftest_wavefront_fault(out))
    assert list(out) == [1, 1]
    c = c1_poisson(8)
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(k) for k in (c["diag"], c["lower"], c["upper"]))
    assert torch.isfinite(DICPreconditioner(m).precond_diag).all()
    x = torch.zeros(c["n"], dtype=torch.float64, device="cuda")
    gs_sweep(m, x, torch.as_tensor(c["b"]).cuda())
    assert torch.isfinite(x).all() and torch.count_nonzero(x) > 0


@pytest.mark.parametrize("launch", ["single", "kernels"])
def test_breakdown_and_nan_follow_the_reference(launch):
    """Failure modes of the reference solvers, reproduced (no exception, no
    hang): a zero matrix breaks down at the first p.Ap (|pAp| < 1e-30,
    pcg.py:153-156) and returns x0 unconverged after one check; a NaN in the
    right-hand side makes every comparison false, so the solve runs to
    max_iter and returns unconverged -- the same outcome as the oracle."""
    c = c1_poisson(6)
    n = c["n"]
    m = LduMatrix(n, torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    # zero matrix: breakdown
    x, it, res = PCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=50, launch=launch)(
        m, torch.as_tensor(c["b"]), torch.zeros(n, dtype=torch.float64))
    zeros = np.zeros(m.n_internal_faces)
    pd = O.dic_build(c["owner"], c["neighbour"], np.zeros(n), zeros)
    o = O.pcg(c["owner"], c["neighbour"], np.zeros(n), zeros, zeros, c["b"], np.zeros(n), pd,
              0.0, 1e-8, 50)
    assert it == o.iterations == 1 and not o.converged
    assert torch.count_nonzero(x) == 0
    # NaN right-hand side: runs to max_iter, unconverged, NaN solution
    m.diag, m.lower, m.upper = (torch.as_tensor(c[k]) for k in ("diag", "lower", "upper"))
    b = torch.as_tensor(c["b"]).clone()
    b[3] = float("nan")
    s = PCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=7, launch=launch)
    x, it, res = s(m, b, torch.zeros(n, dtype=torch.float64))
    bn = c["b"].copy()
    bn[3] = np.nan
    o = O.pcg(c["owner"], c["neighbour"], c["diag"], c["lower"], c["upper"], bn, np.zeros(n),
              O.dic_build(c["owner"], c["neighbour"], c["diag"], c["upper"]), 0.0, 1e-8, 7)
    assert not s.last_info.converged and not o.converged
    assert it == o.iterations
    assert np.isnan(res) and not torch.isfinite(x).all()


def test_pbicgstab_fp64_x_within_1e12_of_oracle_when_converged_to_1e14():
    """The FP64 path's x against the oracle's on an upwind convection-diffusion
    system: at 1e-8 the two solves stop on different trajectories (their dot
    products round in different orders), so x agrees only to ~cond * 1e-8;
    both driven to 1e-14 converge to the same x within 1e-12 relative."""
    from pyopenfoam_gb300.mesh.poisson import convection_diffusion

    d = convection_diffusion(40, seed=1)
    args = (d["owner"], d["neighbour"], d["diag"], d["lower"], d["upper"])
    m = mat(d["n"], *args)
    s = PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-14, max_iter=4000, omega="standard")
    x, it, _ = s(m, torch.as_tensor(d["b"]), torch.zeros(d["n"], dtype=f64))
    o = O.pbicgstab(*args, d["b"], np.zeros(d["n"]), O.dilu_build(*args), 0.0, 1e-14, 4000,
                    threads=8, omega="standard")
    assert s.last_info.converged and o.converged
    assert relerr(x.cpu().numpy(), o.x) < 1e-12
