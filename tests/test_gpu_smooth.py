"""SmoothSolver (GaussSeidel / DIC / DILU smoothers) and the standalone
smoothers (GaussSeidelSmoother, JacobiSmoother, DICGSmoother) on the GPU
against the reference's own outputs (tests/golden/reference_smooth.npz,
make_golden.py --smooth) on 4^3 systems with triangular and with permuted
face order (a third of the faces owner > neighbour).

Bars: x bitwise and the same iteration count; the final residual norm to
1e-13 relative (a different summation order of the same residual)."""

import os

import numpy as np
import pytest
import torch

from oracle import oracle as O

from pyopenfoam_gb300 import LduMatrix, create_solver, solver_from_dict
from pyopenfoam_gb300.solvers import (DICGSmoother, GaussSeidelSmoother, JacobiSmoother,
                                      SmoothSolver)
from tests.golden.cases import hex_poisson, random_ldu

pytestmark = pytest.mark.gpu
SM = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_smooth.npz"))


def _case(perm):
    c = random_ldu(4, seed=31, permute_faces=perm)
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(c[k]) for k in ("diag", "lower", "upper"))
    return m, torch.as_tensor(c["r"]), torch.as_tensor(c["x"])


def _eq(a, b):
    return (np.ascontiguousarray(a).view(np.int64) == np.ascontiguousarray(b).view(np.int64)).all()


@pytest.mark.parametrize("tag,perm", [("tri", False), ("perm", True)])
@pytest.mark.parametrize("sm", ["GaussSeidel", "DIC", "DILU"])
def test_smooth_solver_matches_reference(tag, perm, sm):
    m, b, x0 = _case(perm)
    s = SmoothSolver(tolerance=0.0, rel_tol=0.0, max_iter=3, smoother=sm, n_sweeps=2,
                     omega=0.9 if sm != "GaussSeidel" else 1.0)
    x, it, res = s(m, b, x0)
    assert x.device.type == "cuda"
    assert _eq(x.cpu().numpy(), SM[f"{tag}_ss_{sm}_x"]), sm
    assert it == int(SM[f"{tag}_ss_{sm}_it"])
    assert abs(res - float(SM[f"{tag}_ss_{sm}_res"])) <= 1e-13 * float(SM[f"{tag}_ss_{sm}_res"])


@pytest.mark.parametrize("tag,perm", [("tri", False), ("perm", True)])
def test_smoothers_match_reference(tag, perm):
    m, b, x0 = _case(perm)
    assert _eq(GaussSeidelSmoother(m, omega=0.8).smooth(x0, b, 2).cpu().numpy(), SM[f"{tag}_gs_x"])
    assert _eq(JacobiSmoother(m).smooth(x0, b, 3).cpu().numpy(), SM[f"{tag}_jac_x"])
    assert _eq(DICGSmoother(m, omega=0.9).smooth(x0, b, 2).cpu().numpy(), SM[f"{tag}_dicg_x"])


def test_smooth_solver_converges_and_factory():
    d = hex_poisson(12, seed=3)
    m = LduMatrix(d["n"], torch.as_tensor(d["owner"]), torch.as_tensor(d["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(d[k]) for k in ("diag", "lower", "upper"))
    b = torch.as_tensor(d["b"])
    s = solver_from_dict("smoothSolver", {"smoother": "GaussSeidel", "nSweeps": 3,
                                          "tolerance": 0.0, "relTol": 1e-3, "maxIter": 2000})
    assert isinstance(s, SmoothSolver) and s._n_sweeps == 3
    x, it, res = s(m, b, torch.zeros_like(b))
    assert s.last_info.converged
    r = b.cuda() - m.Ax(x)
    assert float(r.norm()) / float(b.norm()) < 1e-3
    assert isinstance(create_solver("smoothsolver", smoother="DIC"), SmoothSolver)
    with pytest.raises(ValueError):
        SmoothSolver(smoother="Jacobi")(m, b, torch.zeros_like(b))


@pytest.mark.parametrize("N,perm", [(24, True), (40, False)])
def test_wavefront_single_launch_matches_per_level_launches(N, perm):
    """The cooperative single-launch wavefronts (barrier memory given) and
    the per-level launches (NULL) give the same bits: DIC and DILU
    factorisations, both apply_full sweeps, Gauss-Seidel forward and
    backward (plain and relaxed)."""
    from pyopenfoam_gb300 import _lib
    from pyopenfoam_gb300.solvers.smoothers import _gs_schedule

    c = random_ldu(N, seed=17, permute_faces=perm)
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(k) for k in (c["diag"], c["lower"], c["upper"]))
    L = _lib.lib()
    topo, coef, st = m.topology(), m.packed(), _lib.stream_ptr(m.device)
    n = m.n_cells

    def both(fn):
        out = []
        for bar in (None, _lib.wavefront_barrier(m.device)):
            out.append(fn(None if bar is None else bar.data_ptr()))
            if bar is not None:
                _lib.check_wavefront(bar, "wavefront", m.device)
        return out

    def dic(b):
        d = torch.empty(n, dtype=torch.float64, device="cuda")
        s = topo.dic_schedule()
        _lib.check(L.gbf_dic_build_f64(topo.layout_ref, coef.data_ptr(), m.diag.data_ptr(),
                                       s.ptr.data_ptr(), s.items.data_ptr(), s.n_levels,
                                       s.max_level_size, d.data_ptr(), b, st))
        return d.cpu().numpy()

    def dilu(b):
        d = torch.empty(n, dtype=torch.float64, device="cuda")
        s = topo.dilu_schedule()
        _lib.check(L.gbf_dilu_build_f64(topo.layout_ref, m.lower.data_ptr(), m.upper.data_ptr(),
                                        m.diag.data_ptr(), s.ptr.data_ptr(), s.items.data_ptr(),
                                        s.n_levels, s.max_level_size, d.data_ptr(), b, st))
        return d.cpu().numpy()

    for fn in (dic, dilu):
        a, b = both(fn)
        assert _eq(a, b), fn.__name__
    pd = torch.as_tensor(dilu(None)).cuda()
    for reverse in (0, 1):
        for lower_only in (True, False):
            def sweep(b, reverse=reverse, lower_only=lower_only):
                s = topo.sweep_schedule(bool(reverse), lower_only)
                res = torch.as_tensor(c["r"]).cuda().clone()
                _lib.check(L.gbf_sweep_f64(topo.layout_ref, m.upper.data_ptr(), pd.data_ptr(),
                                           s.ptr.data_ptr(), s.items.data_ptr(), s.n_levels,
                                           s.max_level_size, reverse, res.data_ptr(), b, st))
                return res.cpu().numpy()
            a, b = both(sweep)
            assert _eq(a, b), ("sweep", reverse, lower_only)
    rhs = torch.as_tensor(c["r"]).cuda()
    for reverse in (False, True):
        for relax, omega in ((0, 1.0), (1, 0.8)):
            def gs(b, reverse=reverse, relax=relax, omega=omega):
                sch = _gs_schedule(m, reverse)
                x = torch.as_tensor(c["x"]).cuda().clone()
                _lib.check(L.gbf_gauss_seidel_f64(topo.layout_ref, coef.data_ptr(),
                                                  m.diag.data_ptr(), rhs.data_ptr(),
                                                  sch.ptr.data_ptr(), sch.cells.data_ptr(),
                                                  sch.ptr_h.ctypes.data, sch.n_levels, omega,
                                                  relax, x.data_ptr(), b, st))
                return x.cpu().numpy()
            a, b = both(gs)
            assert _eq(a, b), ("gs", reverse, relax)


@pytest.mark.parametrize("N,perm", [(12, True), (24, False), (48, True)])
def test_gauss_seidel_flow_matches_level_walks(N, perm):
    """The Gauss-Seidel sweep as a dataflow walk (gbf_gauss_seidel_flow_f64,
    the default of gs_sweep) gives the bits of the level walks (grid barrier
    per level, and a launch per level), forward and backward, plain and
    relaxed, on sorted and shuffled face orders; and the oracle's serial
    sweep.  A zero diagonal entry keeps its cell's value, and a NaN
    propagates as in the reference."""
    from pyopenfoam_gb300.solvers.smoothers import GS_FORMS, gs_sweep

    c = random_ldu(N, seed=21, permute_faces=perm)
    c["diag"] = c["diag"].copy()
    c["diag"][7] = 0.0
    c["x"] = c["x"].copy()
    c["x"][11] = np.nan
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(k) for k in (c["diag"], c["lower"], c["upper"]))
    rhs = torch.as_tensor(c["r"]).cuda()
    for reverse in (False, True):
        for relax, omega in ((False, 1.0), (True, 0.8)):
            out = {}
            for form in GS_FORMS:
                x = torch.as_tensor(c["x"]).cuda().clone()
                gs_sweep(m, x, rhs, reverse=reverse, omega=omega, relax=relax, form=form)
                gs_sweep(m, x, rhs, reverse=reverse, omega=omega, relax=relax, form=form)
                out[form] = x.cpu().numpy()
            for form in GS_FORMS[1:]:
                np.testing.assert_array_equal(out["flow"], out[form],
                                              err_msg=f"{form} {reverse} {relax}")
            if not reverse and not relax:
                ref = O.gauss_seidel(c["owner"], c["neighbour"], c["diag"], c["lower"],
                                     c["upper"], c["r"], c["x"], 2)
                np.testing.assert_array_equal(out["flow"], ref)


@pytest.mark.parametrize("N,perm", [(12, True), (32, False), (40, True)])
def test_apply_full_flow_matches_level_walks(N, perm):
    """DIC and DILU apply_full with their triangular sweeps as dataflow walks
    (gbf_sweep_flow_f64, the default) give the bits of the barrier walk and
    of the per-level launches, and of the oracle, on sorted and shuffled
    face orders (a face may read a cell that later faces still update)."""
    from pyopenfoam_gb300.solvers.preconditioners import DICPreconditioner, DILUPreconditioner
    from pyopenfoam_gb300.solvers.sweeps import SWEEP_FORMS, dic_apply_full, dilu_apply_full

    c = random_ldu(N, seed=33, permute_faces=perm)
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(k) for k in (c["diag"], c["lower"], c["upper"]))
    r = torch.as_tensor(c["r"]).cuda()
    for cls, fn, ofn in ((DICPreconditioner, dic_apply_full, O.dic_apply_full),
                         (DILUPreconditioner, dilu_apply_full, O.dilu_apply_full)):
        pre = cls(m)
        out = {f: fn(pre, r, form=f).cpu().numpy() for f in SWEEP_FORMS}
        for f in SWEEP_FORMS[1:]:
            np.testing.assert_array_equal(out["flow"], out[f], err_msg=f"{cls.__name__} {f}")
        pd = pre.precond_diag.cpu().numpy()
        if cls is DICPreconditioner:
            ref = ofn(c["owner"], c["neighbour"], c["upper"], pd, c["r"])
        else:
            ref = ofn(c["owner"], c["neighbour"], c["lower"], c["upper"], pd, c["r"])
        np.testing.assert_array_equal(out["flow"], ref)
