"""Times the reference's own PyTorch CPU path beside the oracle's C port -- a
MEASUREMENT RECIPE, test infrastructure like the rest of ``oracle/``.

The reference (pyOpenFOAM) is Python on PyTorch; it is imported from a
checkout given on the command line and run through its public classes
(``LduMatrix``, ``DICPreconditioner``, ``DILUPreconditioner``, ``PCGSolver``,
``PBiCGSTABSolver``, ``fvm.laplacian``, ``DifferentiableLinearSolve``) with
``torch.set_num_threads`` = the usable cores.  The oracle's threaded C port
(``oracle.py``) runs the same cases on the same cores, so the two CPU figures
compare directly.  Nothing here runs on a GPU, and nothing in the product,
the tests or ``bench.py`` imports this file.

    PYTHONDONTWRITEBYTECODE=1 python oracle/time_reference_cpu.py /path/to/pyOpenFOAM \
        [--c1] [--c2] [--c3] [--c5]

One JSON line per case:

* ``--c1`` 32^3 Poisson (seed 0), PCG+DIC to 1e-6 relative: full solves,
  median of 3 (``solvers/pcg.py:97-187``).
* ``--c2`` 128^3 upwind convection-diffusion (``convection_diffusion(128)``),
  PBiCGStab+DILU (``solvers/pbicgstab.py:103-239``,
  ``solvers/preconditioners.py:228-272``): ``Ax``, the DILU factorisation,
  ``DILUPreconditioner.apply``, and the cost of an iteration (two solves of
  different lengths without a preconditioner, plus two applications); a
  full solve is extrapolated to the FP64 GPU solver's 387 iterations.
* ``--c3`` 256^3 Poisson (seed 2), PCG+DIC: ``Ax``
  (``core/ldu_matrix.py:172-217``, median of 3), the DIC factorisation
  (``solvers/preconditioners.py:88-133``), ``DICPreconditioner.apply`` and
  the cost of an iteration as for c2 (one application); a full solve is
  extrapolated to the 1991 iterations of the FP64 PCG on this system.
* ``--c5`` 96^3 adjoint workload (per-face LogNormal(0, 1) diffusivity,
  20 implicit steps of dt = 1e-3): the reference's gradient through
  ``fvm.laplacian`` and ``DifferentiableLinearSolve`` with
  ``PCGSolver(tolerance=0, rel_tol=1e-13, preconditioner="none")``
  (``differentiable/linear_solver.py:99-151``), forward and backward timed
  apart; the port's forward + adjoint (PCG+DIC to 1e-14) beside it.
"""

from __future__ import annotations

import json
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.dont_write_bytecode = True

FP64_ITERATIONS_C2 = 387   # FP64 GPU PBiCGStab+DILU on the 128^3 system, 1e-8
FP64_ITERATIONS_C3 = 1991  # FP64 GPU PCG+DIC on the 256^3 system, 1e-10


def _cores() -> int:
    return len(os.sched_getaffinity(0))


def _cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def _emit(case: str, **kw) -> None:
    print(json.dumps({"case": case, "cores": _cores(), "cpu": _cpu_model(), **kw}), flush=True)


def _timed(fn):
    t0 = time.perf_counter()
    out = fn()
    return time.perf_counter() - t0, out


def _ref_matrix(torch, LduMatrix, d):
    t = torch.from_numpy
    m = LduMatrix(int(d["n"]), t(d["owner"]), t(d["neighbour"]))
    m.diag, m.lower, m.upper = t(d["diag"]), t(d["lower"]), t(d["upper"])
    return m


def case_c1(torch, ref) -> None:
    from oracle import oracle as O
    from pyopenfoam_gb300.mesh.poisson import hex_poisson

    d = hex_poisson(32, seed=0)
    m = _ref_matrix(torch, ref.LduMatrix, d)
    b, x0 = torch.from_numpy(d["b"]), torch.zeros(d["n"], dtype=torch.float64)
    s = ref.PCGSolver(tolerance=0.0, rel_tol=1e-6, max_iter=1000, preconditioner="DIC")
    runs = [_timed(lambda: s(m, b, x0)) for _ in range(3)]
    ref_s = statistics.median(r[0] for r in runs)
    it = runs[0][1][1]

    def port():
        pd = O.dic_build(d["owner"], d["neighbour"], d["diag"], d["upper"])
        return O.pcg(d["owner"], d["neighbour"], d["diag"], d["lower"], d["upper"], d["b"],
                     np.zeros(d["n"]), pd, 0.0, 1e-6, 1000, threads=_cores())

    pruns = [_timed(port) for _ in range(3)]
    _emit("c1: 32^3 Poisson PCG+DIC to 1e-6, full solve", reference_s=ref_s,
          reference_iterations=int(it), port_s=statistics.median(p[0] for p in pruns),
          port_iterations=pruns[0][1].iterations)


def _ref_iteration_cost(make_solver, m, b, x0, k1, k2):
    """Seconds per iteration of the reference solver without a
    preconditioner: two solves of k1 and k2 iterations, the difference over
    k2 - k1 (the per-call set-up cancels)."""
    s1, s2 = make_solver(k1), make_solver(k2)
    t1, _ = _timed(lambda: s1(m, b, x0))
    t2, _ = _timed(lambda: s2(m, b, x0))
    return max(t2 - t1, 0.0) / (k2 - k1)


def case_c2(torch, ref) -> None:
    from oracle import oracle as O
    from pyopenfoam_gb300.mesh.poisson import convection_diffusion

    d = convection_diffusion(128, seed=1)
    m = _ref_matrix(torch, ref.LduMatrix, d)
    b, x0 = torch.from_numpy(d["b"]), torch.zeros(d["n"], dtype=torch.float64)
    k = 10
    t_ax = statistics.median(_timed(lambda: m.Ax(b))[0] for _ in range(3))
    t_dilu, P = _timed(lambda: ref.DILUPreconditioner(m))
    t_apply = statistics.median(_timed(lambda: P.apply(b))[0] for _ in range(5))
    # the DILU factorisation (a Python loop over the faces, ~140 s here) varies by
    # more than a few iterations cost, so the iterations are timed without a
    # preconditioner and the two diagonal applications per iteration
    # (z = r / D) added from their own timing
    per_none = _ref_iteration_cost(
        lambda j: ref.PBiCGSTABSolver(tolerance=0.0, rel_tol=0.0, max_iter=j,
                                      preconditioner="none"), m, b, x0, 5, 5 + 2 * k)
    per_it = per_none + 2 * t_apply

    own, nei = d["owner"], d["neighbour"]
    p_dilu, pd = _timed(lambda: O.dilu_build(own, nei, d["diag"], d["lower"], d["upper"]))

    def psolve(j):
        return _timed(lambda: O.pbicgstab(own, nei, d["diag"], d["lower"], d["upper"], d["b"],
                                          np.zeros(d["n"]), pd, 0.0, 0.0, j,
                                          threads=_cores()))[0]

    p_short, p_long = psolve(2), psolve(2 + k)
    p_it = max(p_long - p_short, 0.0) / k
    _emit("c2: 128^3 convection-diffusion PBiCGStab+DILU", reference_ax_s=t_ax,
          reference_dilu_build_s=t_dilu, reference_apply_s=t_apply,
          reference_s_per_iteration_unpreconditioned=per_none,
          reference_s_per_iteration=per_it,
          reference_full_solve_s_extrapolated=t_dilu + t_ax + FP64_ITERATIONS_C2 * per_it,
          port_dilu_build_s=p_dilu, port_s_per_iteration=p_it,
          port_full_solve_s_extrapolated=p_dilu + p_short + FP64_ITERATIONS_C2 * p_it,
          iterations_extrapolated_to=FP64_ITERATIONS_C2, extrapolated=True)


def case_c3(torch, ref) -> None:
    from oracle import oracle as O
    from pyopenfoam_gb300.mesh.poisson import hex_poisson

    d = hex_poisson(256, seed=2)
    m = _ref_matrix(torch, ref.LduMatrix, d)
    b, x0 = torch.from_numpy(d["b"]), torch.zeros(d["n"], dtype=torch.float64)
    k = 10
    m.Ax(b)
    t_ax = statistics.median(_timed(lambda: m.Ax(b))[0] for _ in range(3))
    print("c3: Ax", t_ax, flush=True)
    t_dic, P = _timed(lambda: ref.DICPreconditioner(m))
    print("c3: DIC build", t_dic, flush=True)
    t_apply = statistics.median(_timed(lambda: P.apply(b))[0] for _ in range(5))
    # as for c2: iterations timed without a preconditioner, plus one diagonal
    # application per iteration
    per_none = _ref_iteration_cost(
        lambda j: ref.PCGSolver(tolerance=0.0, rel_tol=0.0, max_iter=j, preconditioner="none"),
        m, b, x0, 2, 2 + k)
    per_it = per_none + t_apply

    own, nei = d["owner"], d["neighbour"]
    p_dic, pd = _timed(lambda: O.dic_build(own, nei, d["diag"], d["upper"]))

    def psolve(j):
        return _timed(lambda: O.pcg(own, nei, d["diag"], d["lower"], d["upper"], d["b"],
                                    np.zeros(d["n"]), pd, 0.0, 0.0, j, threads=_cores()))[0]

    p_short, p_long = psolve(2), psolve(2 + 2 * k)
    p_it = max(p_long - p_short, 0.0) / (2 * k)
    _emit("c3: 256^3 Poisson PCG+DIC", reference_ax_s=t_ax, reference_dic_build_s=t_dic,
          reference_apply_s=t_apply, reference_s_per_iteration_unpreconditioned=per_none,
          reference_s_per_iteration=per_it,
          reference_full_solve_s_extrapolated=t_dic + t_ax + FP64_ITERATIONS_C3 * per_it,
          port_dic_build_s=p_dic, port_s_per_iteration=p_it,
          port_full_solve_s_extrapolated=p_dic + p_short + FP64_ITERATIONS_C3 * p_it,
          iterations_extrapolated_to=FP64_ITERATIONS_C3, extrapolated=True)


def case_c5(torch, ref) -> None:
    from oracle.adjoint import unrolled_adjoint
    from pyopenfoam_gb300.mesh import HexMesh
    from tests.golden.cases import unroll_case

    N = 96
    uc = unroll_case(N)
    mesh = uc["mesh"]
    t = torch.from_numpy
    gam = t(uc["gamma"]).clone().requires_grad_(True)
    solver = ref.PCGSolver(tolerance=0.0, rel_tol=1e-13, max_iter=50000, preconditioner="none")
    own = mesh.owner[: mesh.n_internal_faces]

    def forward():
        lap = ref.fvm.laplacian(gam, torch.zeros(mesh.n_cells, dtype=torch.float64), mesh=mesh)
        dg = lap.diag + 1.0 / uc["dt"]
        x = t(uc["x0"])
        for _ in range(uc["steps"]):
            x = ref.DifferentiableLinearSolve.apply(dg, lap.lower, lap.upper, x / uc["dt"],
                                                    solver, own, mesh.neighbour, x, 0.0, 50000)
        return ((x - t(uc["target"])) ** 2).sum()

    t_f, loss = _timed(forward)
    print("c5: reference forward", t_f, flush=True)
    t_b, _ = _timed(loss.backward)
    g_ref = gam.grad.numpy().copy()

    hm = HexMesh(N)
    p_loss, p_grad, p_f, p_b = unrolled_adjoint(hm, uc["gamma"], uc["x0"], uc["target"],
                                                uc["dt"], uc["steps"], _cores())
    _emit("c5: 96^3 adjoint, 20 implicit steps", reference_forward_s=t_f,
          reference_backward_s=t_b, reference_total_s=t_f + t_b,
          reference_solver="PCG, no preconditioner, rel_tol 1e-13",
          reference_loss=float(loss.item()), port_forward_s=p_f, port_backward_s=p_b,
          port_total_s=p_f + p_b, port_solver="PCG+DIC, rel_tol 1e-14", port_loss=p_loss,
          grad_rel_err_port_vs_reference=float(np.abs(p_grad - g_ref).max() /
                                               np.abs(g_ref).max()))


def main() -> None:
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("PYFOAM_REFERENCE", "")
    if not root:
        sys.exit("usage: time_reference_cpu.py /path/to/pyOpenFOAM [--c1] [--c2] [--c3] [--c5]")
    sys.path.insert(0, os.path.join(root, "src"))
    import torch
    from types import SimpleNamespace

    from pyfoam.core.ldu_matrix import LduMatrix
    from pyfoam.differentiable.linear_solver import DifferentiableLinearSolve
    from pyfoam.discretisation.operators import fvm
    from pyfoam.solvers.pbicgstab import PBiCGSTABSolver
    from pyfoam.solvers.pcg import PCGSolver
    from pyfoam.solvers.preconditioners import DICPreconditioner, DILUPreconditioner

    torch.set_num_threads(_cores())
    ref = SimpleNamespace(LduMatrix=LduMatrix, DICPreconditioner=DICPreconditioner,
                          DILUPreconditioner=DILUPreconditioner, PCGSolver=PCGSolver,
                          PBiCGSTABSolver=PBiCGSTABSolver, fvm=fvm,
                          DifferentiableLinearSolve=DifferentiableLinearSolve)
    flags = [a for a in sys.argv[1:] if a.startswith("--")] or ["--c1", "--c2", "--c3", "--c5"]
    for f, fn in (("--c1", case_c1), ("--c2", case_c2), ("--c3", case_c3), ("--c5", case_c5)):
        if f in flags:
            fn(torch, ref)


if __name__ == "__main__":
    main()
