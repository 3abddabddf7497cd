"""Generate the golden fixtures of the parity tests from the reference itself.

Run in a checkout that has the reference project next to it:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM

It imports the reference's own classes (``pyfoam.core.ldu_matrix``,
``pyfoam.solvers.*``, ``pyfoam.discretisation.operators.fvm``,
``pyfoam.differentiable.linear_solver``) and stores their outputs on seeded
inputs in ``tests/golden/*.npz``.  Bitwise results are stored as SHA-256 of
the little-endian float64 bytes (plus the arrays where small); solver
solutions are stored in full.  The tests never import the reference: they
only read these files.
"""

from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.dont_write_bytecode = True

from tests.golden.cases import (  # noqa: E402
    c1_poisson, jitter_case, random_ldu, sha, unroll_case,
)


def main(ref_root: str) -> None:
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import torch
    from pyfoam.core.ldu_matrix import LduMatrix
    from pyfoam.differentiable.linear_solver import DifferentiableLinearSolve
    from pyfoam.discretisation.operators import fvm
    from pyfoam.solvers.pbicgstab import PBiCGSTABSolver
    from pyfoam.solvers.pcg import PCGSolver
    from pyfoam.solvers.preconditioners import DICPreconditioner, DILUPreconditioner
    from pyfoam.solvers.residual import ResidualMonitor

    torch.set_num_threads(8)
    t = torch.from_numpy

    def ldu(n, own, nei, d, lo, up, dtype=torch.float64):
        m = LduMatrix(n, t(own), t(nei), dtype=dtype)
        m.diag, m.lower, m.upper = t(d), t(lo), t(up)
        return m

    out = {}

    # ---- 1. Amul / Ax_T / DIC / DILU on a seeded random LDU over a 32^3 mesh
    for name, N, perm in (("ldu32", 32, False), ("ldu12p", 12, True)):
        case = random_ldu(N, seed=5, permute_faces=perm)
        own, nei = case["owner"], case["neighbour"]
        m = ldu(case["n"], own, nei, case["diag"], case["lower"], case["upper"])
        x = t(case["x"])
        out[f"{name}_Ax_sha"] = sha(m.Ax(x).numpy())
        out[f"{name}_AxT_sha"] = sha(m.Ax_T(x).numpy())
        out[f"{name}_dic_sha"] = sha(DICPreconditioner(m)._precond_diag.numpy())
        out[f"{name}_dilu_sha"] = sha(DILUPreconditioner(m)._precond_diag.numpy())
        m32 = ldu(case["n"], own, nei, case["diag"], case["lower"], case["upper"], torch.float32)
        out[f"{name}_Ax_f32_sha"] = sha(m32.Ax(x.float()).numpy())
        if N <= 12:
            r = t(case["r"])
            out[f"{name}_dic_full_sha"] = sha(DICPreconditioner(m).apply_full(r).numpy())
            out[f"{name}_dilu_full_sha"] = sha(DILUPreconditioner(m).apply_full(r).numpy())
        print(name, "done", flush=True)

    # ---- 2. Config-1 Poisson (32^3, Dirichlet x=0), PCG+DIC to rel 1e-6
    c1 = c1_poisson(32)
    m = ldu(c1["n"], c1["owner"], c1["neighbour"], c1["diag"], c1["lower"], c1["upper"])
    out["c1_coeff_sha"] = sha(np.concatenate([c1["diag"], c1["lower"], c1["upper"]]))
    mon = ResidualMonitor(tolerance=0.0, rel_tol=1e-6, min_iter=0)
    solver = PCGSolver(tolerance=0.0, rel_tol=1e-6, max_iter=1000, preconditioner="DIC")
    x, info = solver._solve(m, t(c1["b"]), torch.zeros(c1["n"], dtype=torch.float64), mon, 1000)
    out["c1_pcg_x"] = x.numpy()
    out["c1_pcg_iterations"] = np.int64(info.iterations)
    out["c1_pcg_history"] = np.array(info.residual_history)
    # same system, fixed 50 iterations, tolerance 0 (trajectory comparison)
    solver50 = PCGSolver(tolerance=0.0, rel_tol=0.0, max_iter=50, preconditioner="DIC")
    x50, it50, _ = solver50(m, t(c1["b"]), torch.zeros(c1["n"], dtype=torch.float64))
    out["c1_pcg50_x"] = x50.numpy()
    out["c1_pcg50_iterations"] = np.int64(it50)
    print("c1 done, iterations", info.iterations, flush=True)

    # ---- 3. Jittered 6^3 mesh: fvm.laplacian(gamma) and fvm.div(phi, upwind),
    #         A = L - D solved by PBiCGStab+DILU and PCG+DIC on L
    jc = jitter_case(6, seed=1)
    mesh = jc["mesh"]
    L = fvm.laplacian(t(jc["gamma"]), torch.zeros(mesh.n_cells, dtype=torch.float64), mesh=mesh)
    Dv = fvm.div(t(jc["phi"]), torch.zeros(mesh.n_cells, dtype=torch.float64), "Gauss upwind",
                 mesh=mesh)
    for k, a in (("lap_lower", L.lower), ("lap_upper", L.upper), ("lap_diag", L.diag),
                 ("div_lower", Dv.lower), ("div_upper", Dv.upper), ("div_diag", Dv.diag)):
        out[f"j6_{k}"] = a.numpy().copy()
    # per-cell diffusivity (linear interpolation to faces) and a scalar one
    dcell = np.random.default_rng(7).lognormal(0.0, 1.0, mesh.n_cells)
    Lc = fvm.laplacian(t(dcell), torch.zeros(mesh.n_cells, dtype=torch.float64), mesh=mesh)
    Ls = fvm.laplacian(1.5, torch.zeros(mesh.n_cells, dtype=torch.float64), mesh=mesh)
    out["j6_dcell"] = dcell
    for k, a in (("lapc_lower", Lc.lower), ("lapc_upper", Lc.upper), ("lapc_diag", Lc.diag),
                 ("laps_lower", Ls.lower), ("laps_upper", Ls.upper), ("laps_diag", Ls.diag)):
        out[f"j6_{k}"] = a.numpy().copy()
    A = LduMatrix(mesh.n_cells, mesh.owner[: mesh.n_internal_faces], mesh.neighbour)
    A.diag, A.lower, A.upper = L.diag - Dv.diag, L.lower - Dv.lower, L.upper - Dv.upper
    b = t(jc["b"])
    s2 = PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-10, max_iter=500, preconditioner="DILU")
    x2, it2, r2 = s2(A, b, torch.zeros(mesh.n_cells, dtype=torch.float64))
    out["j6_bicg_x"], out["j6_bicg_iterations"] = x2.numpy(), np.int64(it2)
    s3 = PCGSolver(tolerance=0.0, rel_tol=1e-10, max_iter=500, preconditioner="DIC")
    x3, it3, _ = s3(L, b, torch.zeros(mesh.n_cells, dtype=torch.float64))
    out["j6_pcg_x"], out["j6_pcg_iterations"] = x3.numpy(), np.int64(it3)
    print("j6 done", it2, it3, flush=True)

    # ---- 4. DifferentiableLinearSolve gradients on the 6^3 Laplacian + I
    diag = (L.diag + 10.0).clone().requires_grad_(True)
    lower = L.lower.clone().requires_grad_(True)
    upper = L.upper.clone().requires_grad_(True)
    bb = b.clone().requires_grad_(True)
    sol = PCGSolver(tolerance=0.0, rel_tol=1e-14, max_iter=2000, preconditioner="none")
    own_t = mesh.owner[: mesh.n_internal_faces]
    xs = DifferentiableLinearSolve.apply(diag, lower, upper, bb, sol, own_t, mesh.neighbour,
                                         torch.zeros(mesh.n_cells, dtype=torch.float64), 0.0,
                                         2000)
    w = t(jc["w"])
    loss = (w * xs).sum() + (xs * xs).sum()
    loss.backward()
    out["dls_x"] = xs.detach().numpy()
    out["dls_grad_diag"] = diag.grad.numpy()
    out["dls_grad_lower"] = lower.grad.numpy()
    out["dls_grad_upper"] = upper.grad.numpy()
    out["dls_grad_b"] = bb.grad.numpy()
    print("dls done", flush=True)

    # ---- 5. Unrolled implicit diffusion: 20 steps of (I/dt + L(gamma)) x' = x/dt
    #         through fvm.laplacian (autograd) and DifferentiableLinearSolve
    uc = unroll_case(10)
    mesh10 = uc["mesh"]
    gam = t(uc["gamma"]).clone().requires_grad_(True)
    solver = PCGSolver(tolerance=0.0, rel_tol=1e-14, max_iter=5000, preconditioner="none")
    own10 = mesh10.owner[: mesh10.n_internal_faces]

    def run(gamma, x0):
        lap = fvm.laplacian(gamma, torch.zeros(mesh10.n_cells, dtype=torch.float64), mesh=mesh10)
        d = lap.diag + 1.0 / uc["dt"]
        x = x0
        for _ in range(uc["steps"]):
            x = DifferentiableLinearSolve.apply(d, lap.lower, lap.upper, x / uc["dt"], solver,
                                                own10, mesh10.neighbour, x, 0.0, 5000)
        return x

    xT = run(gam, t(uc["x0"]))
    loss = ((xT - t(uc["target"])) ** 2).sum()
    loss.backward()
    out["unroll_target"] = uc["target"]
    out["unroll_xT"] = xT.detach().numpy()
    out["unroll_loss"] = np.float64(loss.item())
    out["unroll_grad"] = gam.grad.numpy()
    print("unroll done", float(loss), flush=True)

    path = os.path.join(HERE, "reference_outputs.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYFOAM_REFERENCE", ""))
