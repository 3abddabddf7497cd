"""Generate the golden fixtures of the parity tests from the reference itself.

Run in a checkout that has the reference project next to it:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM --dlap
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM --geometry
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM --pressure
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM --smooth
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM --gamg
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM --pbicg
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM --ldu128
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM --unroll24
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/pyOpenFOAM --unroll96

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

    # ---- 2. 32^3 Poisson (Dirichlet x=0), PCG+DIC to rel 1e-6
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


# 2-cell stacked-cube mesh of the reference's differentiable-operator unit
# tests (tests/unit/differentiable/test_operators.py:26-72): points, faces,
# owner / neighbour and patches as given there.
_TWO_CELL_POINTS = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1],
                    [0, 1, 1], [0, 0, 2], [1, 0, 2], [1, 1, 2], [0, 1, 2]]
_TWO_CELL_FACES = [[4, 5, 6, 7], [0, 3, 2, 1], [0, 1, 5, 4], [3, 7, 6, 2], [0, 4, 7, 3],
                   [1, 2, 6, 5], [8, 9, 10, 11], [4, 5, 9, 8], [7, 11, 10, 6], [4, 8, 11, 7],
                   [5, 6, 10, 9]]
_TWO_CELL_OWNER = [0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1]


def dlap(ref_root: str) -> None:
    """DifferentiableLaplacian forward / backward goldens
    (differentiable/operators.py:409-643) and the pressure-equation caller
    (solvers/pressure_equation.py:49-184) -> reference_dlap.npz."""
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import torch
    from pyfoam.core.dtype import INDEX_DTYPE
    from pyfoam.differentiable.operators import DifferentiableLaplacian
    from pyfoam.mesh.fv_mesh import FvMesh

    torch.set_num_threads(8)
    t = torch.from_numpy
    out = {}

    def run(tag, mesh, phi, D, g):
        ph = t(phi).clone().requires_grad_(True)
        Dt = D
        if isinstance(D, np.ndarray):
            Dt = t(D).clone().requires_grad_(True)
        elif isinstance(D, torch.Tensor):
            Dt = D.clone().requires_grad_(True)
        lap = DifferentiableLaplacian.apply(ph, Dt, mesh)
        (lap * t(g)).sum().backward()
        out[f"{tag}_lap"] = lap.detach().numpy().copy()
        out[f"{tag}_grad_phi"] = ph.grad.numpy().copy()
        if isinstance(Dt, torch.Tensor):
            out[f"{tag}_grad_D"] = Dt.grad.numpy().copy()

    # jittered 6^3 mesh: per-face, per-cell, 0-d tensor and float D
    jc = jitter_case(6, seed=1)
    mesh = jc["mesh"]
    rng = np.random.default_rng(8)
    phi = rng.uniform(-1.0, 1.0, mesh.n_cells)
    out["j6_phi"] = phi
    dcell = np.random.default_rng(7).lognormal(0.0, 1.0, mesh.n_cells)
    run("j6_face", mesh, phi, jc["gamma"], jc["w"])
    run("j6_cell", mesh, phi, dcell, jc["w"])
    run("j6_scalar", mesh, phi, torch.tensor(1.5, dtype=torch.float64), jc["w"])
    run("j6_float", mesh, phi, 2.0, jc["w"])

    # the reference unit-test mesh
    m2 = FvMesh(points=torch.tensor(_TWO_CELL_POINTS, dtype=torch.float64),
                faces=[torch.tensor(f, dtype=INDEX_DTYPE) for f in _TWO_CELL_FACES],
                owner=torch.tensor(_TWO_CELL_OWNER, dtype=INDEX_DTYPE),
                neighbour=torch.tensor([1], dtype=INDEX_DTYPE),
                boundary=[{"name": "bottom", "type": "wall", "startFace": 1, "nFaces": 5},
                          {"name": "top", "type": "wall", "startFace": 6, "nFaces": 5}])
    m2.compute_geometry()
    for k, a in (("owner", m2.owner), ("neighbour", m2.neighbour), ("face_areas", m2.face_areas),
                 ("delta", m2.delta_coefficients), ("volumes", m2.cell_volumes),
                 ("cell_centres", m2.cell_centres), ("face_centres", m2.face_centres)):
        out[f"two_{k}"] = a.numpy().copy()
    out["two_n_internal"] = np.int64(m2.n_internal_faces)
    ones = np.ones(2)
    run("two_float", m2, np.array([1.0, 2.0]), 1.0, ones)
    run("two_scalar", m2, np.array([1.0, 2.0]), torch.tensor(1.5, dtype=torch.float64), ones)
    run("two_face", m2, np.array([1.0, 2.0]), np.linspace(0.5, 1.5, m2.n_faces), ones)

    # assemble_pressure_equation / solve_pressure_equation on the jittered
    # 6^3 mesh (solvers/pressure_equation.py:49-184)
    from pyfoam.discretisation.weights import compute_centre_weights
    from pyfoam.solvers.pcg import PCGSolver
    from pyfoam.solvers.pressure_equation import (assemble_pressure_equation,
                                                  solve_pressure_equation)

    prng = np.random.default_rng(9)
    A_p = prng.uniform(0.5, 3.0, mesh.n_cells) * np.where(prng.random(mesh.n_cells) < 0.2, -1, 1)
    A_p[3] = 0.0  # clamp to 1e-30
    phiH = prng.uniform(-1.0, 1.0, mesh.n_faces)
    wts = compute_centre_weights(mesh.cell_centres, mesh.face_centres, mesh.owner,
                                 mesh.neighbour, mesh.n_internal_faces, mesh.n_faces,
                                 dtype=torch.float64)
    peq = assemble_pressure_equation(t(phiH), t(A_p), mesh, face_weights=wts)
    out["p_A_p"], out["p_phiHbyA"] = A_p, phiH
    for k in ("lower", "upper", "diag", "source"):
        out[f"p_{k}"] = getattr(peq, k).numpy().copy()
    # a well-posed solve: A_p > 0, pinned reference cell
    A_s = prng.uniform(0.5, 3.0, mesh.n_cells)
    out["p_A_s"] = A_s
    peq = assemble_pressure_equation(t(phiH), t(A_s), mesh, face_weights=wts)
    psol = PCGSolver(tolerance=0.0, rel_tol=1e-6, max_iter=2000, preconditioner="DIC")
    p_new, p_it, p_res = solve_pressure_equation(peq, torch.zeros(mesh.n_cells,
                                                                  dtype=torch.float64),
                                                 psol, tolerance=0.0, max_iter=2000,
                                                 reference_cell=5)
    out["p_x"], out["p_iterations"], out["p_residual"] = (p_new.numpy().copy(), np.int64(p_it),
                                                          np.float64(p_res))
    print("pressure", p_it, p_res, flush=True)

    path = os.path.join(HERE, "reference_dlap.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def geometry(ref_root: str) -> None:
    """FvMesh geometry goldens (mesh/fv_mesh.py:75-148 on
    mesh/mesh_geometry.py:35-395) of a jittered hex polyMesh, a triangular
    prism polyMesh and the reference's own two-cell unit-test mesh, inputs
    included -> reference_geometry.npz."""
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import torch
    from pyfoam.core.dtype import INDEX_DTYPE
    from pyfoam.mesh.fv_mesh import FvMesh

    from tests.golden.cases import hex_polymesh, prism_polymesh

    torch.set_num_threads(8)
    out = {}
    two = dict(points=np.array(_TWO_CELL_POINTS, np.float64),
               face_ptr=np.arange(0, 4 * len(_TWO_CELL_FACES) + 1, 4),
               face_pts=np.array(_TWO_CELL_FACES, np.int64).ravel(),
               owner=np.array(_TWO_CELL_OWNER, np.int64), neighbour=np.array([1], np.int64))
    for tag, mesh in (("hex", hex_polymesh(4, 3, 3)), ("prism", prism_polymesh(3, 2, 2)),
                      ("two", two)):
        ptr, pts = mesh["face_ptr"], mesh["face_pts"]
        faces = [torch.tensor(pts[ptr[i]:ptr[i + 1]], dtype=INDEX_DTYPE)
                 for i in range(ptr.shape[0] - 1)]
        m = FvMesh(points=torch.tensor(mesh["points"], dtype=torch.float64), faces=faces,
                   owner=torch.tensor(mesh["owner"], dtype=INDEX_DTYPE),
                   neighbour=torch.tensor(mesh["neighbour"], dtype=INDEX_DTYPE))
        m.compute_geometry()
        for k in ("points", "face_ptr", "face_pts", "owner", "neighbour"):
            out[f"{tag}_{k}"] = np.asarray(mesh[k])
        for k in ("face_centres", "face_areas", "cell_volumes", "cell_centres", "face_weights",
                  "delta_coefficients"):
            out[f"{tag}_{k}"] = getattr(m, k).numpy().copy()
        out[f"{tag}_n_cells"] = np.int64(m.n_cells)
        print(tag, m.n_cells, float(m.total_volume), flush=True)
    path = os.path.join(HERE, "reference_geometry.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def pressure(ref_root: str) -> None:
    """Pressure-corrector steps either side of the solve on the jittered 6^3
    mesh: correct_velocity, correct_face_flux, adjust_phi
    (solvers/pressure_equation.py:187-377) and the Rhie-Chow functions
    (solvers/rhie_chow.py:56-250) -> reference_pressure.npz."""
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import torch
    from pyfoam.discretisation.weights import compute_centre_weights
    from pyfoam.solvers import rhie_chow as RC
    from pyfoam.solvers.pressure_equation import (adjust_phi, correct_face_flux,
                                                  correct_velocity)

    torch.set_num_threads(8)
    t = torch.from_numpy
    jc = jitter_case(6, seed=1)
    mesh = jc["mesh"]
    n, nf, ni = mesh.n_cells, mesh.n_faces, mesh.n_internal_faces
    w = compute_centre_weights(mesh.cell_centres, mesh.face_centres, mesh.owner, mesh.neighbour,
                               ni, nf, dtype=torch.float64)
    mesh.face_weights = w
    rng = np.random.default_rng(21)
    A_p = rng.uniform(0.5, 3.0, n) * np.where(rng.random(n) < 0.2, -1, 1)
    A_p[4] = 0.0
    p = rng.uniform(-1.0, 1.0, n)
    H = rng.normal(0.0, 1.0, (n, 3))
    HbyA = rng.normal(0.0, 1.0, (n, 3))
    HbyA[7] = [3e4, -2e4, 1e4]  # above the 1e4 velocity limit
    phi = rng.normal(0.0, 1.0, nf)
    out = dict(A_p=A_p, p=p, H=H, HbyA=HbyA, phi=phi, weights=w.numpy().copy())
    out["cv"] = correct_velocity(t(HbyA), t(HbyA), t(p), t(A_p), mesh).numpy().copy()
    out["cv_a07"] = correct_velocity(t(HbyA), t(HbyA), t(p), t(A_p), mesh,
                                     alpha=0.7).numpy().copy()
    out["cff"] = correct_face_flux(t(phi), t(p), t(A_p), mesh, face_weights=w).numpy().copy()
    ph = t(phi).clone()
    out["adj_ret"] = np.int64(adjust_phi(ph, mesh))
    out["adj_phi"] = ph.numpy().copy()
    own, nei = mesh.owner, mesh.neighbour
    S, dl, V = mesh.face_areas, mesh.delta_coefficients, mesh.cell_volumes
    out["hbya"] = RC.compute_HbyA(t(H), t(A_p)).numpy().copy()
    out["ffh_w"] = RC.compute_face_flux_HbyA(t(HbyA), S, own, nei, ni, w).numpy().copy()
    out["ffh_half"] = RC.compute_face_flux_HbyA(t(HbyA), S, own, nei, ni).numpy().copy()
    out["rc_w"] = RC.rhie_chow_correction(t(p), t(A_p), S, dl, own, nei, ni, V, w).numpy().copy()
    out["rc_half"] = RC.rhie_chow_correction(t(p), t(A_p), S, dl, own, nei, ni, V).numpy().copy()
    out["ff_w"] = RC.compute_face_flux(t(HbyA), t(p), t(A_p), S, dl, own, nei, ni, V,
                                       w).numpy().copy()
    path = os.path.join(HERE, "reference_pressure.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def smoothers(ref_root: str) -> None:
    """SmoothSolver (solvers/smooth_solver.py:37-232) with its three
    smoothers and the standalone smoothers (solvers/smoothers.py:63-260) on
    seeded diagonally dominant 4^3 systems, triangular and permuted face
    order -> reference_smooth.npz."""
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import torch
    from pyfoam.core.ldu_matrix import LduMatrix
    from pyfoam.solvers.smooth_solver import SmoothSolver
    from pyfoam.solvers.smoothers import DICGSmoother, GaussSeidelSmoother, JacobiSmoother

    torch.set_num_threads(8)
    t = torch.from_numpy
    out = {}
    for tag, perm in (("tri", False), ("perm", True)):
        c = random_ldu(4, seed=31, permute_faces=perm)
        m = LduMatrix(c["n"], t(c["owner"]), t(c["neighbour"]))
        m.diag, m.lower, m.upper = t(c["diag"]), t(c["lower"]), t(c["upper"])
        b, x0 = t(c["r"]), t(c["x"])
        for sm in ("GaussSeidel", "DIC", "DILU"):
            s = SmoothSolver(tolerance=0.0, rel_tol=0.0, max_iter=3, smoother=sm, n_sweeps=2,
                             omega=0.9 if sm != "GaussSeidel" else 1.0)
            x, it, res = s(m, b, x0)
            out[f"{tag}_ss_{sm}_x"] = x.numpy().copy()
            out[f"{tag}_ss_{sm}_it"] = np.int64(it)
            out[f"{tag}_ss_{sm}_res"] = np.float64(res)
        out[f"{tag}_gs_x"] = GaussSeidelSmoother(m, omega=0.8).smooth(x0, b, 2).numpy().copy()
        out[f"{tag}_jac_x"] = JacobiSmoother(m).smooth(x0, b, 3).numpy().copy()
        out[f"{tag}_dicg_x"] = DICGSmoother(m, omega=0.9).smooth(x0, b, 2).numpy().copy()
        print(tag, flush=True)
    path = os.path.join(HERE, "reference_smooth.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def pbicg(ref_root: str) -> None:
    """PBiCGSolver (solvers/pbicg.py:40-220) with DILU / DIC / none and
    DiagonalSolver (solvers/diagonal.py:25-85) on a random asymmetric 5^3
    system -> reference_pbicg.npz."""
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import torch
    from pyfoam.core.ldu_matrix import LduMatrix
    from pyfoam.solvers.diagonal import DiagonalSolver
    from pyfoam.solvers.pbicg import PBiCGSolver

    torch.set_num_threads(1)
    t = torch.from_numpy
    out = {}
    c = random_ldu(5, seed=51, permute_faces=False)
    m = LduMatrix(c["n"], t(c["owner"]), t(c["neighbour"]))
    m.diag, m.lower, m.upper = t(c["diag"]), t(c["lower"]), t(c["upper"])
    b, x0 = t(c["r"]), torch.zeros(c["n"], dtype=torch.float64)
    # the reference's shadow update uses the primal direction, so its residual
    # does not converge on this system; parity is over the first iterations
    for pc in ("DILU", "DIC", "none"):
        for k in (1, 3, 6):
            s = PBiCGSolver(tolerance=0.0, rel_tol=0.0, max_iter=k, preconditioner=pc)
            x, it, res = s(m, b, x0)
            out[f"pbicg_{pc}_{k}_x"] = x.numpy().copy()
            out[f"pbicg_{pc}_{k}_it"] = np.int64(it)
            out[f"pbicg_{pc}_{k}_res"] = np.float64(res)
        print(pc, it, res, flush=True)
    d = DiagonalSolver()
    dg = c["diag"].copy()
    dg[3] = -dg[3]
    dg[7] = 0.0
    md = LduMatrix(c["n"], t(c["owner"]), t(c["neighbour"]))
    md.diag = t(dg)
    x, it, res = d(md, b, x0)
    out["diag_d"], out["diag_x"], out["diag_it"], out["diag_res"] = dg, x.numpy().copy(), \
        np.int64(it), np.float64(res)
    path = os.path.join(HERE, "reference_pbicg.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def gamg(ref_root: str) -> None:
    """GAMGSolver (solvers/gamg.py:104-585) on a 6^3 Poisson system and a
    random diagonally dominant 5^3 system with permuted faces: hierarchy
    (aggregation maps, coarse coefficients) and x after a fixed number of
    V-cycles -> reference_gamg.npz."""
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import torch
    from pyfoam.core.ldu_matrix import LduMatrix
    from pyfoam.solvers.gamg import GAMGSolver

    torch.set_num_threads(8)
    t = torch.from_numpy
    out = {}
    cases = {"poi": c1_poisson(6, seed=4), "rnd": random_ldu(5, seed=41, permute_faces=True)}
    cases["rnd"]["b"] = cases["rnd"]["r"]
    for tag, c in cases.items():
        m = LduMatrix(c["n"], t(c["owner"]), t(c["neighbour"]))
        m.diag, m.lower, m.upper = t(c["diag"]), t(c["lower"]), t(c["upper"])
        s = GAMGSolver(tolerance=0.0, rel_tol=0.0, max_iter=4, min_cells_coarse=10)
        x, it, res = s(m, t(c["b"]), torch.zeros(c["n"], dtype=torch.float64))
        out[f"{tag}_x"] = x.numpy().copy()
        out[f"{tag}_it"] = np.int64(it)
        out[f"{tag}_res"] = np.float64(res)
        # the hierarchy, rebuilt with the reference's own static methods
        temp = m
        sizes = [m.n_cells]
        for lvl in range(3):
            if temp.n_cells <= 10:
                break
            agg = GAMGSolver._build_aggregates(temp, max(temp.n_cells // 2, 10))
            if agg.n_coarse >= temp.n_cells:
                break
            cl = GAMGSolver._build_coarse_matrix(temp, agg)
            out[f"{tag}_f2c{lvl}"] = agg.fine_to_coarse.numpy().copy()
            for k in ("diag", "lower", "upper", "owner", "neighbour"):
                out[f"{tag}_L{lvl + 1}_{k}"] = getattr(cl, k).numpy().copy()
            sizes.append(cl.n_cells)
            temp = LduMatrix(cl.n_cells, cl.owner, cl.neighbour)
            temp.diag, temp.lower, temp.upper = cl.diag, cl.lower, cl.upper
        out[f"{tag}_sizes"] = np.array(sizes, np.int64)
        print(tag, it, res, sizes, flush=True)
    path = os.path.join(HERE, "reference_gamg.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def ldu128(ref_root: str) -> None:
    """128^3 hex topology (2,097,152 cells, 6,242,304 faces):
    Ax, Ax_T, FP32 Ax, the DIC and DILU factorised diagonals
    (core/ldu_matrix.py:172-258, solvers/preconditioners.py:88-133,228-272)
    and PBiCGStab+DILU (solvers/pbicgstab.py:103-239) on a seeded random LDU
    system whose coefficients are exact draws of default_rng (bit-identical
    on every machine) -> reference_ldu128.npz.  Bitwise results as SHA-256;
    the solve as its iteration count, residual history and every 97th entry
    of x."""
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import time

    import torch
    from pyfoam.core.ldu_matrix import LduMatrix
    from pyfoam.solvers.pbicgstab import PBiCGSTABSolver
    from pyfoam.solvers.preconditioners import DICPreconditioner, DILUPreconditioner
    from pyfoam.solvers.residual import ResidualMonitor

    torch.set_num_threads(8)
    t = torch.from_numpy
    out = {}
    c = random_ldu(128, seed=5)
    m = LduMatrix(c["n"], t(c["owner"]), t(c["neighbour"]))
    m.diag, m.lower, m.upper = t(c["diag"]), t(c["lower"]), t(c["upper"])
    out["coeff_sha"] = sha(np.concatenate([c["diag"], c["lower"], c["upper"], c["x"], c["r"]]))
    x = t(c["x"])
    out["Ax_sha"] = sha(m.Ax(x).numpy())
    out["AxT_sha"] = sha(m.Ax_T(x).numpy())
    m32 = LduMatrix(c["n"], t(c["owner"]), t(c["neighbour"]), dtype=torch.float32)
    m32.diag, m32.lower, m32.upper = t(c["diag"]), t(c["lower"]), t(c["upper"])
    out["Ax_f32_sha"] = sha(m32.Ax(x.float()).numpy())
    print("Ax done", flush=True)
    t0 = time.time()
    out["dic_sha"] = sha(DICPreconditioner(m)._precond_diag.numpy())
    print("DIC build", time.time() - t0, flush=True)
    t0 = time.time()
    out["dilu_sha"] = sha(DILUPreconditioner(m)._precond_diag.numpy())
    print("DILU build", time.time() - t0, flush=True)
    t0 = time.time()
    mon = ResidualMonitor(tolerance=0.0, rel_tol=1e-10, min_iter=0)
    solver = PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-10, max_iter=200, preconditioner="DILU")
    xs, info = solver._solve(m, t(c["r"]), torch.zeros(c["n"], dtype=torch.float64), mon, 200)
    out["bicg_iterations"] = np.int64(info.iterations)
    out["bicg_history"] = np.array(info.residual_history)
    out["bicg_x97"] = xs.numpy()[::97].copy()
    print("PBiCGStab", info.iterations, info.converged, time.time() - t0, flush=True)
    path = os.path.join(HERE, "reference_ldu128.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


UNROLL_SAMPLES = {24: 1024, 96: 4096}


def unroll(ref_root: str, N: int) -> None:
    """The adjoint workload (per-face LogNormal(0, 1) diffusivity, x0 ~
    U[0, 1], 20 implicit steps of dt = 1e-3, loss ||x_T - x_target||^2) on
    the uniform N^3 mesh -- 24^3 (13,824 cells) or the full 96^3 (884,736
    cells) -- differentiated by the reference itself: fvm.laplacian under
    autograd and DifferentiableLinearSolve per step with
    PCGSolver(tolerance=0, rel_tol=1e-13, preconditioner="none")
    (differentiable/linear_solver.py:99-151).  The full gradient is large, so
    the fixture keeps it on UNROLL_SAMPLES[N] seeded faces, plus its L2 norm,
    its sum, the loss and x_T on seeded cells.  The target comes from the
    oracle (one thread at 24^3; all cores at 96^3, where the reference's
    forward and backward take about 7 minutes on 8 cores)."""
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import torch
    from pyfoam.differentiable.linear_solver import DifferentiableLinearSolve
    from pyfoam.discretisation.operators import fvm
    from pyfoam.solvers.pcg import PCGSolver

    torch.set_num_threads(8)
    t = torch.from_numpy
    uc = unroll_case(N, threads=1 if N <= 24 else len(os.sched_getaffinity(0)))
    mesh = uc["mesh"]
    gam = t(uc["gamma"]).clone().requires_grad_(True)
    solver = PCGSolver(tolerance=0.0, rel_tol=1e-13, max_iter=50000, preconditioner="none")
    own = mesh.owner[: mesh.n_internal_faces]
    lap = fvm.laplacian(gam, torch.zeros(mesh.n_cells, dtype=torch.float64), mesh=mesh)
    d = lap.diag + 1.0 / uc["dt"]
    x = t(uc["x0"])
    for _ in range(uc["steps"]):
        x = DifferentiableLinearSolve.apply(d, lap.lower, lap.upper, x / uc["dt"], solver, own,
                                            mesh.neighbour, x, 0.0, 50000)
    loss = ((x - t(uc["target"])) ** 2).sum()
    loss.backward()
    g = gam.grad.numpy()
    rng = np.random.default_rng(N)
    faces = np.sort(rng.choice(g.shape[0], UNROLL_SAMPLES[N], replace=False))
    cells = np.sort(rng.choice(x.shape[0], 256, replace=False))
    xT = x.detach().numpy()
    out = dict(faces=faces, grad_at_faces=g[faces], grad_norm=np.float64(np.linalg.norm(g)),
               grad_sum=np.float64(g.sum()), loss=np.float64(loss.item()), cells=cells,
               xT_at_cells=xT[cells], xT_norm=np.float64(np.linalg.norm(xT)),
               rel_tol=np.float64(1e-13))
    path = os.path.join(HERE, f"reference_unroll{N}.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes; loss", float(loss))


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("PYFOAM_REFERENCE", "")
    if "--dlap" in sys.argv:
        dlap(root)
    elif "--geometry" in sys.argv:
        geometry(root)
    elif "--pressure" in sys.argv:
        pressure(root)
    elif "--smooth" in sys.argv:
        smoothers(root)
    elif "--gamg" in sys.argv:
        gamg(root)
    elif "--pbicg" in sys.argv:
        pbicg(root)
    elif "--ldu128" in sys.argv:
        ldu128(root)
    elif "--unroll24" in sys.argv:
        unroll(root, 24)
    elif "--unroll96" in sys.argv:
        unroll(root, 96)
    else:
        main(root)
