"""Differentiation: DifferentiableLinearSolve against the reference's golden
gradients and finite differences; the checkpointed unrolled implicit
diffusion against the reference's autograd chain (fvm.laplacian +
DifferentiableLinearSolve over 20 steps) and central differences."""

import numpy as np
import pytest
import torch

from pyopenfoam_gb300 import PCGSolver
from pyopenfoam_gb300.differentiable import DifferentiableLinearSolve
from pyopenfoam_gb300.differentiable.unrolled import UnrolledDiffusion, UnrolledImplicitDiffusion
from tests.golden.cases import FIXTURE, jitter_case, mesh_from_arrays, unroll_case

pytestmark = pytest.mark.gpu
G = np.load(FIXTURE)
f64 = torch.float64


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_dls_gradients_against_reference_golden():
    jc = jitter_case(6)
    nint = int(jc["n_internal"])
    own = torch.as_tensor(jc["owner"][:nint]).cuda()
    nei = torch.as_tensor(jc["neighbour"]).cuda()
    diag = torch.as_tensor(G["j6_lap_diag"] + 10.0).cuda().requires_grad_(True)
    lower = torch.as_tensor(G["j6_lap_lower"]).cuda().requires_grad_(True)
    upper = torch.as_tensor(G["j6_lap_upper"]).cuda().requires_grad_(True)
    b = torch.as_tensor(jc["b"]).cuda().requires_grad_(True)
    sol = PCGSolver(tolerance=0.0, rel_tol=1e-14, max_iter=2000, preconditioner="none")
    x = DifferentiableLinearSolve.apply(diag, lower, upper, b, sol, own, nei,
                                        torch.zeros(diag.shape[0], dtype=f64, device="cuda"),
                                        0.0, 2000)
    w = torch.as_tensor(jc["w"]).cuda()
    ((w * x).sum() + (x * x).sum()).backward()
    assert rel(x.detach().cpu().numpy(), G["dls_x"]) < 1e-12
    for t, key in ((b, "dls_grad_b"), (diag, "dls_grad_diag"), (lower, "dls_grad_lower"),
                   (upper, "dls_grad_upper")):
        assert rel(t.grad.cpu().numpy(), G[key]) < 1e-10, key


def test_dls_reference_unit_case_finite_differences():
    # tests/unit/differentiable/test_linear_solver.py:122-156, tighter bound
    own = torch.tensor([0, 1], device="cuda")
    nei = torch.tensor([1, 2], device="cuda")
    diag = torch.tensor([4.0, 6.0, 4.0], dtype=f64, device="cuda").requires_grad_(True)
    lower = torch.tensor([-1.0, -1.0], dtype=f64, device="cuda").requires_grad_(True)
    upper = torch.tensor([-1.5, -1.0], dtype=f64, device="cuda").requires_grad_(True)
    b = torch.tensor([1.0, 2.0, 3.0], dtype=f64, device="cuda").requires_grad_(True)
    sol = PCGSolver(tolerance=1e-14, rel_tol=0.0, max_iter=1000, preconditioner="none")
    x0 = torch.zeros(3, dtype=f64, device="cuda")
    x = DifferentiableLinearSolve.apply(diag, lower, upper, b, sol, own, nei, x0, 1e-14, 1000)
    x.sum().backward()
    eps = 1e-6
    for i in range(3):
        bp, bm = b.detach().clone(), b.detach().clone()
        bp[i] += eps
        bm[i] -= eps
        fp = DifferentiableLinearSolve.apply(diag.detach(), lower.detach(), upper.detach(), bp,
                                             sol, own, nei, x0, 1e-14, 1000).sum()
        fm = DifferentiableLinearSolve.apply(diag.detach(), lower.detach(), upper.detach(), bm,
                                             sol, own, nei, x0, 1e-14, 1000).sum()
        assert abs(float((fp - fm) / (2 * eps)) - float(b.grad[i])) < 1e-7


def _model(uc, k):
    mesh = mesh_from_arrays(uc, device="cuda")
    sol = PCGSolver(tolerance=0.0, rel_tol=1e-14, max_iter=5000, preconditioner="none")
    return UnrolledImplicitDiffusion(mesh, dt=uc["dt"], steps=uc["steps"], checkpoint_every=k,
                                     solver=sol)


def test_unrolled_gradient_against_reference_autograd():
    uc = unroll_case(10)
    model = _model(uc, 5)
    gamma = torch.as_tensor(uc["gamma"]).cuda()
    x0 = torch.as_tensor(uc["x0"]).cuda()
    target = torch.as_tensor(G["unroll_target"]).cuda()
    loss, grad = model.loss_and_grad(gamma, x0, target)
    assert abs(loss - float(G["unroll_loss"])) <= 1e-11 * float(G["unroll_loss"])
    assert rel(grad.cpu().numpy(), G["unroll_grad"]) < 1e-8
    # the same through autograd
    g = gamma.clone().requires_grad_(True)
    xT = UnrolledDiffusion.apply(g, x0, model)
    ((xT - target) ** 2).sum().backward()
    assert rel(g.grad.cpu().numpy(), G["unroll_grad"]) < 1e-8
    assert rel(xT.detach().cpu().numpy(), G["unroll_xT"]) < 1e-12


def test_unrolled_gradient_against_reference_autograd_24cube():
    """24^3 (13,824 cells, 20 steps): the gradient on 1024 seeded faces, its
    norm and sum, the loss and x_T against the reference's own autograd chain
    (reference_unroll24.npz, made by make_golden.py --unroll24 with the
    reference's PCG to 1e-13, no preconditioner).  Both sides solve every
    step to 1e-13..1e-14; measured on GB300: 3.1e-13 on the sampled faces,
    2.9e-14 on the norm, 2.2e-14 on the loss."""
    import os

    R = np.load(os.path.join(os.path.dirname(FIXTURE), "reference_unroll24.npz"))
    uc = unroll_case(24)
    model = _model(uc, 5)
    gamma = torch.as_tensor(uc["gamma"]).cuda()
    x0 = torch.as_tensor(uc["x0"]).cuda()
    target = torch.as_tensor(uc["target"]).cuda()
    loss, grad = model.loss_and_grad(gamma, x0, target)
    g = grad.cpu().numpy()
    assert abs(loss - float(R["loss"])) <= 1e-12 * float(R["loss"])
    assert rel(g[R["faces"]], R["grad_at_faces"]) < 1e-11
    assert abs(np.linalg.norm(g) - float(R["grad_norm"])) <= 1e-12 * float(R["grad_norm"])
    assert abs(g.sum() - float(R["grad_sum"])) <= 1e-9 * np.abs(g).sum()
    xT = model.final_state(gamma, x0).cpu().numpy()
    assert rel(xT[R["cells"]], R["xT_at_cells"]) < 1e-10


def test_unrolled_gradient_against_reference_autograd_96cube():
    """The full-size adjoint workload (96^3, 884,736 cells, 2,681,856 faces,
    20 steps) against the reference's own autograd chain at that size
    (reference_unroll96.npz, made by make_golden.py --unroll96: the
    reference's fvm.laplacian under autograd and DifferentiableLinearSolve
    per step, PCG to 1e-13 without preconditioner): the gradient on 4096
    seeded faces, its norm and sum, the loss and x_T.  Here the target
    x_T(gamma') comes from the GPU solver, there from the oracle; both solve
    every step to 1e-13..1e-14.  Measured on GB300: loss 4.1e-13, faces
    2.8e-12, norm 2.3e-12, sum 1.6e-11, x_T 7.7e-13; the bars are those
    values times 4 to 7 (the GPU path is deterministic)."""
    import os

    R = np.load(os.path.join(os.path.dirname(FIXTURE), "reference_unroll96.npz"))
    uc = unroll_case(96, with_target=False)
    model = _model(uc, 5)
    gamma, gamma2, x0 = (torch.as_tensor(uc[k]).cuda() for k in ("gamma", "gamma2", "x0"))
    target = model.final_state(gamma2, x0)
    loss, grad = model.loss_and_grad(gamma, x0, target)
    g = grad.cpu().numpy()
    xT = model.final_state(gamma, x0).cpu().numpy()
    errs = {"loss": abs(loss - float(R["loss"])) / float(R["loss"]),
            "faces": rel(g[R["faces"]], R["grad_at_faces"]),
            "norm": abs(np.linalg.norm(g) - float(R["grad_norm"])) / float(R["grad_norm"]),
            "sum": abs(g.sum() - float(R["grad_sum"])) / np.abs(g).sum(),
            "xT": rel(xT[R["cells"]], R["xT_at_cells"])}
    print("96^3 against the reference:", errs)
    assert errs["loss"] <= 2e-12, errs
    assert errs["faces"] < 2e-11, errs
    assert errs["norm"] <= 1e-11, errs
    assert errs["sum"] <= 1e-10, errs
    assert errs["xT"] < 5e-12, errs


def test_checkpoint_interval_does_not_change_the_gradient():
    uc = unroll_case(10)
    gamma = torch.as_tensor(uc["gamma"]).cuda()
    x0 = torch.as_tensor(uc["x0"]).cuda()
    target = torch.as_tensor(G["unroll_target"]).cuda()
    grads = []
    for k in (1, 5, 20):
        m = _model(uc, k)
        _, gr = m.loss_and_grad(gamma, x0, target)
        grads.append(gr.cpu().numpy())
        # each segment [s, s+k) recomputes its k-1 inner states
        n_seg = -(-uc["steps"] // k)
        assert m.stats.recompute_solves == uc["steps"] - n_seg
        assert m.stats.forward_solves == uc["steps"] == m.stats.backward_solves
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[1], grads[2])


def test_unrolled_gradient_central_differences():
    """Adjoint gradient against central differences (h = 1e-6) on random
    faces, to 1e-6 relative; the difference quotient is evaluated without
    cancellation (UnrolledImplicitDiffusion.central_difference)."""
    uc = unroll_case(10)
    model = _model(uc, 5)
    gamma = torch.as_tensor(uc["gamma"]).cuda()
    x0 = torch.as_tensor(uc["x0"]).cuda()
    target = torch.as_tensor(G["unroll_target"]).cuda()
    _, grad = model.loss_and_grad(gamma, x0, target)
    rng = np.random.default_rng(0)
    for f in rng.choice(gamma.shape[0], 8, replace=False):
        fd = model.central_difference(gamma, x0, target, int(f), 1e-6)
        g = float(grad[f])
        assert abs(fd - g) <= 1e-6 * abs(g) + 1e-15, (int(f), fd, g)
