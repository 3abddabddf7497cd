"""Gradients through unrolled implicit time steps with checkpointing.

    A(gamma) x_{t+1} = x_t / dt,   A = I/dt + fvm.laplacian(gamma)   (t < T)
    L = || x_T - x_target ||^2

The gradient with respect to every face diffusivity gamma_f comes from the
discrete adjoint: g_T = 2 (x_T - x_target); for t = T .. 1 solve
A^T lam_t = g_t, accumulate dL/dgamma -= lam_t^T (dA/dgamma) x_t with the
fused face kernel ``gbf_adjoint_face_grad_f64``, and pass g_{t-1} = lam_t/dt.
Only every ``checkpoint_every``-th state is kept during the forward sweep;
the backward sweep recomputes each segment from its checkpoint, so memory
holds (T / k) + k states instead of T.

No reference counterpart as a whole: the reference differentiates one solve
at a time (``DifferentiableLinearSolve``) and through ``fvm.laplacian`` by
autograd; chaining those over T steps stores every state.
``UnrolledDiffusion`` is the autograd entry point; ``loss_and_grad`` the
explicit one used by the benchmark.
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import torch

from .. import _lib
from ..core.ldu_matrix import LduMatrix
from ..discretisation.operators import fvm, mesh_data
from ..solvers.pcg import PCGSolver

__all__ = ["UnrolledImplicitDiffusion", "UnrolledDiffusion", "GradStats"]


@dataclass
class GradStats:
    forward_s: float = 0.0
    backward_s: float = 0.0
    forward_solves: int = 0
    backward_solves: int = 0
    recompute_solves: int = 0
    iterations: list = field(default_factory=list)
    peak_bytes: int = 0


class UnrolledImplicitDiffusion:
    """Implicit diffusion steps on ``mesh`` with per-face diffusivity.

    Parameters
    ----------
    mesh : duck-typed FvMesh on a CUDA device
    dt, steps : time step and number of implicit steps
    checkpoint_every : states kept every k steps (k = steps keeps only x_0)
    solver : linear solver for forward and adjoint systems (default FP64
        PCG+DIC to a 1e-14 relative residual)
    """

    def __init__(self, mesh, dt: float = 1e-3, steps: int = 20, checkpoint_every: int = 5,
                 solver=None) -> None:
        if steps < 1 or checkpoint_every < 1:
            raise ValueError("steps and checkpoint_every must be >= 1")
        self.mesh = mesh
        self.md = mesh_data(mesh)
        self.dt = float(dt)
        self.steps = int(steps)
        self.k = int(checkpoint_every)
        self.solver = solver or PCGSolver(tolerance=0.0, rel_tol=1e-14, max_iter=50000,
                                          preconditioner="DIC")
        self.stats = GradStats()

    # ------------------------------------------------------------------
    def system(self, gamma: torch.Tensor) -> LduMatrix:
        """A = I/dt + Laplacian(gamma) (no autograd)."""
        with torch.no_grad():
            lap = fvm.laplacian(gamma.detach(), torch.zeros(1), mesh=self.mesh)
        A = LduMatrix(self.md.n_cells, lap.owner, lap.neighbour, device=lap.device)
        A._topology = lap.topology()
        A.diag = lap.diag + 1.0 / self.dt
        A.lower = lap.lower
        A.upper = lap.upper
        return A

    @staticmethod
    def transpose(A: LduMatrix) -> LduMatrix:
        At = LduMatrix(A.n_cells, A.owner, A.neighbour, device=A.device)
        At._topology = A.topology()
        At.diag, At.lower, At.upper = A.diag, A.upper, A.lower
        return At

    def _solve_normalised(self, A: LduMatrix, b: torch.Tensor, x0: torch.Tensor):
        """Solve A x = b with b and x0 scaled by the power of two that brings
        max|b| into [2^29, 2^30), and the solution scaled back.  Power-of-two
        scaling is exact, so the iterates are those of the unscaled solve
        multiplied by 2^k -- except that the solver's absolute thresholds
        (the 1e-30 breakdown test on p.Ap) no longer stop a solve whose
        right-hand side is tiny (adjoint and difference systems) before it
        reaches its relative tolerance."""
        m = float(b.abs().max()) if b.numel() else 0.0
        if m == 0.0 or not math.isfinite(m):
            return self.solver(A, b, x0)
        k = 30 - math.frexp(m)[1]
        s, inv = math.ldexp(1.0, k), math.ldexp(1.0, -k)
        x, it, res = self.solver(A, b * s, x0 * s)
        return x * inv, it, res * inv

    def _step(self, A: LduMatrix, x: torch.Tensor) -> torch.Tensor:
        # warm start from the previous state
        xn, it, _ = self.solver(A, x / self.dt, x)
        self.stats.iterations.append(it)
        return xn

    def forward_states(self, A: LduMatrix, x0: torch.Tensor):
        """x_T and the checkpoints {t: x_t} (t multiple of k, t < T)."""
        ckpt = {0: x0}
        x = x0
        for t in range(1, self.steps + 1):
            x = self._step(A, x)
            self.stats.forward_solves += 1
            if t % self.k == 0 and t < self.steps:
                ckpt[t] = x
        return x, ckpt

    def backward_grad(self, A: LduMatrix, ckpt: dict, xT: torch.Tensor, gT: torch.Tensor):
        """(dL/dgamma over all faces, dL/dx_0) for dL/dx_T = gT."""
        md = self.md
        At = self.transpose(A)
        topo = A.topology()
        dev = md.device
        grad = torch.zeros(max(md.n_faces, 1), device=dev, dtype=torch.float64)
        areas = md.field("face_areas")
        delta = md.field("delta_coefficients")
        vols = md.field("cell_volumes")
        g = gT
        starts = sorted(ckpt)
        L = _lib.lib()
        for s in reversed(starts):
            e = min(s + self.k, self.steps)
            # recompute x_{s+1} .. x_{e-1}; x_e is the next checkpoint or x_T
            seg = {s: ckpt[s]}
            x = ckpt[s]
            for t in range(s + 1, e):
                x = self._step(A, x)
                self.stats.recompute_solves += 1
                seg[t] = x
            seg[e] = xT if e == self.steps else ckpt[e]
            for t in range(e, s, -1):
                lam, it, _ = self._solve_normalised(At, g, torch.zeros_like(g))
                self.stats.iterations.append(it)
                self.stats.backward_solves += 1
                xt = seg[t].contiguous()
                lam = lam.contiguous()
                _lib.check(L.gbf_adjoint_face_grad_f64(
                    topo.layout_ref, md.n_faces, md.owner_all32.data_ptr(), areas.data_ptr(),
                    delta.data_ptr(), vols.data_ptr(), lam.data_ptr(), xt.data_ptr(), 1.0, 1,
                    grad.data_ptr(), _lib.stream_ptr(dev)), "gbf_adjoint_face_grad_f64")
                g = lam / self.dt
                del seg[t]
        return grad[: md.n_faces], g

    # ------------------------------------------------------------------
    def loss_and_grad(self, gamma: torch.Tensor, x0: torch.Tensor, target: torch.Tensor):
        """Loss ||x_T - target||^2 and its gradient over all face
        diffusivities, with timing and memory statistics in ``self.stats``."""
        self.stats = GradStats()
        dev = self.md.device
        torch.cuda.synchronize(dev)
        torch.cuda.reset_peak_memory_stats(dev)
        base = torch.cuda.memory_allocated(dev)
        t0 = time.perf_counter()
        A = self.system(gamma)
        xT, ckpt = self.forward_states(A, x0.to(dev, torch.float64))
        torch.cuda.synchronize(dev)
        t1 = time.perf_counter()
        diff = xT - target
        loss = float(torch.dot(diff, diff))
        grad, _ = self.backward_grad(A, ckpt, xT, 2.0 * diff)
        torch.cuda.synchronize(dev)
        t2 = time.perf_counter()
        self.stats.forward_s = t1 - t0
        self.stats.backward_s = t2 - t1
        self.stats.peak_bytes = torch.cuda.max_memory_allocated(dev) - base
        return loss, grad

    def central_difference(self, gamma: torch.Tensor, x0: torch.Tensor, target: torch.Tensor,
                           face: int, h: float = 1e-6) -> float:
        """(L(gamma + h e_f) - L(gamma - h e_f)) / (2h), evaluated without
        cancellation.

        The assembled matrix is linear in gamma, A(gamma +- h e_f) =
        A(gamma) +- h E with E = fvm.laplacian(e_f), so the perturbed
        matrices are formed from A(gamma) and E instead of by re-assembly.
        (Re-assembling would round the perturbed diagonals, |diag| ~ 1/dt +
        sum c >> h c_f, and that rounding -- which breaks the zero row sum
        of the perturbation -- enters the quotient divided by h; since the
        gradient results from a near-cancellation between the diagonal and
        off-diagonal parts of dA/dgamma, it would dominate the check.)

        The difference d_t = x+_t - x-_t of the two trajectories obeys
            A+ d_{t+1} = d_t / dt - 2h E x-_{t+1},   d_0 = 0,
        so d is solved for directly, accurate to the solver tolerance
        relative to |d| rather than |x|, and L+ - L- = sum d (x+ + x- -
        2 target).  The difference systems are solved with power-of-two
        normalisation (``_solve_normalised``): their right-hand sides are
        small and local, and the solver's absolute breakdown threshold
        would otherwise end the solves early."""
        e = torch.zeros_like(gamma)
        e[face] = 1.0
        A0 = self.system(gamma)
        with torch.no_grad():
            E = fvm.laplacian(e, torch.zeros(1), mesh=self.mesh)

        def shifted(sign: float) -> LduMatrix:
            M = LduMatrix(A0.n_cells, A0.owner, A0.neighbour, device=A0.device)
            M._topology = A0.topology()
            M.diag = A0.diag + (sign * h) * E.diag
            M.lower = A0.lower + (sign * h) * E.lower
            M.upper = A0.upper + (sign * h) * E.upper
            return M

        Ap, Am = shifted(1.0), shifted(-1.0)
        dA = LduMatrix(A0.n_cells, A0.owner, A0.neighbour, device=A0.device)
        dA._topology = A0.topology()
        dA.diag, dA.lower, dA.upper = (2.0 * h) * E.diag, (2.0 * h) * E.lower, (2.0 * h) * E.upper
        xm = x0.to(self.md.device, torch.float64)
        d = torch.zeros_like(xm)
        for _ in range(self.steps):
            xm_next, _, _ = self.solver(Am, xm / self.dt, xm)
            rhs = d / self.dt - dA.Ax(xm_next)
            d, _, _ = self._solve_normalised(Ap, rhs, d)
            xm = xm_next
        xp = xm + d
        return float(torch.dot(d, xp + xm - 2.0 * target)) / (2.0 * h)

    def final_state(self, gamma: torch.Tensor, x0: torch.Tensor) -> torch.Tensor:
        A = self.system(gamma)
        x = x0.to(self.md.device, torch.float64)
        for _ in range(self.steps):
            x = self._step(A, x)
        return x


class UnrolledDiffusion(torch.autograd.Function):
    """``x_T = UnrolledDiffusion.apply(gamma, x0, model)``: differentiable with
    respect to the per-face diffusivity ``gamma`` and the initial state."""

    @staticmethod
    def forward(ctx, gamma, x0, model: UnrolledImplicitDiffusion):
        A = model.system(gamma)
        xT, ckpt = model.forward_states(A, x0.detach().to(model.md.device, torch.float64))
        ctx.model, ctx.A, ctx.ckpt = model, A, ckpt
        ctx.save_for_backward(xT)
        return xT

    @staticmethod
    def backward(ctx, g):
        (xT,) = ctx.saved_tensors
        grad_gamma, grad_x0 = ctx.model.backward_grad(ctx.A, ctx.ckpt, xT, g.contiguous())
        return grad_gamma, grad_x0, None
