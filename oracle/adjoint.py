"""The unrolled implicit-diffusion adjoint on the host cores -- TEST
INFRASTRUCTURE ONLY, like the rest of ``oracle/``.

The CPU restatement of the adjoint workload: the oracle's ``fvm.laplacian``
(``discretisation/operators.py:432-518``), ``steps`` implicit steps solved by
the oracle's threaded PCG+DIC, then the reverse sweep that
``DifferentiableLinearSolve.backward`` (``differentiable/linear_solver.py:
99-151``) performs per step -- one solve with the transposed matrix for the
adjoint lam, then the gradient of the face coefficients -- chained through
``fvm.laplacian``'s dependence on the face diffusivity.  ``bench.py``'s
CPU-baseline leg of the adjoint workload times it; the tests pin it against
the reference's own autograd gradient.  The product never imports it.
"""

from __future__ import annotations

import math
import time

import numpy as np

from . import oracle as O


def unrolled_adjoint(h, gamma, x0, target, dt, steps, threads):
    """Loss ||x_steps - target||^2 of ``steps`` implicit diffusion steps
    (A + I/dt) x_{k+1} = x_k / dt on the mesh ``h`` (a HexMesh: owner,
    neighbour, face areas, delta coefficients, cell volumes), and its
    gradient with respect to the per-face diffusivity ``gamma``.

    Forward: all states kept, each step by PCG+DIC to 1e-14 on ``threads``
    threads.  Backward: one transposed solve per step (right-hand side
    scaled by a power of two, so the 1e-30 breakdown test does not stop a
    small adjoint solve) and the face gradient s_f (x_N - x_P)(lam_P/V_P -
    lam_N/V_N) on internal faces, -s_b lam_P x_P / V_P on boundary faces.
    Returns (loss, gradient, forward s, backward s)."""
    own_all, nei = h.numpy("owner"), h.numpy("neighbour")
    S, dl, V = h.numpy("face_areas"), h.numpy("delta_coefficients"), h.numpy("cell_volumes")
    nint = nei.shape[0]
    own = own_all[:nint]
    t0 = time.perf_counter()
    lo, up, dg = O.laplacian(h.n_cells, own_all, nei, S, dl, gamma, V)
    d = dg + 1.0 / dt
    pd = O.dic_build(own, nei, d, up)
    xs = [x0]
    x = x0
    for _ in range(steps):
        x = O.pcg(own, nei, d, lo, up, x / dt, x, pd, 0.0, 1e-14, 50000, threads=threads).x
        xs.append(x)
    t1 = time.perf_counter()
    diff = x - target
    loss = float(diff @ diff)
    g = 2.0 * diff
    sd = np.sqrt((S * S).sum(axis=1)) * dl
    grad = np.zeros(own_all.shape[0])
    pdT = O.dic_build(own, nei, d, lo)
    for t in range(steps, 0, -1):
        k = 30 - math.frexp(float(np.abs(g).max()))[1]
        sc = math.ldexp(1.0, k)
        lam = O.pcg(own, nei, d, up, lo, g * sc, np.zeros_like(g), pdT, 0.0, 1e-14, 50000,
                    threads=threads).x * math.ldexp(1.0, -k)
        xt = xs[t]
        lv = lam / V
        grad[:nint] += sd[:nint] * (xt[nei] - xt[own]) * (lv[own] - lv[nei])
        ob = own_all[nint:]
        grad[nint:] += sd[nint:] * (-lv[ob] * xt[ob])
        g = lam / dt
    t2 = time.perf_counter()
    return loss, grad, t1 - t0, t2 - t1
