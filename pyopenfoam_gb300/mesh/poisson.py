"""The Poisson systems of the benchmark configurations, generated directly as
LDU arrays on the unit-cube hex mesh.

``hex_poisson(N, seed)`` is ``fvm.laplacian(1, ...)`` per unit volume on the
uniform N^3 mesh (``src/pyfoam/discretisation/operators.py:432-518``) with a
fixed-value patch at x = 0 and zero gradient elsewhere: off-diagonals
-|S| delta / V = -N^2, diagonal = N^2 per internal face of the cell plus 2 N^2
on the x = 0 boundary face (delta_b = 1 / (h/2)).  Every coefficient is an
exact binary number, so the arrays are identical on every machine; the RHS is
U[-1, 1] from ``numpy.random.default_rng(seed)``.

``convection_diffusion(N, seed, peclet)`` is an asymmetric momentum-type
system on the same topology: log-normal face diffusion plus first-order
upwind convection of a uniform velocity with the direction weights
(1, 0.5, 0.25), fixed value on x = 0 and outflow on the far faces.
"""

from __future__ import annotations

import numpy as np

__all__ = ["hex_faces", "hex_poisson", "convection_diffusion"]


def hex_faces(nx: int, ny: int | None = None, nz: int | None = None):
    """(n_cells, owner, neighbour) of the internal faces of an nx*ny*nz hex
    mesh in upper-triangular cell order (per cell +x, +y, +z)."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n = nx * ny * nz
    c = np.arange(n, dtype=np.int64)
    i, j, k = c % nx, (c // nx) % ny, c // (nx * ny)
    has = np.stack([i < nx - 1, j < ny - 1, k < nz - 1], axis=1)
    flat = np.flatnonzero(has.ravel())
    cell, d = flat // 3, flat % 3
    step = np.array([1, nx, nx * ny], dtype=np.int64)
    return n, cell, cell + step[d]


def hex_poisson(N: int, seed: int = 0, with_rhs: bool = True) -> dict:
    n, own, nei = hex_faces(N)
    F = own.shape[0]
    coeff = float(N) * float(N)
    c = np.arange(n)
    cnt = np.bincount(own, minlength=n) + np.bincount(nei, minlength=n)
    diag = cnt.astype(np.float64) * coeff + np.where(c % N == 0, 2.0 * coeff, 0.0)
    out = dict(n=n, owner=own, neighbour=nei, lower=np.full(F, -coeff),
               upper=np.full(F, -coeff), diag=diag)
    if with_rhs:
        out["b"] = np.random.default_rng(seed).uniform(-1.0, 1.0, n)
    return out


def convection_diffusion(N: int, seed: int = 1, peclet: float = 10.0) -> dict:
    """Upwind convection-diffusion LDU system on the N^3 hex topology.

    Face diffusion D_f ~ LogNormal(0, 1); face flux F_f = peclet * w_f > 0
    from owner to neighbour, w_f = 1, 0.5, 0.25 for x, y, z faces.  Upwind
    rows: upper (owner row, neighbour column) = -D_f, lower (neighbour row,
    owner column) = -D_f - F_f, diagonal = sum of D_f plus the outflow F_f of
    the cell's internal faces; boundary faces add 2 on x = 0 (fixed value)
    and their outflow flux on x, y, z = N - 1 (zero-gradient outflow), so the
    matrix is a column-diagonally dominant M-matrix."""
    n, own, nei = hex_faces(N)
    rng = np.random.default_rng(seed)
    D = rng.lognormal(0.0, 1.0, own.shape[0])
    step = nei - own
    w = np.where(step == 1, 1.0, np.where(step == N, 0.5, 0.25))
    flux = peclet * w
    diag = np.zeros(n)
    np.add.at(diag, own, D + flux)
    np.add.at(diag, nei, D)
    c = np.arange(n)
    i, j, k = c % N, (c // N) % N, c // (N * N)
    diag += (np.where(i == 0, 2.0, 0.0) + np.where(i == N - 1, peclet, 0.0)
             + np.where(j == N - 1, 0.5 * peclet, 0.0) + np.where(k == N - 1, 0.25 * peclet, 0.0))
    return dict(n=n, owner=own, neighbour=nei, lower=-D - flux, upper=-D.copy(), diag=diag,
                b=rng.uniform(-1.0, 1.0, n))
