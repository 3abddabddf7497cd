"""The Poisson systems of the benchmark configurations, generated directly as
LDU arrays on the unit-cube hex mesh.

``hex_poisson(N, seed)`` is ``fvm.laplacian(1, ...)`` per unit volume on the
uniform N^3 mesh (``src/pyfoam/discretisation/operators.py:432-518``) with a
fixed-value patch at x = 0 and zero gradient elsewhere: off-diagonals
-|S| delta / V = -N^2, diagonal = N^2 per internal face of the cell plus 2 N^2
on the x = 0 boundary face (delta_b = 1 / (h/2)).  Every coefficient is an
exact binary number, so the arrays are identical on every machine; the RHS is
U[-1, 1] from ``numpy.random.default_rng(seed)``.
"""

from __future__ import annotations

import numpy as np

__all__ = ["hex_faces", "hex_poisson"]


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
