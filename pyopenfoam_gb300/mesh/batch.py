"""The batch of independent Poisson systems of the batching configuration:
S uniform unit-cube hex meshes with sides drawn from U{lo..hi}, per-face
diffusivity LogNormal(0, sigma), fixed value on x = 0, RHS U[-1, 1]; the
coefficients are assembled on the GPU by fvm.laplacian."""

from __future__ import annotations

import numpy as np
import torch

__all__ = ["poisson_batch"]


def poisson_batch(n_systems: int = 64, lo: int = 16, hi: int = 96, sigma: float = 0.5,
                  seed: int = 3, device="cuda"):
    """(matrices, sources, sides) for a seeded batch of Poisson systems."""
    from ..discretisation import fvm
    from .hex_mesh import HexMesh

    rng = np.random.default_rng(seed)
    sides = rng.integers(lo, hi + 1, size=n_systems)
    mats, rhs = [], []
    cache = {}
    for N in sides:
        N = int(N)
        mesh = cache.get(N)
        if mesh is None:
            mesh = HexMesh(N, device=device)
            cache[N] = mesh
        gamma = torch.as_tensor(rng.lognormal(0.0, sigma, mesh.n_faces))
        mats.append(fvm.laplacian(gamma, torch.zeros(1), mesh=mesh))
        rhs.append(torch.as_tensor(rng.uniform(-1.0, 1.0, mesh.n_cells)).to(device))
    return mats, rhs, [int(s) for s in sides]
