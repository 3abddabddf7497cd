"""Rhie-Chow face fluxes, drop-in for ``pyfoam.solvers.rhie_chow``
(``src/pyfoam/solvers/rhie_chow.py:56-250``):

    HbyA  = H / max(|A_p|, 1e-30)
    phi_f = (w HbyA_P + (1 - w) HbyA_N) . S_f   (HbyA_P . S_f on boundary faces)
          + (1/A_p)_f (p_P - p_N) |S_f| delta_f  (internal faces)

Each function is one libgbfoam kernel (``csrc/pressure.cu``) with the
reference's order of operations, so the results are bitwise its own.  The
arguments are the reference's raw arrays; ``face_weights=None`` means 0.5.
"""

from __future__ import annotations

import torch

from .. import _lib
from ..core.device import resolve_device

__all__ = ["compute_HbyA", "compute_face_flux_HbyA", "rhie_chow_correction",
           "compute_face_flux"]


def _f64(t, dev) -> torch.Tensor:
    return torch.as_tensor(t).detach().to(device=dev, dtype=torch.float64).contiguous()


def _i32(t, dev) -> torch.Tensor:
    return torch.as_tensor(t).detach().to(device=dev, dtype=torch.int32).contiguous()


def compute_HbyA(H: torch.Tensor, A_p: torch.Tensor) -> torch.Tensor:
    dev = resolve_device(H.device)
    Hh, A = _f64(H, dev), _f64(A_p, dev)
    n = A.shape[0]
    if Hh.shape != (n, 3):
        raise ValueError(f"H must have shape ({n}, 3), got {tuple(Hh.shape)}")
    out = torch.empty(n, 3, device=dev, dtype=torch.float64)
    _lib.check(_lib.lib().gbf_hbya_f64(n, Hh.data_ptr(), A.data_ptr(), out.data_ptr(),
                                       _lib.stream_ptr(dev)), "gbf_hbya_f64")
    return out


def inv_abs_clamped(A_p: torch.Tensor) -> torch.Tensor:
    """1 / max(|A_p|, 1e-30) per cell, on the GPU."""
    A = torch.as_tensor(A_p).detach().to(dtype=torch.float64).contiguous()
    dev = resolve_device(A.device)
    A = A.to(dev)
    inv = torch.empty_like(A)
    _lib.check(_lib.lib().gbf_inv_abs_clamped_f64(A.shape[0], A.data_ptr(), inv.data_ptr(),
                                                  _lib.stream_ptr(dev)),
               "gbf_inv_abs_clamped_f64")
    return inv


def _flux(HbyA, face_areas, owner, neighbour, n_internal_faces, face_weights, p=None, A_p=None,
          delta_coefficients=None):
    dev = resolve_device(HbyA.device)
    Hh, S = _f64(HbyA, dev), _f64(face_areas, dev)
    nf = S.shape[0]
    own, nei = _i32(owner, dev), _i32(neighbour, dev)
    ni = int(n_internal_faces)
    if own.shape[0] < nf or nei.shape[0] < ni:
        raise ValueError("owner needs n_faces entries and neighbour n_internal_faces")
    w = None if face_weights is None else _f64(face_weights, dev)
    ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    pp = None if p is None else _f64(p, dev)
    A = None if A_p is None else inv_abs_clamped(_f64(A_p, dev))
    d = None if delta_coefficients is None else _f64(delta_coefficients, dev)
    phi = torch.empty(nf, device=dev, dtype=torch.float64)
    _lib.check(_lib.lib().gbf_face_flux_f64(nf, ni, own.data_ptr(),
                                            nei.data_ptr() if nei.numel() else None,
                                            Hh.data_ptr(), S.data_ptr(), ptr(w), ptr(pp), ptr(A),
                                            ptr(d), phi.data_ptr(), _lib.stream_ptr(dev)),
               "gbf_face_flux_f64")
    return phi


def compute_face_flux_HbyA(HbyA: torch.Tensor, face_areas: torch.Tensor, owner: torch.Tensor,
                           neighbour: torch.Tensor, n_internal_faces: int,
                           face_weights: torch.Tensor | None = None) -> torch.Tensor:
    return _flux(HbyA, face_areas, owner, neighbour, n_internal_faces, face_weights)


def rhie_chow_correction(p: torch.Tensor, A_p: torch.Tensor, face_areas: torch.Tensor,
                         delta_coefficients: torch.Tensor, owner: torch.Tensor,
                         neighbour: torch.Tensor, n_internal_faces: int,
                         cell_volumes: torch.Tensor,
                         face_weights: torch.Tensor | None = None) -> torch.Tensor:
    dev = resolve_device(p.device)
    S = _f64(face_areas, dev)
    nf, ni = S.shape[0], int(n_internal_faces)
    own, nei = _i32(owner, dev), _i32(neighbour, dev)
    pp, A, d = _f64(p, dev), inv_abs_clamped(_f64(A_p, dev)), _f64(delta_coefficients, dev)
    w = None if face_weights is None else _f64(face_weights, dev)
    out = torch.empty(nf, device=dev, dtype=torch.float64)
    _lib.check(_lib.lib().gbf_rhie_chow_f64(nf, ni, own.data_ptr(),
                                            nei.data_ptr() if nei.numel() else None,
                                            pp.data_ptr(), A.data_ptr(), S.data_ptr(),
                                            d.data_ptr(), None if w is None else w.data_ptr(),
                                            None, out.data_ptr(), _lib.stream_ptr(dev)),
               "gbf_rhie_chow_f64")
    return out


def compute_face_flux(HbyA: torch.Tensor, p: torch.Tensor, A_p: torch.Tensor,
                      face_areas: torch.Tensor, delta_coefficients: torch.Tensor,
                      owner: torch.Tensor, neighbour: torch.Tensor, n_internal_faces: int,
                      cell_volumes: torch.Tensor,
                      face_weights: torch.Tensor | None = None) -> torch.Tensor:
    return _flux(HbyA, face_areas, owner, neighbour, n_internal_faces, face_weights, p, A_p,
                 delta_coefficients)
