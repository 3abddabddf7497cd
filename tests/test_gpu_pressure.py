"""Pressure-corrector steps either side of the pressure solve
(correct_velocity, correct_face_flux, adjust_phi) and the Rhie-Chow
functions, on the GPU, against the reference's own outputs on the jittered
6^3 mesh (tests/golden/reference_pressure.npz, make_golden.py --pressure).
Bitwise, except adjust_phi whose boundary-flux sum is a tree sum
(tolerance 1e-15 relative on phi)."""

import os

import numpy as np
import pytest
import torch

from pyopenfoam_gb300.solvers import rhie_chow as RC
from pyopenfoam_gb300.solvers.pressure_equation import (adjust_phi, correct_face_flux,
                                                        correct_velocity)
from tests.golden.cases import jitter_case, mesh_from_arrays

pytestmark = pytest.mark.gpu
PR = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_pressure.npz"))


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.int64)


def _mesh():
    jc = jitter_case(6)
    m = mesh_from_arrays(jc, device="cuda")
    m.face_weights = torch.as_tensor(PR["weights"]).cuda()
    return m


def t(k):
    return torch.as_tensor(PR[k]).cuda()


def test_correct_velocity_and_face_flux_bitwise():
    m = _mesh()
    U = correct_velocity(t("HbyA"), t("HbyA"), t("p"), t("A_p"), m)
    assert (_bits(U.cpu().numpy()) == _bits(PR["cv"])).all()
    assert float(U[7].norm()) <= 1e4 * (1 + 1e-15)  # the limiter acted on row 7
    U = correct_velocity(t("HbyA"), t("HbyA"), t("p"), t("A_p"), m, alpha=0.7)
    assert (_bits(U.cpu().numpy()) == _bits(PR["cv_a07"])).all()
    phi = correct_face_flux(t("phi"), t("p"), t("A_p"), m, face_weights=t("weights"))
    assert (_bits(phi.cpu().numpy()) == _bits(PR["cff"])).all()


def test_adjust_phi_removes_net_boundary_flux():
    m = _mesh()
    ph = t("phi").clone()
    assert adjust_phi(ph, m) == bool(PR["adj_ret"])
    np.testing.assert_allclose(ph.cpu().numpy(), PR["adj_phi"], rtol=1e-15, atol=1e-15)
    ni = m.n_internal_faces
    assert abs(float(ph[ni:].sum())) < 1e-12
    assert (_bits(ph[:ni].cpu().numpy()) == _bits(PR["phi"][:ni])).all()
    assert adjust_phi(ph, m, closed=False) is False


def test_rhie_chow_functions_bitwise():
    m = _mesh()
    own, nei, ni = m.owner, m.neighbour, m.n_internal_faces
    S, dl, V = m.face_areas, m.delta_coefficients, m.cell_volumes
    w = t("weights")
    checks = {
        "hbya": RC.compute_HbyA(t("H"), t("A_p")),
        "ffh_w": RC.compute_face_flux_HbyA(t("HbyA"), S, own, nei, ni, w),
        "ffh_half": RC.compute_face_flux_HbyA(t("HbyA"), S, own, nei, ni),
        "rc_w": RC.rhie_chow_correction(t("p"), t("A_p"), S, dl, own, nei, ni, V, w),
        "rc_half": RC.rhie_chow_correction(t("p"), t("A_p"), S, dl, own, nei, ni, V),
        "ff_w": RC.compute_face_flux(t("HbyA"), t("p"), t("A_p"), S, dl, own, nei, ni, V, w),
    }
    for k, v in checks.items():
        assert v.device.type == "cuda"
        assert (_bits(v.cpu().numpy()) == _bits(PR[k])).all(), k
