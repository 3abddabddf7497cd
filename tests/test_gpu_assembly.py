"""fvm.laplacian / fvm.div assembly and the full DIC/DILU sweeps on the GPU:
bitwise against the reference's golden outputs and the oracle."""

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyopenfoam_gb300 import DICPreconditioner, DILUPreconditioner, LduMatrix
from pyopenfoam_gb300.discretisation import fvm
from pyopenfoam_gb300.mesh import HexMesh
from tests.golden.cases import FIXTURE, jitter_case, mesh_from_arrays, random_ldu, sha

pytestmark = pytest.mark.gpu
G = np.load(FIXTURE)


def gpu_mesh():
    jc = jitter_case(6)
    return jc, mesh_from_arrays(jc, device="cuda")


def bits(a):
    return np.asarray(a).view(np.int64)


@pytest.mark.parametrize("kind", ["face", "cell", "scalar"])
def test_laplacian_bitwise_against_reference(kind):
    jc, mesh = gpu_mesh()
    D = {"face": torch.as_tensor(jc["gamma"]), "cell": torch.as_tensor(G["j6_dcell"]),
         "scalar": 1.5}[kind]
    key = {"face": "lap", "cell": "lapc", "scalar": "laps"}[kind]
    A = fvm.laplacian(D, torch.zeros(1), mesh=mesh)
    assert A.device.type == "cuda" and A.n_internal_faces == int(jc["n_internal"])
    for part in ("lower", "upper", "diag"):
        np.testing.assert_array_equal(getattr(A, part).cpu().numpy(), G[f"j6_{key}_{part}"])


def test_div_upwind_bitwise_against_reference():
    jc, mesh = gpu_mesh()
    A = fvm.div(torch.as_tensor(jc["phi"]), torch.zeros(1), "Gauss upwind", mesh=mesh)
    for part in ("lower", "upper", "diag"):
        np.testing.assert_array_equal(getattr(A, part).cpu().numpy(), G[f"j6_div_{part}"])
    with pytest.raises(ValueError, match="upwind"):
        fvm.div(torch.as_tensor(jc["phi"]), torch.zeros(1), "Gauss linear", mesh=mesh)


def test_laplacian_jittered_16_against_oracle():
    m = HexMesh(16, jitter=0.2, seed=3)
    gamma = np.random.default_rng(3).lognormal(0.0, 1.0, m.n_faces)
    A = fvm.laplacian(torch.as_tensor(gamma), torch.zeros(1), mesh=m.to("cuda"))
    lo, up, dg = O.laplacian(m.n_cells, m.numpy("owner"), m.numpy("neighbour"),
                             m.numpy("face_areas"), m.numpy("delta_coefficients"), gamma,
                             m.numpy("cell_volumes"))
    for got, ref in ((A.lower, lo), (A.upper, up), (A.diag, dg)):
        assert (bits(got.cpu().numpy()) == bits(ref)).all()


def test_laplacian_gamma_gradient_matches_autograd_of_formula():
    """dL/dgamma from the backward kernel equals torch autograd through the
    reference formula (operators.py:488-517) written with torch ops."""
    jc, mesh = gpu_mesh()
    g = torch.as_tensor(jc["gamma"]).cuda().requires_grad_(True)
    A = fvm.laplacian(g, torch.zeros(1), mesh=mesh)
    rng = np.random.default_rng(9)
    wl, wu, wd = (torch.as_tensor(rng.uniform(-1, 1, k)).cuda() for k in
                  (A.n_internal_faces, A.n_internal_faces, A.n_cells))
    (A.lower * wl).sum().add((A.upper * wu).sum()).add((A.diag * wd).sum()).backward()
    ours = g.grad.clone()

    g2 = torch.as_tensor(jc["gamma"]).cuda().requires_grad_(True)
    nint = int(jc["n_internal"])
    own = mesh.owner
    S = mesh.face_areas.norm(dim=1)
    c = g2 * S * mesh.delta_coefficients
    V = mesh.cell_volumes
    lower = -c[:nint] / V[own[:nint]]
    upper = -c[:nint] / V[mesh.neighbour]
    diag = torch.zeros(A.n_cells, dtype=torch.float64, device="cuda")
    diag = diag.index_add(0, own[:nint], c[:nint] / V[own[:nint]])
    diag = diag.index_add(0, mesh.neighbour, c[:nint] / V[mesh.neighbour])
    diag = diag.index_add(0, own[nint:], c[nint:] / V[own[nint:]])
    (lower * wl).sum().add((upper * wu).sum()).add((diag * wd).sum()).backward()
    ref = g2.grad
    assert torch.allclose(ours, ref, rtol=1e-12, atol=1e-12 * ref.abs().max().item())


@pytest.mark.parametrize("name,N,perm", [("ldu12p", 12, True)])
def test_apply_full_bitwise_against_reference(name, N, perm):
    c = random_ldu(N, 5, perm)
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(c[k]) for k in ("diag", "lower", "upper"))
    r = torch.as_tensor(c["r"])
    assert sha(DICPreconditioner(m).apply_full(r).cpu().numpy()) == str(G[f"{name}_dic_full_sha"])
    assert sha(DILUPreconditioner(m).apply_full(r).cpu().numpy()) == str(
        G[f"{name}_dilu_full_sha"])


@pytest.mark.parametrize("perm", [False, True])
def test_apply_full_against_oracle_at_32(perm):
    c = random_ldu(32, 8, perm)
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(c[k]) for k in ("diag", "lower", "upper"))
    r = torch.as_tensor(c["r"])
    dic = DICPreconditioner(m)
    dilu = DILUPreconditioner(m)
    zd = O.dic_apply_full(c["owner"], c["neighbour"], c["upper"],
                          dic.precond_diag.cpu().numpy(), c["r"])
    zl = O.dilu_apply_full(c["owner"], c["neighbour"], c["lower"], c["upper"],
                           dilu.precond_diag.cpu().numpy(), c["r"])
    assert (bits(dic.apply_full(r).cpu().numpy()) == bits(zd)).all()
    assert (bits(dilu.apply_full(r).cpu().numpy()) == bits(zl)).all()
