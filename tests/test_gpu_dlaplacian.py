"""DifferentiableLaplacian on the GPU (differentiable/operators.py:409-643):
forward, phi-gradient and D-gradient against the reference's golden outputs
(jittered 6^3 mesh and the reference's own 2-cell unit-test mesh) bit for
bit, against the oracle at a larger size, and the reference's unit-test
properties (constant field -> 0, linear in D, gradcheck)."""

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyopenfoam_gb300.differentiable import DifferentiableLaplacian
from pyopenfoam_gb300.mesh import HexMesh
from tests.golden.cases import DLAP_CASES, dlap_case, mesh_from_arrays

pytestmark = pytest.mark.gpu
f64 = torch.float64


def bits(a):
    return np.asarray(a).view(np.int64)


def _mesh(d):
    return mesh_from_arrays(d, device="cuda")


def _run(mesh, phi, D, g):
    ph = torch.as_tensor(phi, dtype=f64, device="cuda").clone().requires_grad_(True)
    Dt = torch.as_tensor(D, dtype=f64, device="cuda").clone().requires_grad_(True)
    lap = DifferentiableLaplacian.apply(ph, Dt, mesh)
    (lap * torch.as_tensor(g, dtype=f64, device="cuda")).sum().backward()
    return lap.detach().cpu().numpy(), ph.grad.cpu().numpy(), Dt.grad.cpu().numpy()


@pytest.mark.parametrize("tag", DLAP_CASES)
def test_against_reference_golden(tag):
    d = dlap_case(tag)
    e = d["expect"]
    D = d["D"]
    if d["kind"] == "scalar":
        D = torch.tensor(D, dtype=f64, device="cuda", requires_grad=True)
    ph = torch.as_tensor(d["phi"], dtype=f64, device="cuda").clone().requires_grad_(True)
    Dt = (torch.as_tensor(D, dtype=f64, device="cuda").clone().requires_grad_(True)
          if isinstance(D, np.ndarray) else D)
    lap = DifferentiableLaplacian.apply(ph, Dt, _mesh(d))
    assert lap.device.type == "cuda" and lap.dtype == f64
    (lap * torch.as_tensor(d["g"], dtype=f64, device="cuda")).sum().backward()
    assert (bits(lap.detach().cpu().numpy()) == bits(e["lap"])).all()
    assert (bits(ph.grad.cpu().numpy()) == bits(e["grad_phi"])).all()
    if "grad_D" in e:
        gD = Dt.grad.cpu().numpy()
        assert gD.shape == e["grad_D"].shape
        if d["kind"] == "scalar":
            # the reference sums the face gradients with torch's own order
            np.testing.assert_allclose(gD, e["grad_D"], rtol=1e-13, atol=0)
        else:
            assert (bits(gD) == bits(e["grad_D"])).all()
    else:
        assert not isinstance(Dt, torch.Tensor)


def test_against_oracle_on_a_jittered_mesh():
    m = HexMesh(24, jitter=0.2, seed=3)
    rng = np.random.default_rng(4)
    own, nei = m.numpy("owner"), m.numpy("neighbour")
    args = (m.numpy("face_areas"), m.numpy("delta_coefficients"))
    V = m.numpy("cell_volumes")
    phi = rng.uniform(-1, 1, m.n_cells)
    g = rng.uniform(-1, 1, m.n_cells)
    for kind in ("face", "cell"):
        if kind == "face":
            D = rng.lognormal(0, 1, m.n_faces)
            Df = D
        else:
            D = rng.lognormal(0, 1, m.n_cells)
            w = O.centre_weights(own, nei, m.numpy("cell_centres"), m.numpy("face_centres"))
            Df = O.face_values(own, nei, D, w)
        mesh = m.to("cuda")
        lap, gphi, gD = _run(mesh, phi, D, g)
        ref = O.explicit_laplacian(m.n_cells, own, nei, *args, Df, V, phi)
        assert (bits(lap) == bits(ref)).all()
        assert (bits(gphi) == bits(O.explicit_laplacian(m.n_cells, own, nei, *args, Df, V, g))).all()
        gf = O.explicit_laplacian_grad_d(own, nei, *args, V, phi, g)
        if kind == "cell":
            gf = O.face_grad_to_cells(m.n_cells, own, nei, gf)
        assert (bits(gD) == bits(gf)).all()


def test_reference_unit_properties():
    d = dlap_case("two_float")
    mesh = _mesh(d)
    # tests/unit/differentiable/test_operators.py:192-213
    c = torch.tensor([5.0, 5.0], dtype=f64, device="cuda")
    assert torch.allclose(DifferentiableLaplacian.apply(c, 1.0, mesh),
                          torch.zeros(2, dtype=f64, device="cuda"), atol=1e-10)
    phi = torch.tensor([1.0, 2.0], dtype=f64, device="cuda")
    l1 = DifferentiableLaplacian.apply(phi, 1.0, mesh)
    l2 = DifferentiableLaplacian.apply(phi, 2.0, mesh)
    assert torch.allclose(l2, 2.0 * l1, atol=1e-10)
    # :215-235 gradcheck in phi and in a 0-d D
    p = phi.clone().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda q: DifferentiableLaplacian.apply(q, 1.0, mesh), (p,),
                                    eps=1e-6, atol=1e-4)
    D = torch.tensor(1.5, dtype=f64, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda q, s: DifferentiableLaplacian.apply(q, s, mesh),
                                    (p, D), eps=1e-6, atol=1e-4)


def test_bad_d_shape_raises():
    d = dlap_case("two_float")
    with pytest.raises(ValueError, match="n_faces"):
        DifferentiableLaplacian.apply(torch.ones(2, dtype=f64, device="cuda"),
                                      torch.ones(5, dtype=f64, device="cuda"), _mesh(d))


def test_pressure_equation_against_reference_golden():
    """assemble_pressure_equation bitwise (a negative and a zero A_p
    included) and solve_pressure_equation with PCG+DIC on the pinned system:
    the reference's iteration count and solution
    (solvers/pressure_equation.py:49-184)."""
    from pyopenfoam_gb300 import PCGSolver
    from pyopenfoam_gb300.solvers import assemble_pressure_equation, solve_pressure_equation
    from tests.golden.cases import DLAP_FIXTURE, jitter_case

    z = np.load(DLAP_FIXTURE)
    jc = jitter_case(6, seed=1)
    mesh = mesh_from_arrays(jc, device="cuda")
    cuda = lambda a: torch.as_tensor(a, dtype=f64, device="cuda")  # noqa: E731
    peq = assemble_pressure_equation(cuda(z["p_phiHbyA"]), cuda(z["p_A_p"]), mesh)
    for k in ("lower", "upper", "diag", "source"):
        assert (bits(getattr(peq, k).cpu().numpy()) == bits(z[f"p_{k}"])).all(), k
    peq = assemble_pressure_equation(cuda(z["p_phiHbyA"]), cuda(z["p_A_s"]), mesh)
    solver = PCGSolver(tolerance=0.0, rel_tol=1e-6, max_iter=2000, preconditioner="DIC")
    p, it, res = solve_pressure_equation(peq, torch.zeros(mesh.n_cells, dtype=f64, device="cuda"),
                                         solver, tolerance=0.0, max_iter=2000, reference_cell=5)
    assert it == int(z["p_iterations"])
    np.testing.assert_allclose(res, z["p_residual"], rtol=1e-9)
    np.testing.assert_allclose(p.cpu().numpy(), z["p_x"], rtol=0,
                               atol=1e-9 * np.abs(z["p_x"]).max())
