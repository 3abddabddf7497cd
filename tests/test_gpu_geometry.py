"""GPU mesh geometry (FvMesh on gbf_face_geometry_f64 / gbf_cell_geometry_f64
/ gbf_face_interp_f64) against the reference's own FvMesh outputs
(tests/golden/reference_geometry.npz, made by make_golden.py --geometry) and,
at a size the reference cannot reach, against the vectorised hex-mesh
geometry of the harness; plus the polyMesh reader round trip.

Bars: face centres and area vectors bitwise; cell volumes, centres, weights
and delta coefficients to 1e-14 relative (the reference averages a Python
set of vertex ids and calls a library dot product, whose order is not
reproduced)."""

import os

import numpy as np
import pytest
import torch

from pyopenfoam_gb300.io import read_fv_mesh, write_mesh
from pyopenfoam_gb300.io.mesh_io import BoundaryPatch
from pyopenfoam_gb300.mesh import FvMesh, HexMesh
from tests.golden.cases import hex_polymesh

pytestmark = pytest.mark.gpu
GEO = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_geometry.npz"))
KEYS = ("face_centres", "face_areas", "cell_volumes", "cell_centres", "face_weights",
        "delta_coefficients")


def _mesh(tag) -> FvMesh:
    return FvMesh(GEO[f"{tag}_points"], (GEO[f"{tag}_face_ptr"], GEO[f"{tag}_face_pts"]),
                  GEO[f"{tag}_owner"], GEO[f"{tag}_neighbour"], device="cuda")


def _rel(a, b):
    scale = np.maximum(np.abs(b), 1e-300)
    return float(np.max(np.abs(a - b) / np.where(np.abs(b) > 0, scale, 1.0)))


@pytest.mark.parametrize("tag", ["hex", "prism", "two"])
def test_geometry_matches_reference_fvmesh(tag):
    m = _mesh(tag)
    m.compute_geometry()
    assert m.n_cells == int(GEO[f"{tag}_n_cells"])
    for k in ("face_centres", "face_areas"):
        got = getattr(m, k).cpu().numpy()
        assert got.view(np.int64).tolist() == GEO[f"{tag}_{k}"].view(np.int64).tolist(), k
    for k in ("cell_volumes", "cell_centres", "face_weights", "delta_coefficients"):
        got, ref = getattr(m, k).cpu().numpy(), GEO[f"{tag}_{k}"]
        assert got.shape == ref.shape
        assert np.allclose(got, ref, rtol=1e-14, atol=1e-15), (k, _rel(got, ref))
    assert abs(float(m.total_volume) - float(GEO[f"{tag}_cell_volumes"].sum())) < 1e-13
    # boundary conventions of the reference: weight 1, delta 0
    ni = m.n_internal_faces
    assert torch.all(m.face_weights[ni:] == 1.0) and torch.all(m.delta_coefficients[ni:] == 0)


def test_polymesh_files_round_trip(tmp_path):
    d = hex_polymesh(5, 4, 3, jitter=0.2, seed=3)
    ptr, pts = d["face_ptr"], d["face_pts"]
    faces = [pts[ptr[i]:ptr[i + 1]] for i in range(ptr.shape[0] - 1)]
    patches = [BoundaryPatch(b["name"], b["type"], b["nFaces"], b["startFace"])
               for b in d["boundary"]]
    write_mesh(tmp_path / "polyMesh", d["points"], faces, d["owner"], d["neighbour"], patches)
    m = read_fv_mesh(tmp_path / "polyMesh", device="cuda")
    ref = FvMesh(d["points"], (ptr, pts), d["owner"], d["neighbour"], device="cuda")
    for k in KEYS:
        a, b = getattr(m, k).cpu().numpy(), getattr(ref, k).cpu().numpy()
        assert (a.view(np.int64) == b.view(np.int64)).all(), k
    assert [p["name"] for p in m.boundary] == [b["name"] for b in d["boundary"]]


@pytest.mark.parametrize("N", [48])
def test_geometry_at_scale_matches_vectorised_hex_geometry(N):
    """A jittered N^3 hex mesh (110,592 cells): the GPU geometry against the
    harness's numpy restatement of the same formulas."""
    d = hex_polymesh(N, N, N, jitter=0.2, seed=5)
    m = FvMesh(d["points"], (d["face_ptr"], d["face_pts"]), d["owner"], d["neighbour"],
               device="cuda")
    h = HexMesh(N, jitter=0.2, seed=5, dirichlet=())
    for k, hk in (("face_centres", "face_centres"), ("face_areas", "face_areas"),
                  ("cell_volumes", "cell_volumes"), ("cell_centres", "cell_centres"),
                  ("face_weights", "weights"), ("delta_coefficients", "delta_coefficients")):
        got, ref = getattr(m, k).cpu().numpy(), h.numpy(hk)
        tol = 1e-12 * max(float(np.abs(ref).max()), 1e-300)
        assert np.abs(got - ref).max() <= tol, (k, float(np.abs(got - ref).max()))
    assert abs(float(m.total_volume) - 1.0) < 1e-12


def test_fvm_laplacian_on_gpu_fvmesh():
    """fvm.laplacian takes the GPU FvMesh directly (duck-typed like the
    reference's); its coefficients follow the reference formula."""
    from oracle import oracle as O
    from pyopenfoam_gb300.discretisation import fvm

    m = _mesh("prism")
    gamma = torch.as_tensor(np.random.default_rng(2).lognormal(0.0, 0.5, m.n_faces))
    A = fvm.laplacian(gamma, torch.zeros(1), mesh=m)
    lo, up, dg = O.laplacian(m.n_cells, GEO["prism_owner"], GEO["prism_neighbour"],
                             m.face_areas.cpu().numpy(), m.delta_coefficients.cpu().numpy(),
                             gamma.numpy(), m.cell_volumes.cpu().numpy())
    assert np.array_equal(A.lower.cpu().numpy(), lo)
    assert np.array_equal(A.upper.cpu().numpy(), up)
    assert np.array_equal(A.diag.cpu().numpy(), dg)


def test_polymesh_validation_errors():
    d = hex_polymesh(2, 2, 2)
    bad = d["neighbour"].copy()
    bad[0] = d["owner"][0]  # owner == neighbour violates owner < neighbour
    with pytest.raises(ValueError):
        FvMesh(d["points"], (d["face_ptr"], d["face_pts"]), d["owner"], bad, device="cuda")
    pts = d["face_pts"].copy()
    pts[0] = d["points"].shape[0]  # a vertex that does not exist
    with pytest.raises(ValueError):
        FvMesh(d["points"], (d["face_ptr"], pts), d["owner"], d["neighbour"], device="cuda")
    with pytest.raises(ValueError):
        FvMesh(d["points"], (d["face_ptr"], d["face_pts"]), d["owner"], d["neighbour"],
               device="cpu")
