"""Seeded test cases shared by the golden-fixture generator and the tests.

Every generator is deterministic across platforms: indices are integer
arithmetic, random values come from ``numpy.random.default_rng`` (PCG64), and
the 32^3 Poisson coefficients are exact powers of two.  The jittered-mesh case
stores its geometry in the fixture, so no test depends on floating-point
geometry being bit-identical across machines.
"""

from __future__ import annotations

import hashlib
import os
import sys
from types import SimpleNamespace

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "reference_outputs.npz")
JITTER_FIXTURE = os.path.join(HERE, "jitter6_inputs.npz")
LDU128_FIXTURE = os.path.join(HERE, "reference_ldu128.npz")


def sha(a: np.ndarray) -> str:
    """SHA-256 of the little-endian bytes of a float array (float64 unless
    the array is float32)."""
    a = np.asarray(a)
    dt = "<f4" if a.dtype == np.float32 else "<f8"
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dt).tobytes()).hexdigest()


from pyopenfoam_gb300.mesh.poisson import hex_faces, hex_poisson  # noqa: E402


def random_ldu(N: int, seed: int = 5, permute_faces: bool = False) -> dict:
    """Random LDU coefficients on an N^3 hex topology.  With
    ``permute_faces`` the face order is shuffled and a third of the faces
    have owner > neighbour, which exercises unsorted, non-triangular
    addressing."""
    n, own, nei = hex_faces(N)
    rng = np.random.default_rng(seed)
    F = own.shape[0]
    if permute_faces:
        perm = rng.permutation(F)
        own, nei = own[perm].copy(), nei[perm].copy()
        flip = rng.random(F) < 0.33
        own[flip], nei[flip] = nei[flip].copy(), own[flip].copy()
    return dict(
        n=n, owner=own, neighbour=nei,
        lower=rng.uniform(-1.0, 0.0, F), upper=rng.uniform(-1.0, 0.0, F),
        diag=rng.uniform(6.0, 7.0, n), x=rng.uniform(-1.0, 1.0, n),
        r=rng.uniform(-1.0, 1.0, n),
    )


def c1_poisson(N: int = 32, seed: int = 0) -> dict:
    """The 32^3 Poisson system (see pyopenfoam_gb300.mesh.poisson.hex_poisson)."""
    return hex_poisson(N, seed)


def mesh_from_arrays(d: dict, device="cpu", dtype=None):
    """Duck-typed FvMesh (the attributes fvm.laplacian / fvm.div read)."""
    import torch

    dtype = dtype or torch.float64
    t = lambda a, dt=dtype: torch.as_tensor(np.asarray(a)).to(device=device, dtype=dt)  # noqa: E731
    return SimpleNamespace(
        n_cells=int(d["n_cells"]), n_internal_faces=int(d["n_internal"]),
        n_faces=int(d["owner"].shape[0]),
        owner=t(d["owner"], torch.int64), neighbour=t(d["neighbour"], torch.int64),
        face_areas=t(d["face_areas"]), delta_coefficients=t(d["delta"]),
        cell_volumes=t(d["volumes"]), device=torch.device(device), dtype=dtype,
        cell_centres=t(d["cell_centres"]) if "cell_centres" in d else None,
        face_centres=t(d["face_centres"]) if "face_centres" in d else None,
    )


def jitter_case(N: int = 6, seed: int = 1, store: bool = True):
    """Jittered (+-20 % h) N^3 mesh with Dirichlet x0, log-normal face
    diffusivity, an all-positive upwind flux from u = (1, 0.5, 0.25) on the
    nominal face areas, RHS and loss weights.  The arrays are written to /
    read from ``jitter{N}_inputs.npz`` so that every machine uses the same
    bits."""
    path = os.path.join(HERE, f"jitter{N}_inputs.npz")
    if os.path.exists(path):
        z = np.load(path)
        d = {k: z[k] for k in z.files}
    else:
        import sys

        sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
        from pyopenfoam_gb300.mesh import HexMesh

        m = HexMesh(N, jitter=0.2, seed=seed)
        rng = np.random.default_rng(seed + 100)
        nint = m.n_internal_faces
        nom = HexMesh(N)  # unjittered: nominal face area vectors
        u = np.array([1.0, 0.5, 0.25])
        phi = (nom.numpy("face_areas") * u).sum(axis=1) * 3.0 * N
        d = dict(
            n_cells=np.int64(m.n_cells), n_internal=np.int64(nint),
            owner=m.numpy("owner"), neighbour=m.numpy("neighbour"),
            face_areas=m.numpy("face_areas"), delta=m.numpy("delta_coefficients"),
            volumes=m.numpy("cell_volumes"), cell_centres=m.numpy("cell_centres"),
            face_centres=m.numpy("face_centres"),
            gamma=rng.lognormal(0.0, 1.0, m.n_faces), phi=phi,
            b=rng.uniform(-1.0, 1.0, m.n_cells), w=rng.uniform(-1.0, 1.0, m.n_cells),
        )
        if store:
            np.savez_compressed(path, **d)
    d["mesh"] = mesh_from_arrays(d)
    return d


def unroll_case(N: int = 10, dt: float = 1e-3, steps: int = 20, seed: int = 4,
                with_target: bool = True, threads: int = 1) -> dict:
    """The adjoint workload's structure on a uniform N^3 mesh (fixed value on
    x0): per-face diffusivity gamma ~ LogNormal(0, 1), a second draw gamma',
    x0 ~ U[0, 1] (the draws of the 96^3 workload when N = 96), and a target
    produced by the same 20 implicit steps with gamma' (computed here with
    the oracle restatement, fvm.laplacian + PCG on ``threads`` threads;
    ``with_target=False`` leaves it out, ``target`` is then None)."""
    from pyopenfoam_gb300.mesh import HexMesh

    m = HexMesh(N)
    rng = np.random.default_rng(seed)
    gamma = rng.lognormal(0.0, 1.0, m.n_faces)
    gamma2 = rng.lognormal(0.0, 1.0, m.n_faces)
    x0 = rng.uniform(0.0, 1.0, m.n_cells)
    d = dict(n_cells=np.int64(m.n_cells), n_internal=np.int64(m.n_internal_faces),
             owner=m.numpy("owner"), neighbour=m.numpy("neighbour"),
             face_areas=m.numpy("face_areas"), delta=m.numpy("delta_coefficients"),
             volumes=m.numpy("cell_volumes"))
    x = None
    if with_target:
        from oracle import oracle as O

        nint = m.n_internal_faces
        lo, up, dg = O.laplacian(m.n_cells, d["owner"], d["neighbour"], d["face_areas"],
                                 d["delta"], gamma2, d["volumes"])
        x = x0.copy()
        for _ in range(steps):
            x = O.pcg(d["owner"][:nint], d["neighbour"], dg + 1.0 / dt, lo, up, x / dt, x, None,
                      0.0, 1e-14, 5000, threads=threads).x
    d.update(gamma=gamma, gamma2=gamma2, x0=x0, target=x, dt=dt, steps=steps)
    d["mesh"] = mesh_from_arrays(d)
    return d


DLAP_FIXTURE = os.path.join(HERE, "reference_dlap.npz")
DLAP_CASES = ("j6_face", "j6_cell", "j6_scalar", "j6_float", "two_float", "two_scalar",
              "two_face")


def dlap_case(tag: str) -> dict:
    """Inputs of one DifferentiableLaplacian golden (make_golden.py --dlap):
    the mesh arrays, phi, the loss weights g (grad_output) and D as
    ``(kind, value)`` with kind in face / cell / scalar (0-d tensor) /
    float."""
    z = np.load(DLAP_FIXTURE)
    kind = tag.split("_", 1)[1]
    if tag.startswith("j6"):
        jc = jitter_case(6, seed=1)
        d = {k: jc[k] for k in ("owner", "neighbour", "face_areas", "delta", "volumes",
                                "cell_centres", "face_centres")}
        d["n_cells"], d["n_internal"] = int(jc["n_cells"]), int(jc["n_internal"])
        d["phi"], d["g"] = z["j6_phi"], jc["w"]
        D = {"face": jc["gamma"], "cell": np.random.default_rng(7).lognormal(0.0, 1.0, d["n_cells"]),
             "scalar": 1.5, "float": 2.0}[kind]
    else:
        d = {k: z[f"two_{k}"] for k in ("owner", "neighbour", "face_areas", "delta", "volumes",
                                          "cell_centres", "face_centres")}
        d["n_cells"], d["n_internal"] = 2, int(z["two_n_internal"])
        d["phi"], d["g"] = np.array([1.0, 2.0]), np.ones(2)
        nf = d["owner"].shape[0]
        D = {"face": np.linspace(0.5, 1.5, nf), "scalar": 1.5, "float": 1.0}[kind]
    d["kind"], d["D"] = kind, D
    d["expect"] = {k[len(tag) + 1:]: z[k] for k in z.files if k.startswith(tag + "_")}
    return d


# ---------------------------------------------------------------------------
# Polyhedral meshes for the geometry goldens (points, faces, owner,
# neighbour, boundary) in OpenFOAM conventions: owner < neighbour, internal
# faces before boundary faces, normals out of the owner.
# ---------------------------------------------------------------------------
def hex_polymesh(nx: int, ny: int, nz: int, jitter: float = 0.2, seed: int = 11) -> dict:
    """Jittered hex mesh of the unit box as a polyMesh."""
    from pyopenfoam_gb300.mesh.hex_mesh import PATCH_NAMES, HexMesh

    m = HexMesh(nx, ny, nz, jitter=jitter, seed=seed)
    cells = np.concatenate([m._int_cell, m._bnd_cell])
    kind = np.concatenate([m._int_dir, m._bnd_kind + 3])
    faces = m._face_points(cells, kind)
    boundary = [{"name": p, "type": "patch", "startFace": m.patches[p].start,
                 "nFaces": m.patches[p].size} for p in PATCH_NAMES]
    return dict(points=m._points.copy(), face_ptr=np.arange(0, 4 * faces.shape[0] + 1, 4),
                face_pts=faces.ravel().astype(np.int64), owner=m._owner_np.copy(),
                neighbour=m._neigh_np.copy(), boundary=boundary)


def prism_polymesh(nx: int, ny: int, nz: int, jitter: float = 0.15, seed: int = 12) -> dict:
    """Each hex of an nx*ny*nz box split along its xy diagonal into two
    triangular prisms (triangle and quad faces, five faces per cell)."""
    rng = np.random.default_rng(seed)
    P = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)  # noqa: E731
    gx, gy, gz = (np.linspace(0.0, 1.0, n + 1) for n in (nx, ny, nz))
    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    pid = np.arange(pts.shape[0])
    ii, jj, kk = pid % (nx + 1), (pid // (nx + 1)) % (ny + 1), pid // ((nx + 1) * (ny + 1))
    inner = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)
    h = np.array([1.0 / nx, 1.0 / ny, 1.0 / nz])
    pts[inner] += rng.uniform(-jitter, jitter, (int(inner.sum()), 3)) * h
    # cells: triangles (a, b, c) in xy, counter-clockwise seen from +z
    cell_tris = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                p00, p10, p11, p01 = (i, j), (i + 1, j), (i + 1, j + 1), (i, j + 1)
                cell_tris.append((k, (p00, p10, p11)))
                cell_tris.append((k, (p00, p11, p01)))
    n_cells = len(cell_tris)
    centroid = np.array([np.mean([pts[P(a, b, kk_)] for (a, b) in tri for kk_ in (k, k + 1)],
                                 axis=0) for k, tri in cell_tris])
    faces: dict[tuple, list] = {}
    for c, (k, tri) in enumerate(cell_tris):
        bot = [P(a, b, k) for (a, b) in tri]
        top = [P(a, b, k + 1) for (a, b) in tri]
        cand = [bot, top] + [[bot[q], bot[(q + 1) % 3], top[(q + 1) % 3], top[q]]
                              for q in range(3)]
        for f in cand:
            faces.setdefault(tuple(sorted(f)), []).append((c, f))
    internal, bnd = [], []
    for key, users in faces.items():
        if len(users) == 2:
            (c0, f0), (c1, _) = sorted(users)
            internal.append((c0, c1, f0))
        else:
            bnd.append((users[0][0], users[0][1]))
    internal.sort(key=lambda t: (t[0], t[1]))
    bnd.sort(key=lambda t: t[0])

    def orient(f, frm, to):
        v = pts[f]
        a = 0.5 * sum(np.cross(v[q], v[(q + 1) % len(f)]) for q in range(len(f)))
        return f if np.dot(a, to - frm) > 0 else f[::-1]

    flist, own, nei = [], [], []
    for c0, c1, f in internal:
        flist.append(orient(f, centroid[c0], centroid[c1]))
        own.append(c0)
        nei.append(c1)
    for c0, f in bnd:
        flist.append(orient(f, centroid[c0], pts[f].mean(axis=0)))
        own.append(c0)
    ptr = np.concatenate([[0], np.cumsum([len(f) for f in flist])])
    return dict(points=pts, face_ptr=ptr.astype(np.int64),
                face_pts=np.concatenate(flist).astype(np.int64),
                owner=np.array(own, np.int64), neighbour=np.array(nei, np.int64),
                boundary=[{"name": "walls", "type": "wall", "startFace": len(internal),
                           "nFaces": len(bnd)}], n_cells=n_cells)
