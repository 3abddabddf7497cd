"""OpenFOAM ``polyMesh`` files (ASCII) in and out, drop-in for the reference's
``pyfoam.io.mesh_io`` (``src/pyfoam/io/mesh_io.py:56-627``): ``read_points``,
``read_faces``, ``read_owner``, ``read_neighbour``, ``read_boundary``,
``read_mesh`` and the matching writers, plus ``read_fv_mesh`` which hands the
arrays straight to the GPU ``FvMesh``.

Parsing is vectorised with numpy (one tokenisation of the list body instead
of a regular expression per entry); faces with a common vertex count are
decoded in one reshape.  Binary-format files are refused with a
``ValueError``: only ASCII polyMesh files are read.
"""

from __future__ import annotations

import re
from pathlib import Path
from typing import Optional, Union

import numpy as np
import torch

__all__ = ["BoundaryPatch", "MeshData", "read_points", "read_faces", "read_owner",
           "read_neighbour", "read_boundary", "read_mesh", "read_fv_mesh", "write_points",
           "write_faces", "write_owner", "write_neighbour", "write_boundary", "write_mesh"]

PathLike = Union[str, Path]


class BoundaryPatch:
    """One entry of the ``boundary`` file (reference ``BoundaryPatch``)."""

    def __init__(self, name: str, patch_type: str = "patch", n_faces: int = 0,
                 start_face: int = 0, in_groups: Optional[list[str]] = None) -> None:
        self.name = name
        self.patch_type = patch_type
        self.n_faces = n_faces
        self.start_face = start_face
        self.in_groups = in_groups or []

    def as_dict(self) -> dict:
        """The ``PolyMesh`` boundary descriptor of this patch."""
        return {"name": self.name, "type": self.patch_type, "startFace": self.start_face,
                "nFaces": self.n_faces}

    def __repr__(self) -> str:
        return (f"BoundaryPatch(name={self.name!r}, type={self.patch_type!r}, "
                f"n_faces={self.n_faces}, start_face={self.start_face})")


class MeshData:
    """Everything read from one polyMesh directory (reference ``MeshData``).
    ``faces`` is a list of int32 arrays; ``face_ptr`` / ``face_pts`` hold the
    same faces as one CSR pair."""

    def __init__(self, points: torch.Tensor, faces, owner: torch.Tensor, neighbour: torch.Tensor,
                 boundary: list[BoundaryPatch]) -> None:
        self.points = points
        if isinstance(faces, tuple):
            self.face_ptr, self.face_pts = faces
        else:
            lens = np.array([len(f) for f in faces], np.int64)
            self.face_ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
            self.face_pts = (np.concatenate(faces).astype(np.int32) if faces
                             else np.zeros(0, np.int32))
        self.owner = owner
        self.neighbour = neighbour
        self.boundary = boundary

    @property
    def faces(self) -> list[np.ndarray]:
        p = self.face_ptr
        return [self.face_pts[p[i]:p[i + 1]] for i in range(self.n_faces)]

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    @property
    def n_faces(self) -> int:
        return int(self.face_ptr.shape[0] - 1)

    @property
    def n_internal_faces(self) -> int:
        return int(self.neighbour.shape[0])

    @property
    def n_cells(self) -> int:
        return int(self.owner.max().item()) + 1 if self.owner.numel() > 0 else 0

    @property
    def n_boundary_faces(self) -> int:
        return self.n_faces - self.n_internal_faces

    def __repr__(self) -> str:
        return (f"MeshData(n_points={self.n_points}, n_faces={self.n_faces}, "
                f"n_cells={self.n_cells}, n_patches={len(self.boundary)})")


# ---------------------------------------------------------------------------
_HEADER = re.compile(r"FoamFile\s*\{(.*?)\}", re.S)
_COMMENT_BLOCK = re.compile(r"/\*.*?\*/", re.S)
_COMMENT_LINE = re.compile(r"//[^\n]*")


def _read_body(path: PathLike) -> tuple[dict, str]:
    """(header entries, body without comments or header) of a FoamFile."""
    p = Path(path)
    if not p.exists():
        raise FileNotFoundError(f"File not found: {p}")
    text = p.read_bytes().decode("latin-1")
    m = _HEADER.search(text)
    if m is None:
        raise ValueError(f"{p}: no FoamFile header")
    hdr = {}
    for kv in re.finditer(r"(\w+)\s+([^;]+);", m.group(1)):
        hdr[kv.group(1)] = kv.group(2).strip().strip('"')
    if hdr.get("format", "ascii").lower() == "binary":
        raise ValueError(f"{p}: binary polyMesh files are not supported (ASCII only)")
    body = text[m.end():]
    body = _COMMENT_LINE.sub("", _COMMENT_BLOCK.sub("", body))
    return hdr, body


def _list_body(body: str, what: str) -> tuple[int, str]:
    """(count, text between the list's outer parentheses)."""
    m = re.search(r"(\d+)\s*\(", body)
    if m is None:
        raise ValueError(f"cannot find the {what} list")
    n = int(m.group(1))
    start = m.end() - 1
    depth = 0
    for i in range(start, len(body)):
        ch = body[i]
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return n, body[start + 1:i]
    raise ValueError(f"unmatched parenthesis in the {what} list")


def _tokens(text: str, dtype) -> np.ndarray:
    return np.array(text.replace("(", " ").replace(")", " ").split(), dtype=dtype)


def read_points(path: PathLike) -> tuple[dict, torch.Tensor]:
    """(header, points (n, 3) float64)."""
    hdr, body = _read_body(path)
    n, txt = _list_body(body, "points")
    v = _tokens(txt, np.float64)
    if v.shape[0] != 3 * n:
        raise ValueError(f"Expected {n} points, got {v.shape[0] / 3:g}")
    return hdr, torch.from_numpy(v.reshape(n, 3).copy())


def read_faces(path: PathLike) -> tuple[dict, tuple[np.ndarray, np.ndarray]]:
    """(header, (face_ptr int64 [n + 1], face_pts int32)) of a ``faces``
    file (``MeshData`` and ``FvMesh`` take the pair as faces)."""
    hdr, body = _read_body(path)
    n, txt = _list_body(body, "faces")
    t = _tokens(txt, np.int64)
    ptr = np.zeros(n + 1, np.int64)
    if n:
        k = int(t[0])
        if t.shape[0] == n * (k + 1) and np.all(t[:: k + 1] == k):  # one vertex count
            pts = t.reshape(n, k + 1)[:, 1:].ravel()
            ptr[1:] = np.arange(1, n + 1, dtype=np.int64) * k
        else:
            counts = np.empty(n, np.int64)
            pos = 0
            for i in range(n):
                if pos >= t.shape[0]:
                    raise ValueError(f"Expected {n} faces, got {i}")
                c = int(t[pos])
                counts[i] = c
                pos += c + 1
            if pos != t.shape[0]:
                raise ValueError(f"faces list has {t.shape[0] - pos} trailing tokens")
            np.cumsum(counts, out=ptr[1:])
            keep = np.ones(t.shape[0], bool)
            keep[ptr[:-1] + np.arange(n)] = False
            pts = t[keep]
    else:
        pts = np.zeros(0, np.int64)
    return hdr, (ptr, pts.astype(np.int32))


def _read_labels(path: PathLike, what: str) -> tuple[dict, torch.Tensor]:
    hdr, body = _read_body(path)
    n, txt = _list_body(body, what)
    v = _tokens(txt, np.int64)
    if v.shape[0] != n:
        raise ValueError(f"Expected {n} labels, got {v.shape[0]}")
    return hdr, torch.from_numpy(v)


def read_owner(path: PathLike) -> tuple[dict, torch.Tensor]:
    return _read_labels(path, "owner")


def read_neighbour(path: PathLike) -> tuple[dict, torch.Tensor]:
    return _read_labels(path, "neighbour")


def read_boundary(path: PathLike) -> tuple[dict, list[BoundaryPatch]]:
    hdr, body = _read_body(path)
    patches = []
    for bm in re.finditer(r"(\w+)\s*\{([^}]*)\}", body):
        kv = {k.group(1): k.group(2).strip().strip('"')
              for k in re.finditer(r"(\w+)\s+(.+?)\s*;", bm.group(2))}
        groups = kv.get("inGroups", "").strip()
        groups = re.sub(r"^\d+", "", groups).strip("()")
        patches.append(BoundaryPatch(bm.group(1), kv.get("type", "patch"),
                                     int(kv.get("nFaces", 0)), int(kv.get("startFace", 0)),
                                     [g.strip('"') for g in groups.split()] if groups else []))
    return hdr, patches


def read_mesh(mesh_dir: PathLike) -> MeshData:
    """All files of a ``polyMesh`` directory."""
    d = Path(mesh_dir)
    _, points = read_points(d / "points")
    _, faces = read_faces(d / "faces")
    _, owner = read_owner(d / "owner")
    _, neighbour = read_neighbour(d / "neighbour")
    _, boundary = read_boundary(d / "boundary") if (d / "boundary").exists() else ({}, [])
    return MeshData(points, faces, owner, neighbour, boundary)


def read_fv_mesh(mesh_dir: PathLike, device=None):
    """``FvMesh`` (GPU geometry) of a ``polyMesh`` directory."""
    from ..mesh.fv_mesh import FvMesh

    md = read_mesh(mesh_dir)
    return FvMesh(md.points, (md.face_ptr, md.face_pts), md.owner, md.neighbour,
                  [p.as_dict() for p in md.boundary], device=device)


# ---------------------------------------------------------------------------
def _write(path: PathLike, cls: str, obj: str, body: str, overwrite: bool) -> None:
    p = Path(path)
    if p.exists() and not overwrite:
        raise FileExistsError(f"File already exists: {p}")
    p.parent.mkdir(parents=True, exist_ok=True)
    head = ("FoamFile\n{\n    version     2.0;\n    format      ascii;\n"
            f"    class       {cls};\n    location    \"constant/polyMesh\";\n"
            f"    object      {obj};\n}}\n\n")
    p.write_text(head + body + "\n", encoding="utf-8")


def write_points(path: PathLike, points, *, overwrite: bool = False) -> None:
    pts = np.asarray(points.detach().cpu() if isinstance(points, torch.Tensor) else points,
                     np.float64).reshape(-1, 3)
    lines = [f"({x!r} {y!r} {z!r})" for x, y, z in pts.tolist()]
    _write(path, "vectorField", "points", f"{pts.shape[0]}\n(\n" + "\n".join(lines) + "\n)",
           overwrite)


def write_faces(path: PathLike, faces, *, overwrite: bool = False) -> None:
    if isinstance(faces, tuple):
        ptr, pts = (np.asarray(a) for a in faces)
        faces = [pts[ptr[i]:ptr[i + 1]] for i in range(ptr.shape[0] - 1)]
    lines = [f"{len(f)}(" + " ".join(str(int(v)) for v in f) + ")" for f in faces]
    _write(path, "faceList", "faces", f"{len(faces)}\n(\n" + "\n".join(lines) + "\n)", overwrite)


def _write_labels(path: PathLike, obj: str, labels, overwrite: bool) -> None:
    v = np.asarray(labels.detach().cpu() if isinstance(labels, torch.Tensor) else labels,
                   np.int64)
    _write(path, "labelList", obj, f"{v.shape[0]}\n(\n" + "\n".join(map(str, v.tolist()))
           + "\n)", overwrite)


def write_owner(path: PathLike, owner, *, overwrite: bool = False) -> None:
    _write_labels(path, "owner", owner, overwrite)


def write_neighbour(path: PathLike, neighbour, *, overwrite: bool = False) -> None:
    _write_labels(path, "neighbour", neighbour, overwrite)


def write_boundary(path: PathLike, patches: list[BoundaryPatch], *,
                   overwrite: bool = False) -> None:
    lines = [f"{len(patches)}", "("]
    for p in patches:
        lines += [f"    {p.name}", "    {", f"        type            {p.patch_type};",
                  f"        nFaces          {p.n_faces};",
                  f"        startFace       {p.start_face};"]
        if p.in_groups:
            lines.append("        inGroups        (" + " ".join(p.in_groups) + ");")
        lines.append("    }")
    lines.append(")")
    _write(path, "polyBoundaryMesh", "boundary", "\n".join(lines), overwrite)


def write_mesh(mesh_dir: PathLike, points, faces, owner, neighbour,
               boundary: list[BoundaryPatch], *, overwrite: bool = False) -> None:
    """Write the five files of a ``polyMesh`` directory."""
    d = Path(mesh_dir)
    write_points(d / "points", points, overwrite=overwrite)
    write_faces(d / "faces", faces, overwrite=overwrite)
    write_owner(d / "owner", owner, overwrite=overwrite)
    write_neighbour(d / "neighbour", neighbour, overwrite=overwrite)
    write_boundary(d / "boundary", boundary, overwrite=overwrite)
