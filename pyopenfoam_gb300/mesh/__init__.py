"""Mesh inputs of the linear-solve path: structured hex meshes with LDU
addressing (the benchmark harness) and polyhedral meshes with GPU-computed
finite-volume geometry (``FvMesh``)."""

from .fv_mesh import FvMesh, PolyMesh
from .hex_mesh import HexMesh, PATCH_NAMES

__all__ = ["HexMesh", "PATCH_NAMES", "PolyMesh", "FvMesh"]
