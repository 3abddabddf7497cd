"""Mesh inputs of the linear-solve path (hex meshes with LDU addressing)."""

from .hex_mesh import HexMesh, PATCH_NAMES

__all__ = ["HexMesh", "PATCH_NAMES"]
