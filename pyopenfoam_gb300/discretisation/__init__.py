"""Finite-volume operators of the linear-solve path (GPU assembly)."""

from .operators import fvm

__all__ = ["fvm"]
