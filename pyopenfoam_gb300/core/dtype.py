"""dtype helpers mirroring ``src/pyfoam/core/dtype.py``."""

from __future__ import annotations

import torch

__all__ = ["CFD_DTYPE", "INDEX_DTYPE", "assert_floating", "is_floating"]

#: default floating dtype of the linear-solve path (core/dtype.py:38)
CFD_DTYPE: torch.dtype = torch.float64
#: index dtype of owner/neighbour addressing (core/dtype.py:47)
INDEX_DTYPE: torch.dtype = torch.int64


def is_floating(dtype: torch.dtype) -> bool:
    return dtype.is_floating_point


def assert_floating(tensor: torch.Tensor, name: str = "tensor") -> None:
    """Raise ``TypeError`` unless *tensor* is floating point
    (core/dtype.py:169-178)."""
    if not is_floating(tensor.dtype):
        raise TypeError(f"{name} must have a floating-point dtype, got {tensor.dtype}")
