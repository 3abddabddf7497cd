"""Device policy: every tensor of the linear-solve path lives on a CUDA device.

The reference keeps a global CPU/CUDA/MPS configuration
(``src/pyfoam/core/device.py:139-300``).  This package has one backend, the
sm_103a kernels of libgbfoam, so the default device is the current CUDA
device and a CPU device is rejected: there is no CPU fallback.
"""

from __future__ import annotations

import torch

__all__ = ["resolve_device", "get_device"]


def get_device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError(
            "pyopenfoam_gb300 needs a CUDA device (it has no CPU fallback); "
            "torch.cuda.is_available() is False"
        )
    return torch.device("cuda", torch.cuda.current_device())


def resolve_device(device) -> torch.device:
    if device is None:
        return get_device()
    dev = torch.device(device)
    if dev.type != "cuda":
        raise ValueError(
            f"pyopenfoam_gb300 runs on CUDA devices only (no CPU fallback); got device={dev}"
        )
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev
