"""Device policy: every tensor of the linear-solve path lives on a CUDA device.

The reference keeps a global CPU/CUDA/MPS configuration
(``src/pyfoam/core/device.py:139-300``).  This package has one backend, the
sm_103a kernels of libgbfoam, so the default device is the current CUDA
device and a CPU device is rejected: there is no CPU fallback.
"""

from __future__ import annotations

import torch

__all__ = ["resolve_device", "get_device", "to_device", "to_host"]


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


def _sm_copy_ok(t: torch.Tensor) -> bool:
    return t.device.type == "cpu" and t.numel() > 0 and t.is_contiguous() and t.is_pinned()


def to_device(t, device: torch.device, dtype: torch.dtype) -> torch.Tensor:
    """``t`` as a contiguous ``dtype`` tensor on ``device``, like
    ``t.to(device=device, dtype=dtype).contiguous()`` (and, like it, done
    when it returns).

    A page-locked CPU tensor that already has ``dtype`` is moved by the SMs
    (``gbf_copy_from_host``: 16-byte loads over NVLink-C2C at the link's
    rate) instead of the copy engines, whose rate on GB300 hosts varied from
    the link's 210 GB/s down to ~16 GB/s between otherwise identical copies.
    """
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(t)
    if not (_sm_copy_ok(t) and t.dtype == dtype and device.type == "cuda"):
        return t.to(device=device, dtype=dtype).contiguous()
    from .. import _lib

    out = torch.empty(t.shape, dtype=dtype, device=device)
    with torch.cuda.device(out.device):  # the library launches on the current device
        stream = torch.cuda.current_stream(out.device)
        _lib.check(_lib.lib().gbf_copy_from_host(out.data_ptr(), t.data_ptr(),
                                                 t.numel() * t.element_size(),
                                                 stream.cuda_stream),
                   "gbf_copy_from_host")
        stream.synchronize()
    return out


def to_host(t: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """A CPU copy of the CUDA tensor ``t``, done when it returns.  Into
    ``out`` when given: a page-locked, contiguous CPU tensor of ``t``'s
    dtype and size is filled by the SMs (``gbf_copy_to_host``); any other
    ``out`` by ``out.copy_(t)``."""
    if out is None:
        return t.cpu()
    src = t.contiguous()
    if not (_sm_copy_ok(out) and out.dtype == src.dtype and out.numel() == src.numel()
            and src.device.type == "cuda"):
        out.copy_(t)
        return out
    from .. import _lib

    with torch.cuda.device(src.device):
        stream = torch.cuda.current_stream(src.device)
        _lib.check(_lib.lib().gbf_copy_to_host(out.data_ptr(), src.data_ptr(),
                                               src.numel() * src.element_size(),
                                               stream.cuda_stream),
                   "gbf_copy_to_host")
        stream.synchronize()
    return out
