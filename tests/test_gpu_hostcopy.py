"""SM-driven host <-> device copies (gbf_copy_from_host / gbf_copy_to_host)
and the paths that use them: ``to_device`` / ``to_host``, the LduMatrix
setters and the solvers' right-hand side given as page-locked CPU tensors.

The bar is bytewise equality with torch's own copies, for every alignment of
source and destination (the kernel moves the widest word both are aligned
to and the rest byte by byte) and for sizes around the word and grid
boundaries; memory that is not page-locked is refused by the C ABI and
copied by torch instead."""

import numpy as np
import pytest
import torch

from pyopenfoam_gb300 import LduMatrix, MixedPrecisionPCGSolver, _lib
from pyopenfoam_gb300.core.device import to_device, to_host
from pyopenfoam_gb300.mesh.poisson import hex_poisson

pytestmark = pytest.mark.gpu


def _raw(dst, src, nbytes, up=True):
    fn = _lib.lib().gbf_copy_from_host if up else _lib.lib().gbf_copy_to_host
    rc = fn(dst, src, nbytes, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc


@pytest.mark.parametrize("nbytes", [1, 7, 8, 15, 16, 17, 255, 4096, 65537, (1 << 22) + 3,
                                    256 * 16 * 152 * 4 * 16 + 5])
@pytest.mark.parametrize("soff,doff", [(0, 0), (8, 8), (1, 1), (4, 12), (3, 0)])
def test_sm_copies_are_bytewise_for_any_alignment(nbytes, soff, doff):
    g = torch.Generator().manual_seed(nbytes + 31 * soff + doff)
    host = torch.randint(0, 256, (nbytes + 64,), dtype=torch.uint8, generator=g).pin_memory()
    dev = torch.zeros(nbytes + 64, dtype=torch.uint8, device="cuda")
    assert _raw(dev.data_ptr() + doff, host.data_ptr() + soff, nbytes) == 0
    got = dev.cpu().numpy()
    want = np.zeros(nbytes + 64, np.uint8)
    want[doff:doff + nbytes] = host.numpy()[soff:soff + nbytes]
    assert np.array_equal(got, want)
    back = torch.zeros(nbytes + 64, dtype=torch.uint8).pin_memory()
    assert _raw(back.data_ptr() + soff, dev.data_ptr() + doff, nbytes, up=False) == 0
    w2 = np.zeros(nbytes + 64, np.uint8)
    w2[soff:soff + nbytes] = want[doff:doff + nbytes]
    assert np.array_equal(back.numpy(), w2)


def test_sm_copy_refuses_memory_that_is_not_page_locked():
    pageable = torch.arange(1000, dtype=torch.float64)
    dev = torch.empty(1000, dtype=torch.float64, device="cuda")
    rc = _lib.lib().gbf_copy_from_host(dev.data_ptr(), pageable.data_ptr(), 8000,
                                       torch.cuda.current_stream().cuda_stream)
    assert rc == 1  # GBF_ERR_ARG
    assert "page-locked" in _lib.lib().gbf_last_error().decode()
    # device memory as the source of an upload, or host memory as the target
    pinned = pageable.pin_memory()
    assert _lib.lib().gbf_copy_from_host(pinned.data_ptr(), dev.data_ptr(), 8000, None) != 0
    # the Python helpers fall back to torch for pageable memory
    assert torch.equal(to_device(pageable, dev.device, torch.float64).cpu(), pageable)
    out = torch.empty(1000, dtype=torch.float64)
    assert torch.equal(to_host(dev.copy_(pageable.cuda()), out), pageable)


def test_to_device_converts_like_torch():
    """dtype conversion, non-contiguous views and Python sequences go through
    torch (same values); a page-locked tensor of the right dtype through the
    SM copy (same bits)."""
    dev = torch.device("cuda", torch.cuda.current_device())
    p = torch.randn(4097, dtype=torch.float64).pin_memory()
    assert torch.equal(to_device(p, dev, torch.float64).cpu(), p)
    assert torch.equal(to_device(p, dev, torch.float32).cpu(), p.float())
    assert torch.equal(to_device(p[::2], dev, torch.float64).cpu(), p[::2])
    assert torch.equal(to_device([1.0, 2.0], dev, torch.float64).cpu(),
                       torch.tensor([1.0, 2.0], dtype=torch.float64))
    assert to_device(torch.empty(0, dtype=torch.float64).pin_memory(), dev,
                     torch.float64).numel() == 0


def test_setters_and_solver_take_page_locked_host_tensors():
    """The headline's inputs handed over as page-locked host tensors: the
    matrix holds the same bits and the mixed solve gives the same x and
    iteration count as with device inputs; x read back by to_host."""
    d = hex_poisson(24, seed=2)
    own, nei = torch.as_tensor(d["owner"]), torch.as_tensor(d["neighbour"])
    md = LduMatrix(d["n"], own, nei, device="cuda")
    md.diag, md.lower, md.upper = (torch.as_tensor(d[k]).cuda() for k in ("diag", "lower", "upper"))
    mh = LduMatrix(d["n"], own, nei, device="cuda")
    mh.diag, mh.lower, mh.upper = (torch.as_tensor(d[k]).pin_memory()
                                   for k in ("diag", "lower", "upper"))
    for k in ("diag", "lower", "upper"):
        assert torch.equal(getattr(md, k), getattr(mh, k))
    s = MixedPrecisionPCGSolver(tolerance=0.0, rel_tol=1e-10, max_iter=2000, preconditioner="DIC")
    x0 = torch.zeros(d["n"], dtype=torch.float64, device="cuda")
    xd, itd, _ = s(md, torch.as_tensor(d["b"]).cuda(), x0)
    xh, ith, _ = s(mh, torch.as_tensor(d["b"]).pin_memory(), x0)
    assert itd == ith and torch.equal(xd, xh)
    out = torch.empty(d["n"], dtype=torch.float64).pin_memory()
    assert to_host(xh, out) is out and torch.equal(out, xd.cpu())
