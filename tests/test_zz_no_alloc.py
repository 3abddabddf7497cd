"""The no-allocation PCG entry point (gbf_pcg_solve_f64_noalloc).

It exists for callers that cannot allocate device memory at the moment they
solve: real-time loops that must never wait on the allocator, host codes
whose device memory belongs to their own pool or a fixed budget, plugin hosts
that offer the library no allocator.  Its scratch comes from a fixed
file-scope device array, so this test calls it straight through the C ABI (no
torch workspace) and checks, on two calls in a row, that it gives what the
workspace entry point gives on the same input.

The workspace arm runs with variant 1, the same three-kernel iteration the
no-allocation entry point always runs, so the two must agree bit for bit:
x, the residual history and the iteration count.  Systems run large then
small and small then large, so that a layout or offset error in the scratch
carve-up, or a leftover from a longer previous vector, cannot hide in a
tolerance.

The file is named to be collected last, so that a run stopping at the first
failure has already run every other test; it also passes on its own in a
fresh process (the first call on the device sets up the scratch address).
"""

import ctypes

import numpy as np
import pytest
import torch

from pyopenfoam_gb300 import DICPreconditioner, LduMatrix, _lib
from pyopenfoam_gb300.mesh.poisson import hex_poisson

pytestmark = pytest.mark.gpu

MAX_CELLS = 1 << 20


def _system(N, seed):
    d = hex_poisson(N, seed=seed)
    m = LduMatrix(d["n"], torch.as_tensor(d["owner"]), torch.as_tensor(d["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(d[k]) for k in ("diag", "lower", "upper"))
    return m, torch.as_tensor(d["b"]).cuda()


def _solve(m, b, pd, noalloc, max_iter=400, rel_tol=1e-9, variant=1, generic=False):
    L = _lib.lib()
    topo = m.topology()
    plain = topo.uncompressed_layout() if generic else None
    layout = ctypes.byref(plain) if generic else topo.layout_ref
    coef = m.packed()
    x = torch.zeros_like(b)
    hist = torch.zeros(max_iter + 1, dtype=torch.float64, device="cuda")
    P = _lib.SolveParams(0.0, rel_tol, max_iter, 0, 16, variant)
    R = _lib.SolveResult()
    stream = torch.cuda.current_stream().cuda_stream
    args = (layout, coef.data_ptr(), m.diag.data_ptr(), pd.data_ptr(), b.data_ptr(),
            x.data_ptr(), hist.data_ptr(), ctypes.byref(P), ctypes.byref(R))
    if noalloc:
        rc = L.gbf_pcg_solve_f64_noalloc(*args, stream)
    else:
        ws = torch.empty(int(L.gbf_pcg_workspace_bytes(m.n_cells)), dtype=torch.uint8,
                         device="cuda")
        rc = L.gbf_pcg_solve_f64(*args, ws.data_ptr(), ws.numel(), stream)
    _lib.check(rc, "pcg solve")
    torch.cuda.synchronize()
    return x.cpu().numpy(), R.iterations, R.final_residual, hist[: R.iterations].cpu().numpy()


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.int64)


@pytest.mark.parametrize("order", [((40, 4), (24, 3)), ((24, 3), (40, 4))],
                         ids=["large_then_small", "small_then_large"])
@pytest.mark.parametrize("generic", [False, True], ids=["hex_layout", "generic_layout"])
def test_noalloc_matches_workspace_entry_point_twice(order, generic):
    for N, seed in order:
        m, b = _system(N, seed)
        pd = DICPreconditioner(m).precond_diag
        xr, itr, resr, hr = _solve(m, b, pd, noalloc=False, generic=generic)
        assert itr > 1
        for _ in range(2):
            x, it, res, h = _solve(m, b, pd, noalloc=True, generic=generic)
            # the same three kernels on the same grid in the same order
            assert it == itr
            assert np.array_equal(_bits(x), _bits(xr))
            assert np.array_equal(_bits(h), _bits(hr))
            assert _bits(np.float64(res)) == _bits(np.float64(resr))


def test_noalloc_variant_zero_runs_the_three_kernel_form():
    m, b = _system(24, 3)
    pd = DICPreconditioner(m).precond_diag
    xr, itr, _, hr = _solve(m, b, pd, noalloc=False, variant=1)
    x, it, _, h = _solve(m, b, pd, noalloc=True, variant=0)
    assert it == itr and np.array_equal(_bits(x), _bits(xr)) and np.array_equal(_bits(h), _bits(hr))


@pytest.mark.parametrize("variant", [2, -1, 3])
def test_noalloc_refuses_other_variants(variant):
    m, b = _system(8, 1)
    pd = DICPreconditioner(m).precond_diag
    with pytest.raises(_lib.GbfError, match="variant must be 0 or 1"):
        _solve(m, b, pd, noalloc=True, variant=variant, max_iter=5)


def test_noalloc_refuses_systems_beyond_its_scratch():
    n = MAX_CELLS + 1
    own = torch.arange(n - 1)
    m = LduMatrix(n, own, own + 1, device="cuda")
    m.diag = torch.full((n,), 4.0, dtype=torch.float64)
    m.lower = torch.full((n - 1,), -1.0, dtype=torch.float64)
    m.upper = torch.full((n - 1,), -1.0, dtype=torch.float64)
    b = torch.ones(n, dtype=torch.float64, device="cuda")
    pd = m.diag.clone()
    with pytest.raises(_lib.GbfError, match="exceed the fixed scratch limit"):
        _solve(m, b, pd, noalloc=True, max_iter=5)
