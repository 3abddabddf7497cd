"""The no-allocation PCG entry point (gbf_pcg_solve_f64_noalloc).

It exists for callers that cannot allocate device memory at the moment they
solve -- work being recorded into a stream capture, real-time loops that must
never wait on the allocator, programs with a fixed device-memory budget.  Its
scratch comes from a fixed file-scope device array, so this test calls it
straight through the C ABI (no torch workspace) and checks, on two calls in a
row, that it gives what the workspace entry point gives on the same input.

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


def _solve(m, b, pd, noalloc, max_iter=400, rel_tol=1e-9):
    L = _lib.lib()
    topo = m.topology()
    coef = m.packed()
    x = torch.zeros_like(b)
    hist = torch.zeros(max_iter + 1, dtype=torch.float64, device="cuda")
    P = _lib.SolveParams(0.0, rel_tol, max_iter, 0, 16, 0)
    R = _lib.SolveResult()
    stream = torch.cuda.current_stream().cuda_stream
    args = (topo.layout_ref, coef.data_ptr(), m.diag.data_ptr(), pd.data_ptr(), b.data_ptr(),
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


def test_noalloc_matches_workspace_entry_point_twice():
    # two different systems back to back: the second call must not see the
    # first call's leftovers in the shared scratch array
    for N, seed in ((24, 3), (40, 4)):
        m, b = _system(N, seed)
        pd = DICPreconditioner(m).precond_diag
        xr, itr, resr, hr = _solve(m, b, pd, noalloc=False)
        for _ in range(2):
            x, it, res, h = _solve(m, b, pd, noalloc=True)
            assert it == itr
            # same kernels, same grid, same order: the tolerance used across
            # this suite for FP64 PCG solutions is 1e-12 relative
            assert np.abs(x - xr).max() <= 1e-12 * np.abs(xr).max()
            assert abs(res - resr) <= 1e-12 * abs(resr)
            np.testing.assert_allclose(h, hr, rtol=1e-12, atol=0)


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
