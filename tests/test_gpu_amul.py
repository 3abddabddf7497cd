"""Amul / Ax_T parity on the GPU: bitwise against the reference's golden
outputs and against the oracle, through the C ABI (LduMatrix -> ctypes ->
gbf_amul_*)."""

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyopenfoam_gb300 import LduMatrix
from tests.golden.cases import FIXTURE, hex_faces, random_ldu, sha

pytestmark = pytest.mark.gpu
G = np.load(FIXTURE)
DEV = "cuda"


def mat(n, own, nei, diag, lower, upper, dtype=torch.float64):
    m = LduMatrix(n, torch.as_tensor(np.asarray(own)), torch.as_tensor(np.asarray(nei)),
                  device=DEV, dtype=dtype)
    m.diag = torch.as_tensor(np.asarray(diag, np.float64))
    m.lower = torch.as_tensor(np.asarray(lower, np.float64))
    m.upper = torch.as_tensor(np.asarray(upper, np.float64))
    return m


def bits(a):
    return np.asarray(a).view(np.int64)


@pytest.mark.parametrize(
    "n,own,nei,diag,lower,upper,x,expect",
    [
        (2, [0], [1], [3.0, 5.0], [0.0], [0.0], [2.0, 4.0], [6.0, 20.0]),
        (2, [0], [1], [2.0, 2.0], [-1.0], [-1.0], [1.0, 1.0], [1.0, 1.0]),
        (2, [0], [1], [4.0, 4.0], [-1.0], [-2.0], [1.0, 3.0], [1.0, 10.0]),
        (3, [0, 1], [1, 2], [4.0, 6.0, 4.0], [-1.0, -1.0], [-1.0, -1.0], [1.0, 2.0, 3.0],
         [2.0, 8.0, 10.0]),
        (3, [0, 1], [1, 2], [1.0, 2.0, 1.0], [-1.0, -1.0], [-1.0, -1.0], [1.0, 2.0, 3.0],
         [-1.0, 0.0, 1.0]),
    ],
)
def test_reference_known_answers(n, own, nei, diag, lower, upper, x, expect):
    m = mat(n, own, nei, diag, lower, upper)
    y = m.Ax(torch.tensor(x, dtype=torch.float64))
    assert y.device.type == "cuda" and y.dtype == torch.float64
    np.testing.assert_array_equal(y.cpu().numpy(), np.array(expect))


def test_zero_matrix_and_identity():
    m = LduMatrix(2, torch.tensor([0]), torch.tensor([1]), device=DEV)
    y = m.Ax(torch.tensor([5.0, 7.0], dtype=torch.float64))
    assert torch.equal(y.cpu(), torch.zeros(2, dtype=torch.float64))
    e = LduMatrix(3, torch.tensor([], dtype=torch.int64), torch.tensor([], dtype=torch.int64),
                  device=DEV)
    e.diag = torch.tensor([1.0, 2.0, 3.0], dtype=torch.float64)
    y = e.Ax(torch.tensor([1.0, -0.0, 2.0], dtype=torch.float64)).cpu().numpy()
    ref = O.amul([], [], [1.0, 2.0, 3.0], [], [], [1.0, -0.0, 2.0])
    assert (bits(y) == bits(ref)).all()  # -0.0 kept when there are no faces


def test_empty_matrix():
    m = LduMatrix(0, torch.tensor([], dtype=torch.int64), torch.tensor([], dtype=torch.int64),
                  device=DEV)
    assert m.Ax(torch.zeros(0, dtype=torch.float64)).shape == (0,)


@pytest.mark.parametrize("name,N,perm", [("ldu32", 32, False), ("ldu12p", 12, True)])
def test_bitwise_against_reference_golden(name, N, perm):
    c = random_ldu(N, 5, perm)
    m = mat(c["n"], c["owner"], c["neighbour"], c["diag"], c["lower"], c["upper"])
    x = torch.as_tensor(c["x"])
    assert sha(m.Ax(x).cpu().numpy()) == str(G[f"{name}_Ax_sha"])
    assert sha(m.Ax_T(x).cpu().numpy()) == str(G[f"{name}_AxT_sha"])
    m32 = mat(c["n"], c["owner"], c["neighbour"], c["diag"], c["lower"], c["upper"],
              torch.float32)
    y32 = m32.Ax(x.float())
    assert y32.dtype == torch.float64  # reference: float64 scatter accumulation
    assert sha(y32.cpu().numpy()) == str(G[f"{name}_Ax_f32_sha"])


def test_signed_zeros_and_in_place_edits_match_oracle():
    n, own, nei = hex_faces(5)
    rng = np.random.default_rng(11)
    F = own.shape[0]
    lower = rng.choice([-1.0, 0.0, -0.0, 2.5], F)
    upper = rng.choice([-1.0, 0.0, -0.0, 3.0], F)
    diag = rng.choice([1.0, -0.0, 0.0], n)
    x = rng.choice([0.0, -0.0, 1.5, -2.0], n)
    m = mat(n, own, nei, diag, lower, upper)
    y = m.Ax(torch.as_tensor(x)).cpu().numpy()
    assert (bits(y) == bits(O.amul(own, nei, diag, lower, upper, x))).all()
    # in-place edit without invalidate_cache(): the packed copy follows the
    # version counter
    m.lower.mul_(2.0)
    y2 = m.Ax(torch.as_tensor(x)).cpu().numpy()
    assert (bits(y2) == bits(O.amul(own, nei, diag, 2.0 * lower, upper, x))).all()


def test_float32_inner_amul_matches_float_oracle():
    from pyopenfoam_gb300 import _lib

    c = random_ldu(9, 7, True)
    m = mat(c["n"], c["owner"], c["neighbour"], c["diag"], c["lower"], c["upper"])
    coef32 = m.packed(dtype=torch.float32)
    d32 = m.diag.float()
    x32 = torch.as_tensor(c["x"]).float().cuda()
    y = torch.empty(c["n"], device=DEV, dtype=torch.float32)
    topo = m.topology()
    _lib.check(_lib.lib().gbf_amul_f32(topo.layout_ref, coef32.data_ptr(), d32.data_ptr(),
                                       x32.data_ptr(), y.data_ptr(), 0,
                                       torch.cuda.current_stream().cuda_stream))
    ref = O.amul(c["owner"], c["neighbour"], c["diag"].astype(np.float32),
                 c["lower"].astype(np.float32), c["upper"].astype(np.float32),
                 c["x"].astype(np.float32), float_accumulate=True)
    np.testing.assert_array_equal(y.cpu().numpy(), ref)


def test_argument_errors_like_reference():
    m = mat(3, [0, 1], [1, 2], [1.0, 2.0, 1.0], [-1.0, -1.0], [-1.0, -1.0])
    with pytest.raises(TypeError):
        m.Ax(torch.tensor([1, 2, 3]))
    with pytest.raises(ValueError):
        m.Ax(torch.ones(4, dtype=torch.float64))


@pytest.mark.parametrize("N", [128, 256])
def test_full_size_bitwise_against_oracle(N):
    """128^3 and 256^3: every cell of A x equals the oracle's (threaded
    per-cell gather in reference order) bit for bit."""
    n, own, nei = hex_faces(N)
    rng = np.random.default_rng(N)
    F = own.shape[0]
    lower = rng.uniform(-1, 0, F)
    upper = rng.uniform(-1, 0, F)
    diag = rng.uniform(6, 7, n)
    x = rng.uniform(-1, 1, n)
    m = mat(n, own, nei, diag, lower, upper)
    y = m.Ax(torch.as_tensor(x)).cpu().numpy()
    ref = O.amul(own, nei, diag, lower, upper, x)
    assert (bits(y) == bits(ref)).all()


def test_offset_compression_gives_identical_bits():
    from pyopenfoam_gb300 import _lib

    for perm in (False, True):
        c = random_ldu(20, 13, perm)
        m = mat(c["n"], c["owner"], c["neighbour"], c["diag"], c["lower"], c["upper"])
        topo = m.topology()
        x = torch.as_tensor(c["x"]).cuda()
        y1 = m.Ax(x)
        plain = topo.uncompressed_layout()
        y2 = torch.empty_like(y1)
        import ctypes

        _lib.check(_lib.lib().gbf_amul_f64(ctypes.byref(plain), m.packed().data_ptr(),
                                           m.diag.data_ptr(), x.data_ptr(), y2.data_ptr(), 0,
                                           torch.cuda.current_stream().cuda_stream))
        assert (bits(y1.cpu().numpy()) == bits(y2.cpu().numpy())).all()
        # and through slice_off / slice_w instead of the fixed-width arithmetic
        var = topo.variable_width_layout()
        y3 = torch.empty_like(y1)
        _lib.check(_lib.lib().gbf_amul_f64(ctypes.byref(var), m.packed().data_ptr(),
                                           m.diag.data_ptr(), x.data_ptr(), y3.data_ptr(), 0,
                                           torch.cuda.current_stream().cuda_stream))
        assert (bits(y1.cpu().numpy()) == bits(y3.cpu().numpy())).all()
        if not perm:
            # y1 came through the fixed-width (3 + 3 slot) hex gather, y2 and
            # y3 through the generic one
            assert topo.uniform and topo.n_uniform_entries == topo.n_slots // 32
            assert topo.layout.all_uniform == 1
            assert (topo.layout.uniform_wo, topo.layout.uniform_wn) == (3, 3)
        else:
            assert topo.layout.all_uniform == 0


@pytest.mark.parametrize("N", [20, 64])
def test_staged_float32_amul_matches_generic_gather(N):
    """The FP32 hex Amul with bulk-copy staging (N^3 = 8000 cells leaves a
    partial 64-cell tile, 64^3 is whole tiles) gives the same bits as the
    generic per-slot gather and as the float oracle, forward and transposed,
    float and float64 accumulation; no bounded wait ran out."""
    import ctypes

    from pyopenfoam_gb300 import _lib

    c = random_ldu(N, 17, False)
    m = mat(c["n"], c["owner"], c["neighbour"], c["diag"], c["lower"], c["upper"])
    topo = m.topology()
    assert topo.layout.all_uniform == 1
    L = _lib.lib()
    st = torch.cuda.current_stream().cuda_stream
    d32 = m.diag.float().contiguous()
    x32 = torch.as_tensor(c["x"]).float().cuda()
    var = topo.variable_width_layout()
    for transposed in (False, True):
        coef32 = m.packed(transposed=transposed, dtype=torch.float32)
        for fn, dt in ((L.gbf_amul_f32, torch.float32), (L.gbf_amul_f32_f64out, torch.float64)):
            y1 = torch.empty(c["n"], device=DEV, dtype=dt)
            y2 = torch.empty_like(y1)
            _lib.check(fn(topo.layout_ref, coef32.data_ptr(), d32.data_ptr(), x32.data_ptr(),
                          y1.data_ptr(), int(transposed), st))
            _lib.check(fn(ctypes.byref(var), coef32.data_ptr(), d32.data_ptr(), x32.data_ptr(),
                          y2.data_ptr(), int(transposed), st))
            a, b = y1.cpu().numpy(), y2.cpu().numpy()
            assert (a.view(np.uint8) == b.view(np.uint8)).all()
        if not transposed:
            ref = O.amul(c["owner"], c["neighbour"], c["diag"].astype(np.float32),
                         c["lower"].astype(np.float32), c["upper"].astype(np.float32),
                         c["x"].astype(np.float32), float_accumulate=True)
            y = torch.empty(c["n"], device=DEV, dtype=torch.float32)
            _lib.check(L.gbf_amul_f32(topo.layout_ref, coef32.data_ptr(), d32.data_ptr(),
                                      x32.data_ptr(), y.data_ptr(), 0, st))
            np.testing.assert_array_equal(y.cpu().numpy(), ref)
    fault = ctypes.c_int32(-1)
    _lib.check(L.gbf_stream_fault(ctypes.byref(fault)))
    assert fault.value == 0


@pytest.mark.parametrize("N", [7, 20, 32, 64])
def test_symmetric_half_storage_amul_matches_full_packing(N):
    """A symmetric matrix (lower == upper) stored as its owner-side half:
    gbf_amul_sym_f32 -- staged (aligned) and global-memory (unaligned x)
    paths -- gives the bits of gbf_amul_f32 on the full packing and of the
    float oracle; a non-symmetric matrix is refused by the packing.  N = 32
    and 64 put the y and z mirror coefficients in whole earlier slices
    (staged as 128-byte runs); N = 7 and 20 leave them to the gathers."""
    import ctypes

    from pyopenfoam_gb300 import _lib

    c = random_ldu(N, 23, False)
    m = mat(c["n"], c["owner"], c["neighbour"], c["diag"], c["lower"], c["lower"])
    topo = m.topology()
    assert topo.symmetric_storage
    half = m.packed_sym32()
    assert half is not None and half.numel() == topo.n_slots // 2
    full = m.packed(dtype=torch.float32)
    L = _lib.lib()
    st = torch.cuda.current_stream().cuda_stream
    n = c["n"]
    d32 = m.diag.float().contiguous()
    xa = torch.as_tensor(c["x"]).float().to(DEV)  # 16-byte aligned
    xbuf = torch.zeros(n + 4, device=DEV, dtype=torch.float32)
    xbuf[1:n + 1] = xa
    xu = xbuf[1:n + 1]  # the same values, 4 bytes off alignment
    y_full = torch.empty(n, device=DEV, dtype=torch.float32)
    _lib.check(L.gbf_amul_f32(topo.layout_ref, full.data_ptr(), d32.data_ptr(), xa.data_ptr(),
                              y_full.data_ptr(), 0, st))
    for x in (xa, xu):
        y = torch.empty(n, device=DEV, dtype=torch.float32)
        for _ in range(2):
            _lib.check(L.gbf_amul_sym_f32(topo.layout_ref, half.data_ptr(), d32.data_ptr(),
                                          x.data_ptr(), y.data_ptr(), st))
            a, b = y.cpu().numpy(), y_full.cpu().numpy()
            assert (a.view(np.uint32) == b.view(np.uint32)).all()
    ref = O.amul(c["owner"], c["neighbour"], c["diag"].astype(np.float32),
                 c["lower"].astype(np.float32), c["lower"].astype(np.float32),
                 c["x"].astype(np.float32), float_accumulate=True)
    np.testing.assert_array_equal(y_full.cpu().numpy(), ref)
    fault = ctypes.c_int32(-1)
    _lib.check(L.gbf_stream_fault(ctypes.byref(fault)))
    assert fault.value == 0
    # lower != upper in one face: no half storage
    m.upper = torch.as_tensor(c["lower"]).clone()
    up = m.upper.clone()
    up[5] = up[5] * 0.5
    m.upper = up
    assert m.packed_sym32() is None
    # -0.0 vs +0.0 differ in bits: not symmetric for the packing either
    lo = torch.zeros_like(up)
    m.lower, m.upper = lo, -lo
    assert m.packed_sym32() is None
