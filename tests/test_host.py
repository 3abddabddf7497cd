"""Host-side checks that need no GPU: the C-ABI library loads and exports
every entry point of include/gbfoam.h, the host topology passes (slot
layout, DIC/DILU wavefront schedules) are correct, and the Python surface
validates arguments like the reference."""

import ctypes
import os
import re

import numpy as np
import pytest

from pyopenfoam_gb300 import _lib
from pyopenfoam_gb300.solvers.residual import ResidualMonitor
from tests.golden.cases import hex_faces, random_ldu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        txt = open(os.path.join(ROOT, "include", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(gbf_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    declared = _declared()
    assert declared, "no declarations found"
    for name in sorted(declared):
        assert hasattr(L, name), f"libgbfoam.so does not export {name}"
    # and the ctypes table binds exactly the declared surface
    assert declared == set(_lib.EXPORTED), declared ^ set(_lib.EXPORTED)
    assert L.gbf_version() >= 1


def _declared_arity():
    """Parameter count of every gbf_* function the headers declare."""
    out = {}
    for fn in os.listdir(os.path.join(ROOT, "include")):
        txt = open(os.path.join(ROOT, "include", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        for m in re.finditer(r"\b(gbf_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt):
            params = m.group(2).strip()
            out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_argument_counts_match_the_headers():
    """Every ctypes binding passes as many arguments as its C declaration
    takes (an ABI change in the header without the binding, or the reverse,
    fails here rather than as a wrong call on the GPU)."""
    arity = _declared_arity()
    assert set(arity) == set(_lib.EXPORTED), set(arity) ^ set(_lib.EXPORTED)
    bad = {k: (arity[k], len(v[1])) for k, v in _lib.EXPORTED.items() if len(v[1]) != arity[k]}
    assert not bad, bad


def _layout(n, own, nei, pad=-1):
    L = _lib.lib()
    o = np.ascontiguousarray(own, np.int32)
    q = np.ascontiguousarray(nei, np.int32)
    ns, nsl, mw, uni = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
    _lib.check(L.gbf_layout_plan(n, o.shape[0], o.ctypes.data, q.ctypes.data, pad,
                                 ctypes.byref(ns), ctypes.byref(nsl), ctypes.byref(mw),
                                 ctypes.byref(uni)))
    off = np.empty(ns.value + 1, np.int32)
    w = np.empty(max(ns.value, 1), np.int32)
    col = np.empty(max(nsl.value, 1), np.int32)
    face = np.empty(max(nsl.value, 1), np.int32)
    _lib.check(L.gbf_layout_fill(n, o.shape[0], o.ctypes.data, q.ctypes.data, pad,
                                 off.ctypes.data, w.ctypes.data, col.ctypes.data,
                                 face.ctypes.data))
    return off, w, col[: nsl.value], face[: nsl.value], mw.value


@pytest.mark.parametrize("perm,pad", [(False, -1), (True, -1), (False, 50), (True, 50)])
def test_layout_slots_follow_reference_face_order(perm, pad):
    c = random_ldu(7, seed=3, permute_faces=perm)
    n, own, nei = c["n"], c["owner"], c["neighbour"]
    off, w, col, face, mw = _layout(n, own, nei, pad)
    if pad >= 0 and not perm:
        assert len(set(w.tolist())) == 1  # uniform widths
        assert all(off[s] == 32 * s * ((w[0] & 0xFFFF) + (w[0] >> 16)) for s in range(len(w)))
    seen_own = np.zeros(own.shape[0], int)
    seen_nei = np.zeros(own.shape[0], int)
    for cell in range(n):
        s, lane = cell >> 5, cell & 31
        wo, wn = w[s] & 0xFFFF, w[s] >> 16
        base = off[s] + lane
        ofaces = [face[base + 32 * k] for k in range(wo) if col[base + 32 * k] >= 0]
        nfaces = [face[base + 32 * (wo + k)] for k in range(wn) if col[base + 32 * (wo + k)] >= 0]
        # owner-side: faces with owner == cell in ascending face order (the
        # reference scatter order); neighbour-side likewise
        assert ofaces == sorted(np.flatnonzero(own == cell).tolist())
        assert nfaces == sorted(np.flatnonzero(nei == cell).tolist())
        for k in range(wo):
            f = face[base + 32 * k]
            if f >= 0:
                assert col[base + 32 * k] == nei[f]
                seen_own[f] += 1
        for k in range(wn):
            f = face[base + 32 * (wo + k)]
            if f >= 0:
                assert col[base + 32 * (wo + k)] == own[f]
                seen_nei[f] += 1
        # holes (col = -1) carry no face
        assert all((col[base + 32 * k] < 0) == (face[base + 32 * k] < 0) for k in range(wo + wn))
    assert (seen_own == 1).all() and (seen_nei == 1).all()
    assert mw == max(((x & 0xFFFF) + (x >> 16)) for x in w)


def _schedule(fn, n, own, nei, n_items):
    o = np.ascontiguousarray(own, np.int32)
    q = np.ascontiguousarray(nei, np.int32)
    ptr = np.empty(n_items + 1, np.int32)
    items = np.empty(max(n_items, 1), np.int32)
    nl, mx = ctypes.c_int32(), ctypes.c_int32()
    _lib.check(fn(n, o.shape[0], o.ctypes.data, q.ctypes.data, ptr.ctypes.data,
                  items.ctypes.data, ctypes.byref(nl), ctypes.byref(mx)))
    lvl = np.empty(n_items, int)
    for l in range(nl.value):
        lvl[items[ptr[l]:ptr[l + 1]]] = l
        assert list(items[ptr[l]:ptr[l + 1]]) == sorted(items[ptr[l]:ptr[l + 1]])
    assert mx.value == max(np.diff(ptr[: nl.value + 1]))
    return lvl, nl.value


@pytest.mark.parametrize("perm", [False, True])
def test_dic_schedule_respects_reference_dependencies(perm):
    c = random_ldu(6, seed=4, permute_faces=perm)
    n, own, nei = c["n"], c["owner"], c["neighbour"]
    lvl, nl = _schedule(_lib.lib().gbf_dic_schedule, n, own, nei, n)
    # cell i reads the factored d[j] of every lower neighbour j < i
    for f in range(own.shape[0]):
        i, j = nei[f], own[f]
        if j < i:
            assert lvl[i] > lvl[j]
    if not perm:
        N = 6
        ijk = np.arange(n)
        assert (lvl == ijk % N + (ijk // N) % N + ijk // (N * N)).all()
        assert nl == 3 * N - 2


@pytest.mark.parametrize("perm", [False, True])
def test_dilu_schedule_respects_face_order(perm):
    c = random_ldu(5, seed=6, permute_faces=perm)
    n, own, nei = c["n"], c["owner"], c["neighbour"]
    lvl, _ = _schedule(_lib.lib().gbf_dilu_schedule, n, own, nei, own.shape[0])
    last = {}
    for f in range(own.shape[0]):
        for cell in (own[f], nei[f]):
            if cell in last:
                assert lvl[f] > lvl[last[cell]]
            last[cell] = f


def _flow_links(n, own, nei, items):
    o = np.ascontiguousarray(own, np.int32)
    q = np.ascontiguousarray(nei, np.int32)
    it = np.ascontiguousarray(items, np.int32)
    prev = np.empty(max(2 * o.shape[0], 1), np.int32)
    last = np.empty(max(n, 1), np.int32)
    rc = _lib.lib().gbf_dilu_flow_links(n, o.shape[0], o.ctypes.data, q.ctypes.data,
                                        it.ctypes.data, prev.ctypes.data, last.ctypes.data)
    return rc, prev, last


@pytest.mark.parametrize("perm", [False, True])
def test_dilu_flow_links_name_the_previous_face_of_each_end(perm):
    """Slot links of the dataflow DILU walk against a plain restatement of
    the sequential face loop (preconditioners.py:254-268): item i's owner
    and neighbour read the slot written by the previous face touching that
    cell in face order, and cell_last names each cell's last face."""
    c = random_ldu(5, seed=8, permute_faces=perm)
    n, own, nei = c["n"], c["owner"], c["neighbour"]
    nf = own.shape[0]
    o = np.ascontiguousarray(own, np.int32)
    q = np.ascontiguousarray(nei, np.int32)
    ptr = np.empty(nf + 1, np.int32)
    items = np.empty(nf, np.int32)
    nl, mx = ctypes.c_int32(), ctypes.c_int32()
    _lib.check(_lib.lib().gbf_dilu_schedule(n, nf, o.ctypes.data, q.ctypes.data,
                                            ptr.ctypes.data, items.ctypes.data,
                                            ctypes.byref(nl), ctypes.byref(mx)))
    rc, prev, last = _flow_links(n, own, nei, items)
    assert rc == 0
    pos = np.empty(nf, int)
    pos[items] = np.arange(nf)
    expect_last = {}
    for f in range(nf):
        i = pos[f]
        for side, cell in ((0, own[f]), (1, nei[f])):
            want = expect_last.get(cell, -1)
            assert prev[2 * i + side] == want
            assert want < 0 or want // 2 < i  # an earlier item of the walk
            expect_last[cell] = 2 * i + side
    assert all(last[cl] == expect_last.get(cl, -1) for cl in range(n))
    # refusals: not a permutation; a face placed before one it reads
    bad = items.copy()
    bad[1] = bad[0]
    assert _flow_links(n, own, nei, bad)[0] != 0
    assert _flow_links(n, own, nei, np.arange(nf)[::-1].copy())[0] != 0


@pytest.mark.parametrize("perm,reverse,lower_only", [(False, 0, True), (True, 1, False),
                                                     (True, 0, False), (False, 1, True)])
def test_sweep_flow_links_name_the_last_writes(perm, reverse, lower_only):
    """Slot links of the dataflow triangular sweep against a plain
    restatement of the sequential face loop (preconditioners.py:170-201):
    each item reads the slot last written for its written cell and for its
    read cell, earlier in sweep order; a bad item list is refused."""
    c = random_ldu(5, seed=12, permute_faces=perm)
    n, own, nei = c["n"], c["owner"], c["neighbour"]
    nf = own.shape[0]
    o = np.ascontiguousarray(own, np.int32)
    q = np.ascontiguousarray(nei, np.int32)
    ptr = np.empty(nf + 1, np.int32)
    items = np.empty(nf, np.int32)
    nl, mx = ctypes.c_int32(), ctypes.c_int32()
    _lib.check(_lib.lib().gbf_sweep_schedule(n, nf, o.ctypes.data, q.ctypes.data, reverse,
                                             int(lower_only), ptr.ctypes.data, items.ctypes.data,
                                             ctypes.byref(nl), ctypes.byref(mx)))
    ni = int(ptr[nl.value])
    prev = np.empty(2 * ni, np.int32)
    last = np.empty(n, np.int32)
    _lib.check(_lib.lib().gbf_sweep_flow_links(n, nf, o.ctypes.data, q.ctypes.data, reverse, ni,
                                               items.ctypes.data, prev.ctypes.data,
                                               last.ctypes.data))
    pos = {int(f): i for i, f in enumerate(items[:ni])}
    lastw = {}
    order = range(nf - 1, -1, -1) if reverse else range(nf)
    for f in order:
        if f not in pos:
            assert lower_only and not own[f] < nei[f]
            continue
        i = pos[f]
        R, W = (nei[f], own[f]) if reverse else (own[f], nei[f])
        assert prev[2 * i] == lastw.get(W, -1) and prev[2 * i + 1] == lastw.get(R, -1)
        assert max(prev[2 * i], prev[2 * i + 1]) < i
        lastw[W] = i
    assert all(last[cl] == lastw.get(cl, -1) for cl in range(n))
    bad = items[:ni].copy()
    bad[1] = bad[0]
    assert _lib.lib().gbf_sweep_flow_links(n, nf, o.ctypes.data, q.ctypes.data, reverse, ni,
                                           bad.ctypes.data, prev.ctypes.data,
                                           last.ctypes.data) != 0


def test_topology_rejects_bad_addressing():
    L = _lib.lib()
    o = np.array([0, 5], np.int32)
    q = np.array([1, 2], np.int32)
    a, b, c_ = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
    rc = L.gbf_layout_plan(3, 2, o.ctypes.data, q.ctypes.data, 5, ctypes.byref(a),
                           ctypes.byref(b), ctypes.byref(c_), None)
    assert rc == 4 and b"outside" in L.gbf_last_error()
    o = np.array([1], np.int32)
    rc = L.gbf_layout_plan(3, 1, o.ctypes.data, o.ctypes.data, 5, ctypes.byref(a),
                           ctypes.byref(b), ctypes.byref(c_), None)
    assert rc == 4 and b"owner == neighbour" in L.gbf_last_error()


def test_layout_beyond_32bit_indices_is_refused():
    """A 1024^3 mesh has more slots than the kernels' 32-bit indices reach:
    the C ABI refuses it with an argument error before any CUDA call (the
    pointers below are never dereferenced)."""
    L = _lib.lib()
    n = 1 << 30
    lay = _lib.Layout(n_cells=n, n_faces=n, n_slices=(n + 31) // 32, max_width=6,
                      uniform_wo=3, uniform_wn=3, all_uniform=1, n_slots=6 * n,
                      slice_off=16, slice_w=16, slot_col=16, slot_face=16)
    rc = L.gbf_amul_f64(ctypes.byref(lay), 16, 16, 16, 16, 0, None)
    assert rc == 1 and b"32-bit" in L.gbf_last_error()


def test_python_surface_errors_without_gpu():
    import torch

    from pyopenfoam_gb300 import LduMatrix, PCGSolver, create_solver

    with pytest.raises(ValueError, match="CUDA"):
        LduMatrix(2, torch.tensor([0]), torch.tensor([1]), device="cpu")
    with pytest.raises(ValueError, match="Unknown solver"):
        create_solver("nope")
    assert isinstance(create_solver("pcg", tolerance=1e-8), PCGSolver)
    assert create_solver("PBiCGStab").__class__.__name__ == "PBiCGSTABSolver"
    with pytest.raises(ValueError, match="Unknown preconditioner"):
        PCGSolver(preconditioner="bogus")._make_preconditioner(None)
    from pyopenfoam_gb300 import PBiCGSTABSolver

    with pytest.raises(ValueError, match="omega"):
        PBiCGSTABSolver(omega="fast")


def test_residual_monitor_rules_match_reference():
    # residual.py:112-145: absolute OR relative, only from min_iter on
    m = ResidualMonitor(tolerance=1e-3, rel_tol=0.1, min_iter=2)
    assert not m.check(1.0, 0)
    assert not m.check(0.05, 1)      # below rel_tol but iteration < min_iter
    assert m.check(0.05, 2)
    info = m.build_info(True)
    assert info.iterations == 3 and info.final_residual == 0.05 and info.initial_residual == 1.0
    m = ResidualMonitor(tolerance=0.0, rel_tol=0.0)
    assert not m.check(0.0, 0)       # 0 < 0 is false; res0 = 0 skips the relative test


@pytest.mark.parametrize("perm", [False, True])
def test_layout_offset_compression_reproduces_columns(perm):
    c = random_ldu(9, seed=2, permute_faces=perm)
    n, own, nei = c["n"], c["owner"], c["neighbour"]
    off, w, col, face, mw = _layout(n, own, nei)
    ns = off.shape[0] - 1
    ne = max(col.shape[0] // 32, 1)
    dm = np.empty(2 * ne, np.int32)
    nu = ctypes.c_int64()
    _lib.check(_lib.lib().gbf_layout_compress(ns, off.ctypes.data, w.ctypes.data, col.ctypes.data,
                                              dm.ctypes.data, ctypes.byref(nu)))
    sd, sm = dm[0::2], dm[1::2].view(np.uint32)
    for s in range(ns):
        width = (w[s] & 0xFFFF) + (w[s] >> 16)
        for k in range(width):
            e = off[s] // 32 + k
            for lane in range(32):
                cell = 32 * s + lane
                ref = col[off[s] + 32 * k + lane]
                if sd[e] != np.iinfo(np.int32).min:
                    got = cell + sd[e] if (int(sm[e]) >> lane) & 1 else -1
                    assert got == ref
    if not perm:
        # structured numbering: every slot is one offset per slice
        assert nu.value == col.shape[0] // 32


@pytest.mark.parametrize("N", [32, 20, 16, 7])
def test_layout_mirror_maps_neighbour_slots_to_owner_slots(N):
    """Every neighbour-side slot of a hex layout points (offset + mirror
    slot) at the owner-side slot of the same face, which is what the
    symmetric half storage reads; irregular numberings report ok = 0."""
    n, own, nei = hex_faces(N)
    off, w, col, face, mw = _layout(n, own, nei, pad=5)
    ns = off.shape[0] - 1
    wo, wn = int(w[0] & 0xFFFF), int(w[0] >> 16)
    assert all(int(v) == int(w[0]) for v in w[:ns])  # uniform widths
    W = wo + wn
    ne = ns * W
    dm = np.empty(2 * ne, np.int32)
    nu = ctypes.c_int64()
    L = _lib.lib()
    _lib.check(L.gbf_layout_compress(ns, off.ctypes.data, w.ctypes.data, col.ctypes.data,
                                     dm.ctypes.data, ctypes.byref(nu)))
    assert nu.value == ne
    o32 = np.ascontiguousarray(own, np.int32)
    mir = np.empty(ne, np.int8)
    ok = ctypes.c_int32()
    _lib.check(L.gbf_layout_mirror(own.shape[0], ns, wo, wn, face.ctypes.data, o32.ctypes.data,
                                   dm.ctypes.data, mir.ctypes.data, ctypes.byref(ok)))
    pos_own = {}  # face -> (owner cell, owner-side slot j)
    for s in range(ns):
        for j in range(wo):
            for lane in range(32):
                f = face[32 * (s * W + j) + lane]
                if f >= 0:
                    pos_own[int(f)] = (32 * s + lane, j)
    uniform = True
    for s in range(ns):
        for k in range(wo, W):
            e = s * W + k
            js = set()
            for lane in range(32):
                f = face[32 * e + lane]
                if f < 0:
                    continue
                cell_o, j = pos_own[int(f)]
                assert cell_o == 32 * s + lane + dm[2 * e]
                js.add(j)
            if len(js) > 1:
                uniform = False
            elif js and ok.value:
                assert mir[e] == js.pop()
    assert ok.value == int(uniform)
    if N % 32 == 0:
        assert ok.value == 1
    # bad owner table: refused
    bad = o32.copy()
    bad[0] += 1
    _lib.check(L.gbf_layout_mirror(own.shape[0], ns, wo, wn, face.ctypes.data, bad.ctypes.data,
                                   dm.ctypes.data, mir.ctypes.data, ctypes.byref(ok)))
    assert ok.value == 0


def test_polymesh_reader_round_trip_and_mixed_faces(tmp_path):
    """ASCII polyMesh files: write, read back, compare (uniform quads take
    the reshape path, the prism mesh's triangles + quads the counted path);
    comments are skipped and binary files are refused."""
    from pyopenfoam_gb300.io import read_faces, read_mesh, write_mesh
    from pyopenfoam_gb300.io.mesh_io import BoundaryPatch
    from tests.golden.cases import hex_polymesh, prism_polymesh

    for tag, d in (("hex", hex_polymesh(3, 2, 2)), ("prism", prism_polymesh(2, 2, 1))):
        ptr, pts = d["face_ptr"], d["face_pts"]
        faces = [pts[ptr[i]:ptr[i + 1]] for i in range(ptr.shape[0] - 1)]
        patches = [BoundaryPatch(b["name"], b["type"], b["nFaces"], b["startFace"], ["g1"])
                   for b in d["boundary"]]
        out = tmp_path / tag
        write_mesh(out, d["points"], faces, d["owner"], d["neighbour"], patches)
        md = read_mesh(out)
        assert np.array_equal(md.points.numpy(), d["points"])
        assert np.array_equal(md.face_ptr, ptr) and np.array_equal(md.face_pts, pts)
        assert np.array_equal(md.owner.numpy(), d["owner"])
        assert np.array_equal(md.neighbour.numpy(), d["neighbour"])
        assert [(p.name, p.n_faces, p.start_face, p.in_groups) for p in md.boundary] == \
               [(b["name"], b["nFaces"], b["startFace"], ["g1"]) for b in d["boundary"]]
        assert md.n_cells == int(d["owner"].max()) + 1
    f = tmp_path / "faces_commented"
    f.write_text("/* c */\nFoamFile\n{\n format ascii;\n class faceList;\n}\n// x\n"
                 "2\n(\n3(0 1 2) // tri\n4(2 3 4 5)\n)\n")
    _, (p, q) = read_faces(f)
    assert p.tolist() == [0, 3, 7] and q.tolist() == [0, 1, 2, 2, 3, 4, 5]
    f.write_text("FoamFile\n{\n format binary;\n}\n2\n(\n)\n")
    with pytest.raises(ValueError):
        read_faces(f)
