"""Dataflow DIC / DILU factorisations (gbf_dic_build_flow_f64,
gbf_dilu_build_flow_f64) against the level-scheduled walks and the oracle.

The dataflow walk drops the grid barrier between wavefront levels: each step
waits only on the slots it reads.  It applies the same subtractions in the
same order, so the bar is bitwise equality with the cooperative level walk,
the per-level launches and the oracle's sequential loop
(solvers/preconditioners.py:102-133 DIC, :228-272 DILU), on sorted and on
shuffled face orders (a third of the faces owner > neighbour), on a mesh
large enough that the walk spans many chunks per warp, and on the edge cases
of the reference loop: |d| <= 1e-30 (the subtraction is skipped), NaN, a
cell on no face, a matrix with no faces.  The failure path (a wait that can
never be satisfied) is exercised by a self-test on a cyclic link table: it
runs out after its pass limit and poisons the output, without a GPU fault.
"""

import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyopenfoam_gb300 import LduMatrix, _lib
from pyopenfoam_gb300.solvers.preconditioners import (DICPreconditioner, DILUPreconditioner,
                                                      FACTOR_FORMS, factor_dic, factor_dilu)
from tests.golden.cases import random_ldu

pytestmark = pytest.mark.gpu


def _matrix(c):
    m = LduMatrix(c["n"], torch.as_tensor(c["owner"]), torch.as_tensor(c["neighbour"]),
                  device="cuda")
    m.diag, m.lower, m.upper = (torch.as_tensor(c[k]) for k in ("diag", "lower", "upper"))
    return m


def _forms(m, kind):
    topo = m.topology()
    out = {}
    for form in FACTOR_FORMS:
        d = torch.empty(m.n_cells, dtype=torch.float64, device="cuda")
        if kind == "DIC":
            factor_dic(topo, m.packed(), m.diag, d, m.device, form)
        else:
            factor_dilu(topo, m.lower, m.upper, m.diag, d, m.device, form)
        out[form] = d.cpu().numpy()
    return out


def _oracle(c, kind):
    if kind == "DIC":
        return O.dic_build(c["owner"], c["neighbour"], c["diag"], c["upper"])
    return O.dilu_build(c["owner"], c["neighbour"], c["diag"], c["lower"], c["upper"])


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.int64)


@pytest.mark.parametrize("kind", ["DIC", "DILU"])
@pytest.mark.parametrize("N,perm", [(6, False), (12, True), (24, True), (40, False)])
def test_flow_factorisation_matches_level_walks_and_oracle(kind, N, perm):
    c = random_ldu(N, seed=40 + N, permute_faces=perm)
    m = _matrix(c)
    out = _forms(m, kind)
    ref = _oracle(c, kind)
    for form, d in out.items():
        assert np.array_equal(_bits(d), _bits(ref)), form


@pytest.mark.parametrize("kind", ["DIC", "DILU"])
def test_flow_factorisation_at_96cube(kind):
    """884,736 cells, 2.6M faces: 283 (DIC) / 849 (DILU) levels, every
    resident warp walking many chunks."""
    c = random_ldu(96, seed=3)
    m = _matrix(c)
    topo = m.topology()
    d = torch.empty(m.n_cells, dtype=torch.float64, device="cuda")
    if kind == "DIC":
        factor_dic(topo, m.packed(), m.diag, d, m.device, "flow")
    else:
        factor_dilu(topo, m.lower, m.upper, m.diag, d, m.device, "flow")
    assert np.array_equal(_bits(d.cpu().numpy()), _bits(_oracle(c, kind)))


@pytest.mark.parametrize("kind", ["DIC", "DILU"])
def test_flow_factorisation_edge_values(kind):
    """Tiny and zero pivots (|d| <= 1e-30 skips the subtraction, then the
    clamp), a NaN that propagates along the walk, and an infinite
    coefficient: the dataflow walk agrees with the oracle value for value
    (NaN where the oracle has NaN)."""
    c = random_ldu(8, seed=9, permute_faces=True)
    c["diag"] = c["diag"].copy()
    c["diag"][[0, 5, 17]] = [0.0, 1e-31, -2e-30]
    c["diag"][100] = np.nan
    c["upper"] = c["upper"].copy()
    c["upper"][7] = np.inf
    m = _matrix(c)
    out = _forms(m, kind)
    ref = _oracle(c, kind)
    for form, d in out.items():
        np.testing.assert_array_equal(d, ref, err_msg=form)


def test_flow_factorisation_without_faces():
    """A matrix with cells but no faces: the clamped |diag| (the level walks'
    result), including a cell whose diagonal is zero."""
    n = 5
    e = torch.zeros(0, dtype=torch.int64)
    m = LduMatrix(n, e, e, device="cuda")
    m.diag = torch.tensor([2.0, -3.0, 0.0, 1e-40, 7.0], dtype=torch.float64)
    m.lower = torch.zeros(0, dtype=torch.float64)
    m.upper = torch.zeros(0, dtype=torch.float64)
    want = np.maximum(np.abs(m.diag.cpu().numpy()), 1e-30)
    for cls in (DICPreconditioner, DILUPreconditioner):
        assert cls.factor_form == "flow"
        assert np.array_equal(cls(m).precond_diag.cpu().numpy(), want)


def test_flow_wait_timeout_poisons_the_output():
    """A cyclic link table (two faces each waiting on the other's slot) runs
    out after its pass limit, sets the fault word and the output becomes NaN;
    the context stays usable (a dataflow factorisation afterwards is exact)."""
    out = (ctypes.c_int32 * 2)()
    _lib.check(_lib.lib().gbf_selftest_flow_fault(out))
    assert list(out) == [1, 1]
    c = random_ldu(10, seed=2, permute_faces=True)
    m = _matrix(c)
    d = DILUPreconditioner(m).precond_diag.cpu().numpy()
    assert np.array_equal(_bits(d), _bits(_oracle(c, "DILU")))
