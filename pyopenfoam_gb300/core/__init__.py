"""LDU storage and matrix-vector products on the GPU."""

from .dtype import CFD_DTYPE, INDEX_DTYPE, assert_floating
from .fv_matrix import FvMatrix, LinearSolver
from .ldu_matrix import LduMatrix
from .topology import Topology, get_topology

__all__ = ["LduMatrix", "FvMatrix", "LinearSolver", "Topology", "get_topology", "CFD_DTYPE",
           "INDEX_DTYPE", "assert_floating"]
