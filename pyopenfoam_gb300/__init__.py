"""pyopenfoam_gb300 -- pyOpenFOAM's linear-solve hot path on GB300 (sm_103a).

Drop-in classes with the reference's signatures (``pyfoam.core.LduMatrix``,
``FvMatrix``, ``pyfoam.solvers.PCGSolver`` / ``PBiCGSTABSolver`` / DIC / DILU,
``fvm.laplacian``, ``DifferentiableLinearSolve``) backed by hand-written CUDA
kernels in ``libgbfoam.so`` reached through a C ABI (``include/gbfoam.h``).
"""

from .core import FvMatrix, LduMatrix
from .solvers import (DICPreconditioner, DILUPreconditioner, MixedPrecisionPBiCGSTABSolver,
                      MixedPrecisionPCGSolver, PBiCGSTABSolver, PCGSolver, create_solver,
                      solver_from_dict)

__all__ = ["LduMatrix", "FvMatrix", "PCGSolver", "PBiCGSTABSolver", "MixedPrecisionPCGSolver",
           "MixedPrecisionPBiCGSTABSolver", "DICPreconditioner", "DILUPreconditioner",
           "create_solver", "solver_from_dict"]

__version__ = "0.1.0"
