"""OpenFOAM file input/output of the mesh data the linear-solve path needs."""

from .mesh_io import *  # noqa: F401,F403
from .mesh_io import __all__  # noqa: F401
