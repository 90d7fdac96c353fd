"""easier.numeric counterpart: Linsys, solvers and preconditioners."""
from . import solver, preconditioner
from .linsys import Linsys
