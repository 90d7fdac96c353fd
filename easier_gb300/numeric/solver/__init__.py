from .cg import CG
from .gmres import GMRES
