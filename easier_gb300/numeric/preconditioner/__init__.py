"""Preconditioners.  The reference ships none
(easier/numeric/preconditioner/__init__.py:4); Jacobi and the message-passing
GNN preconditioner are additions of this implementation."""
from .jacobi import Jacobi
