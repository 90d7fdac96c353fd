"""Jacobi (diagonal) preconditioner for a Linsys."""
from torch import nn


class Jacobi(nn.Module):
    """``M(r) = r / Av``: an ``nn.Module`` holding the Linsys diagonal, usable
    as the ``M`` of CG / GMRES on the per-op path; the fused solvers
    recognise it and apply ``r * (1 / Av)`` inside their update kernel."""

    def __init__(self, A) -> None:
        super().__init__()
        self.Av = A.Av

    def forward(self, r):
        return r / self.Av
