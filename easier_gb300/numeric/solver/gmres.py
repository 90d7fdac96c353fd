"""Restarted GMRES, easier/numeric/solver/gmres.py.

``GMRES.solve`` runs every restart cycle as one CUDA graph of fused kernels
(``sparse.FusedGMRES``) when ``A`` is a compiled ``Linsys`` and ``M`` is None
or ``Jacobi``.  Any other operator or preconditioner runs
``gmres_per_op``: restarted, right-preconditioned GMRES as a loop over the
package's device ops, calling ``A`` and ``M`` as given.  Both stop on the
reference's test (gmres.py:222-266): the true residual norm at the start of
a cycle against max(rtol * ||b||, atol), counting cycles.
"""
from __future__ import annotations

import math
from typing import Any, Callable, Dict, Optional

import numpy as np
import torch
from torch import nn

from ... import module as esr
from ...utils import logger
from .cg import _Dots, _PlanCache

# an Arnoldi step whose new basis norm falls below this has found an
# invariant subspace: the cycle ends there (the reference's threshold)
BREAKDOWN = 1e-15


def _identity(x):
    return x


class _GivensLS:
    """min_y || beta e1 - H y || for the (j+2) x (j+1) Hessenberg matrices of
    one Arnoldi cycle, reduced to an upper triangle by one Givens rotation
    per column as the columns arrive (FP64, host)."""

    def __init__(self, m: int, beta: float) -> None:
        self.R = np.zeros((m + 1, m))
        self.g = np.zeros(m + 1)
        self.g[0] = beta
        self.cs = np.zeros(m)
        self.sn = np.zeros(m)
        self.k = 0

    def add_column(self, h: np.ndarray) -> None:
        """h: column j of H, entries 0..j+1."""
        j = self.k
        h = np.array(h, dtype=np.float64)
        for i in range(j):  # earlier rotations
            a, b = h[i], h[i + 1]
            h[i] = self.cs[i] * a + self.sn[i] * b
            h[i + 1] = -self.sn[i] * a + self.cs[i] * b
        a, b = h[j], h[j + 1]
        rho = math.hypot(a, b)
        c, s = (1.0, 0.0) if rho == 0.0 else (a / rho, b / rho)
        self.cs[j], self.sn[j] = c, s
        h[j], h[j + 1] = rho, 0.0
        self.R[: j + 2, j] = h[: j + 2]
        self.g[j + 1] = -s * self.g[j]
        self.g[j] = c * self.g[j]
        self.k = j + 1

    def solve(self) -> np.ndarray:
        """y of the columns added so far (back substitution; a zero pivot,
        which only an exactly singular H gives, contributes zero)."""
        k = self.k
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):
            t = self.g[i] - self.R[i, i + 1:k] @ y[i + 1:]
            y[i] = t / self.R[i, i] if self.R[i, i] != 0.0 else 0.0
        return y


def gmres_per_op(A: Callable, M: Callable, b: torch.Tensor, x: torch.Tensor, r: torch.Tensor, restart: int,
                 rtol: float, atol: Optional[float], maxiter: Optional[int],
                 on_cycle: Callable[[int, float], None] = lambda it, rn: None):
    """Restarted GMRES(restart) with right preconditioner ``M`` for any
    operator ``A`` (callables on device tensors of x's shape).

    Each cycle: r = b - A x and its norm (the stopping test: at most
    max(rtol * ||b||, atol), NaN never stops, or ``maxiter`` cycles done);
    then an orthonormal basis of the Krylov space of A M from r by modified
    Gram-Schmidt (FP64 dot products, basis rows contiguous in device
    memory), the least-squares problem reduced by Givens rotations on the
    host as each Hessenberg column arrives, and x += M(V^T y).  ``x`` is
    updated in place, ``r`` holds the last residual.
    Returns (residual norm, ||b||, cycles)."""
    dot = _Dots(x)
    n = x.numel()
    bnorm = float(dot(b, b).sqrt())
    tol = rtol * bnorm
    if atol:
        tol = max(tol, atol)
    V = torch.empty((restart + 1, n), dtype=x.dtype, device=x.device)
    hcol = torch.empty(restart + 1, dtype=torch.float64, device=x.device)
    cycles = 0
    while True:
        r.copy_(b - A(x))
        beta = float(dot(r, r).sqrt())
        on_cycle(cycles, beta)
        if (beta == beta and beta <= tol) or (maxiter is not None and cycles >= maxiter):
            return beta, bnorm, cycles
        cycles += 1
        ls = _GivensLS(restart, beta)
        V[0].copy_(r.reshape(-1) / beta)
        for j in range(restart):
            w = A(M(V[j].view(x.shape))).reshape(-1).clone()
            for i in range(j + 1):
                hij = dot(V[i], w)
                hcol[i:i + 1].copy_(hij)
                w.sub_(hij.to(w.dtype) * V[i])
            hcol[j + 1:j + 2].copy_(dot(w, w).sqrt())
            col = hcol[: j + 2].cpu().numpy()
            ls.add_column(col)
            if col[j + 1] < BREAKDOWN:
                break
            if j + 1 < restart:
                V[j + 1].copy_(w / col[j + 1])
        y = torch.from_numpy(ls.solve()).to(device=x.device, dtype=x.dtype)
        dx = (y.unsqueeze(0) @ V[: ls.k]).view(x.shape)
        x.add_(M(dx))


class GMRES(esr.Module):
    """General Minimal Residual with restarts (gmres.py:139-266)."""

    def __init__(self, A: nn.Module, b: esr.Tensor, x: esr.Tensor, M: Optional[nn.Module] = None, restart=20):
        super().__init__()
        self.A, self.b, self.x = A, b, x
        self.M = M if M else _identity
        self.restart = restart
        self.r = esr.Tensor(esr.zeros_like(x), mode="partition")
        self.rnorm = esr.Tensor(torch.tensor([0.0], dtype=x.dtype, device=x.device), mode="replicate")
        self.bnorm = esr.Tensor(torch.tensor([0.0], dtype=x.dtype, device=x.device), mode="replicate")
        self._plans = _PlanCache()
        self._fused = None

    # ------------------------------------------------------------ fused --
    def fusable(self) -> bool:
        from ..linsys import Linsys
        from ..preconditioner.jacobi import Jacobi
        if not isinstance(self.A, Linsys) or not (self.M is _identity or isinstance(self.M, Jacobi)):
            return False
        A = self.A
        ok = (A.selector.easier_index_status == "rewritten" and A.reducer.easier_index_status == "rewritten"
              and self.x.easier_data_ready and self.b.easier_data_ready)
        return bool(ok) and self.x.is_cuda and self.x.dtype in (torch.float32, torch.float64) \
            and A.Ae.dtype == self.x.dtype and A.Av.dtype == self.x.dtype and self.x.dim() == 1 \
            and self.x.elempart is None and 1 <= self.restart <= 64

    def _fused_solver(self):
        from ..preconditioner.jacobi import Jacobi
        from ..sparse import FusedGMRES, SellMatrix
        jacobi = isinstance(self.M, Jacobi)
        self._fused = self._plans.get(
            (self.restart, jacobi), self.A,
            lambda: FusedGMRES(SellMatrix.from_linsys(self.A), self.restart, jacobi=jacobi))
        return self._fused

    def solve(self, rtol: float = 1e-5, atol: Optional[float] = None, maxiter: Optional[int] = None,
              debug_iter: Optional[int] = None, *, fused: Optional[bool] = None) -> Dict[str, Any]:
        """Solve to ``rnorm <= max(rtol*||b||, atol)`` (gmres.py:222-266),
        counting restart cycles.  With a compiled ``Linsys`` and ``M`` None
        or ``Jacobi`` every restart cycle runs as one CUDA graph of fused
        kernels (``fused=False`` forces ``gmres_per_op``)."""
        name = self.__class__.__name__

        def log(it, rn):
            if debug_iter is not None and it % debug_iter == 0:
                logger.info(f"{name} residual {rn} at the {it}-th iteration")
        use_fused = self.fusable() if fused is None else fused
        if use_fused:
            eng = self._fused_solver()
            s, iters = eng.solve(self.b.data, self.x.data, self.r.data, rtol, atol, maxiter, log)
            rnorm, bnorm = float(s.rnorm), float(s.bnorm)
        else:
            rnorm, bnorm, iters = gmres_per_op(self.A, self.M, self.b.data, self.x.data, self.r.data,
                                               self.restart, rtol, atol, maxiter, log)
        self.rnorm.data.fill_(rnorm)
        self.bnorm.data.fill_(bnorm)
        logger.info(f"{name} solver completed with residual {rnorm} at the {iters}-th iteration")
        return {"residual": rnorm, "iters": iters}
