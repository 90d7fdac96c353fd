"""Restarted GMRES, easier/numeric/solver/gmres.py.

The Arnoldi process keeps the reference's structure (modified Gram-Schmidt
through small modules, Hessenberg least squares by SVD on the host,
gmres.py:12-266); every Linsys application, dot product and norm inside it
runs in the GB300 kernels.
"""
from __future__ import annotations

from typing import Any, Dict, Optional

import torch
from torch import nn

from ... import module as esr
from ...utils import logger


class UpdateRnorm(esr.Module):
    def __init__(self, A, b, x, r, rnorm):
        super().__init__()
        self.A, self.b, self.x, self.r, self.rnorm = A, b, x, r, rnorm

    def forward(self):
        r = self.b - self.A(self.x)
        self.r[:] = r
        self.rnorm[:] = esr.norm(r).norm()


class Init(esr.Module):
    def __init__(self, b, bnorm) -> None:
        super().__init__()
        self.b, self.bnorm = b, bnorm

    def forward(self) -> None:
        self.bnorm[:] = esr.norm(self.b).norm()


class InitV(esr.Module):
    def __init__(self, r, rnorm, V):
        super().__init__()
        self.r, self.rnorm, self.V = r, rnorm, V

    def forward(self):
        self.V[:, ..., 0] = self.r / self.rnorm


class InitW(esr.Module):
    def __init__(self, A, M, V, w):
        super().__init__()
        self.A, self.M, self.V, self.w = A, M, V, w
        self.j = esr.Tensor(torch.tensor([0], dtype=torch.int32, device=V.device), mode="replicate")

    def forward(self):
        self.w[:] = self.A(self.M(self.V[:, ..., self.j].squeeze(-1)))


class SumW(esr.Module):
    def __init__(self, V, w, h):
        super().__init__()
        self.V, self.w, self.h = V, w, h
        self.i = esr.Tensor(torch.tensor([0], dtype=torch.int32, device=V.device), mode="replicate")

    def forward(self):
        self.h[:] = esr.sum(self.V[:, ..., self.i].squeeze(-1) * self.w).sum()


class NormW(esr.Module):
    def __init__(self, w, h):
        super().__init__()
        self.w, self.h = w, h

    def forward(self):
        self.h[:] = esr.norm(self.w).norm()


class UpdateW(esr.Module):
    def __init__(self, V, w, h):
        super().__init__()
        self.V, self.w, self.h = V, w, h
        self.i = esr.Tensor(torch.tensor([0], dtype=torch.int32, device=V.device), mode="replicate")

    def forward(self):
        self.w.sub_(self.h * self.V[:, ..., self.i].squeeze(-1))


class UpdateV(esr.Module):
    def __init__(self, V, w, h):
        super().__init__()
        self.V, self.w, self.h = V, w, h
        self.i = esr.Tensor(torch.tensor([0], dtype=torch.int32, device=V.device), mode="replicate")

    def forward(self):
        self.V[:, ..., self.i] = (self.w / self.h)[:, ..., None]


class UpdateX(esr.Module):
    def __init__(self, x, V, M, y, i):
        super().__init__()
        self.x, self.V, self.M, self.y, self.i = x, V, M, y, i

    def forward(self):
        V = self.V[:, ..., :self.i]
        dx = torch.matmul(V, self.y[:self.i]).squeeze(dim=-1)
        self.x.add_(self.M(dx))


def _identity(x):
    return x


class GMRES(esr.Module):
    """General Minimal Residual with restarts (gmres.py:139-266)."""

    def __init__(self, A: nn.Module, b: esr.Tensor, x: esr.Tensor, M: Optional[nn.Module] = None, restart=20):
        super().__init__()
        self.A, self.b, self.x = A, b, x
        self.M = M if M else _identity
        self.restart = restart
        self.r = esr.Tensor(esr.zeros_like(x), mode="partition")
        self.rnorm = esr.Tensor(torch.tensor([0.0], dtype=x.dtype, device=x.device), mode="replicate")
        self.update_rnorm = UpdateRnorm(A, b, x, self.r, self.rnorm)
        self.bnorm = esr.Tensor(torch.tensor([0.0], dtype=x.dtype, device=x.device), mode="replicate")
        self.init = Init(self.b, self.bnorm)
        self.H = esr.Tensor(torch.zeros((restart + 1, restart), device=x.device, dtype=x.dtype), mode="replicate")
        self.B = esr.Tensor(torch.zeros((restart + 1, 1), device=x.device, dtype=x.dtype), mode="replicate")
        self.V = esr.Tensor(esr.zeros(tuple(x.shape) + (restart,), dtype=x.dtype, device=x.device), mode="partition")
        self.init_V = InitV(self.r, self.rnorm, self.V)
        self.w = esr.Tensor(esr.zeros_like(x), mode="partition")
        self.init_w = InitW(A, self.M, self.V, self.w)
        self.h = esr.Tensor(torch.tensor([0.0], dtype=x.dtype, device=x.device), mode="replicate")
        self.sum_w = SumW(self.V, self.w, self.h)
        self.update_w = UpdateW(self.V, self.w, self.h)
        self.norm_w = NormW(self.w, self.h)
        self.update_V = UpdateV(self.V, self.w, self.h)
        self.y = esr.Tensor(torch.zeros((restart, 1), dtype=x.dtype, device=x.device), mode="replicate")
        self.update_x = nn.ModuleList([UpdateX(self.x, self.V, self.M, self.y, i) for i in range(1, restart + 1)])

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
        A = self.A
        key = (A.Ae.data.data_ptr(), A.Ae._version, A.Av.data.data_ptr(), A.Av._version, self.restart)
        if getattr(self, "_fused", None) is None or self._fused_key != key:
            self._fused = FusedGMRES(SellMatrix.from_linsys(A), self.restart, jacobi=isinstance(self.M, Jacobi))
            self._fused_key = key
        return self._fused

    def solve(self, rtol: float = 1e-5, atol: Optional[float] = None, maxiter: Optional[int] = None,
              debug_iter: Optional[int] = None, *, fused: Optional[bool] = None) -> Dict[str, Any]:
        """Solve to ``rnorm <= max(rtol*||b||, atol)`` (gmres.py:222-266).
        With a compiled ``Linsys`` and ``M`` None or ``Jacobi`` every restart
        cycle runs as one CUDA graph of fused kernels (``fused=False``
        forces the per-op modules)."""
        name = self.__class__.__name__
        use_fused = self.fusable() if fused is None else fused
        if use_fused:
            eng = self._fused_solver()

            def log(it, rn):
                if debug_iter is not None and it % debug_iter == 0:
                    logger.info(f"{name} residual {rn} at the {it}-th iteration")
            s, iters = eng.solve(self.b.data, self.x.data, self.r.data, rtol, atol, maxiter, log)
            self.rnorm.data.fill_(s.rnorm)
            self.bnorm.data.fill_(s.bnorm)
            logger.info(f"{name} solver completed with residual {s.rnorm} at the {iters}-th iteration")
            return {"residual": float(s.rnorm), "iters": iters}
        self.init()
        rtol_t = rtol * self.bnorm
        tol = torch.maximum(rtol_t, torch.as_tensor(atol, dtype=rtol_t.dtype, device=rtol_t.device)) \
            if atol else rtol_t
        iters = 0
        while True:
            self.update_rnorm()
            if debug_iter is not None and iters % debug_iter == 0:
                logger.info(f"{name} residual {float(self.rnorm)} at the {iters}-th iteration")
            if (not torch.isnan(self.rnorm) and self.rnorm <= tol) or (maxiter is not None and iters >= maxiter):
                break
            iters += 1
            self.B[0, 0] = self.rnorm
            self.init_V()
            for j in range(self.restart):
                self.init_w.j.fill_(j)
                self.init_w()
                for i in range(j + 1):
                    self.sum_w.i.fill_(i)
                    self.sum_w()
                    self.H[i, j] = self.h
                    self.update_w.i.fill_(i)
                    self.update_w()
                self.norm_w()
                self.H[j + 1, j] = self.h
                if self.h < 1e-15:
                    break
                elif j < self.restart - 1:
                    self.update_V.i.fill_(j + 1)
                    self.update_V()
            u, s, vt = torch.linalg.svd(self.H[:j + 2], full_matrices=False)
            self.y[:] = vt.transpose(0, 1) @ torch.diag_embed(1 / torch.clamp(s, min=1e-8)) @ \
                u.transpose(0, 1) @ self.B[:j + 2]
            self.update_x[j]()
        logger.info(f"{name} solver completed with residual {float(self.rnorm)} at the {iters}-th iteration")
        return {"residual": float(self.rnorm), "iters": iters}
