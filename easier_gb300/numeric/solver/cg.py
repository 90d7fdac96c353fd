"""Conjugate gradient, easier/numeric/solver/cg.py.

``Init``/``Step``/``Update`` are the reference's three modules (cg.py:12-71)
and run on the per-op path for any operator ``A`` and preconditioner ``M``.
``CG.solve`` uses the fused PCG kernels instead when ``A`` is a compiled
``Linsys`` and ``M`` is None or ``Jacobi``: same iteration, same stopping
test (cg.py:130-161), evaluated on the device.
"""
from __future__ import annotations

from typing import Any, Dict, Optional

import torch
from torch import nn

from ... import module as esr
from ... import ops
from ...utils import logger
from ..linsys import Linsys
from ..preconditioner.jacobi import Jacobi


class Init(esr.Module):
    def __init__(self, A, b, x, M, r, z, p, bnorm) -> None:
        super().__init__()
        self.A, self.x, self.b, self.M = A, x, b, M
        self.r, self.z, self.p, self.bnorm = r, z, p, bnorm

    def forward(self):
        self.r[:] = self.b - self.A(self.x)
        self.z[:] = self.M(self.r)
        self.p[:] = self.z
        self.bnorm[:] = esr.norm(self.b).norm()


class Step(esr.Module):
    def __init__(self, A, x, r, z, p, rnorm, rzsum):
        super().__init__()
        self.A, self.x, self.p, self.r, self.z = A, x, p, r, z
        self.rnorm, self.rzsum = rnorm, rzsum

    def forward(self):
        Ap = self.A(self.p)
        rzsum = esr.sum(self.r * self.z).sum()
        alpha = rzsum / esr.sum(self.p * Ap).sum()
        r1 = self.r - alpha * Ap
        self.x.add_(alpha * self.p)
        self.rzsum[:] = rzsum
        self.r[:] = r1
        self.rnorm[:] = esr.norm(r1).norm()


class Update(esr.Module):
    def __init__(self, x, M, r, z, p, rzsum):
        super().__init__()
        self.x, self.M, self.r, self.z, self.p, self.rzsum = x, M, r, z, p, rzsum

    def forward(self):
        z1 = self.M(self.r)
        beta = esr.sum(self.r * z1).sum() / self.rzsum
        p1 = z1 + beta * self.p
        self.z[:] = z1
        self.p[:] = p1


def _identity(x):
    return x


class CG(esr.Module):
    """Conjugate Gradient (cg.py:74-137)."""

    def __init__(self, A: nn.Module, b: esr.Tensor, x: esr.Tensor, M: Optional[nn.Module] = None) -> None:
        super().__init__()
        self.A = A
        self.b = b
        self.x = x
        self.M = M if M else _identity
        self.r = esr.Tensor(esr.zeros_like(x), mode="partition")
        self.z = esr.Tensor(esr.zeros_like(x), mode="partition")
        self.p = esr.Tensor(esr.zeros_like(x), mode="partition")
        self.rzsum = esr.Tensor(torch.tensor([0.0], dtype=x.dtype, device=x.device), mode="replicate")
        self.rnorm = esr.Tensor(torch.tensor([0.0], dtype=x.dtype, device=x.device), mode="replicate")
        self.bnorm = esr.Tensor(torch.tensor([0.0], dtype=x.dtype, device=x.device), mode="replicate")
        self.init = Init(A, b, x, self.M, self.r, self.z, self.p, self.bnorm)
        self.step = Step(A, x, self.r, self.z, self.p, self.rnorm, self.rzsum)
        self.update = Update(x, self.M, self.r, self.z, self.p, self.rzsum)
        self._fused = None
        self._fused_key = None
        self.last_info: Dict[str, Any] = {}

    # ------------------------------------------------------------ fused --
    def fusable(self) -> bool:
        if not isinstance(self.A, Linsys):
            return False
        if not (self.M is _identity or isinstance(self.M, Jacobi)):
            return False
        A = self.A
        ok = (A.selector.easier_index_status == "rewritten" and A.reducer.easier_index_status == "rewritten"
              and self.x.easier_data_ready and self.b.easier_data_ready)
        return bool(ok) and self.x.is_cuda and self.x.dtype in (torch.float32, torch.float64) \
            and A.Ae.dtype == self.x.dtype and A.Av.dtype == self.x.dtype and self.x.dim() == 1 \
            and self.x.elempart is None

    def _fused_solver(self, precision: str):
        """The engine for `precision`: FP64 systems ('native' and 'df64') run
        on the batched lockstep engine as a batch of one (autotuned work
        shape, FP64-verified result); 'native' FP32 systems on FusedPCG;
        'mixed' on MixedPCG."""
        from ..sparse import FusedPCG, MixedPCG, SellMatrix
        A = self.A
        key = (precision, A.Ae.data.data_ptr(), A.Ae._version, A.Av.data.data_ptr(), A.Av._version)
        if self._fused is None or self._fused_key != key:
            jacobi = isinstance(self.M, Jacobi)
            if precision in ("mixed", "df64") and A.Av.dtype != torch.float64:
                raise ValueError(f"precision='{precision}' needs an FP64 system")
            if precision == "mixed":
                self._fused = MixedPCG(SellMatrix.from_linsys(A), jacobi=jacobi)
            elif precision == "df64" or A.Av.dtype == torch.float64:
                from ..batched import BatchedPCG, LinsysInstance
                n = A.Av.shape[0]
                inst = LinsysInstance(n, A.reducer.idx.detach().cpu().numpy(), A.selector.idx.detach().cpu().numpy(),
                                      A.Ae.data, A.Av.data, self.b.data)
                self._fused = BatchedPCG([inst], jacobi=jacobi, precision="df64" if precision == "df64" else "fp64",
                                         device=self.x.device)
                self._fused.autotune()
            else:
                self._fused = FusedPCG(SellMatrix.from_linsys(A), jacobi=jacobi)
            self._fused_key = key
        return self._fused

    def solve(self, rtol: float = 1e-5, atol: Optional[float] = None, maxiter: Optional[int] = None,
              debug_iter: Optional[int] = None, *, precision: str = "native",
              fused: Optional[bool] = None) -> Dict[str, Any]:
        """Solve to ``rnorm <= max(rtol*||b||, atol)`` (cg.py:130-161).

        ``precision='native'`` iterates in the system's dtype;
        ``'mixed'`` (FP64 systems) runs the SpMV on FP32 matrix values and an
        FP32 copy of p, keeps the vectors and dots in FP64, replaces the
        residual by the FP64 true residual every 32 iterations and stops on it;
        ``'df64'`` (FP64 systems) iterates in double-float arithmetic (FP32
        pairs, ~48 significand bits) and accepts the result only when the FP64
        true residual meets the tolerance (restarting from it otherwise).
        Returns ``{'residual', 'iters'}`` as the reference, plus
        ``'true_residual'`` (||b - A x||, FP64) on the fused path.
        """
        name = self.__class__.__name__
        use_fused = self.fusable() if fused is None else fused
        if use_fused and debug_iter is None:
            return self._solve_fused(rtol, atol, maxiter, precision)
        if precision != "native":
            raise ValueError(f"precision='{precision}' needs the fused path (Linsys operator, Jacobi or no preconditioner)")
        self.init()
        rtol_t = rtol * self.bnorm
        tol = torch.maximum(rtol_t, torch.as_tensor(atol, dtype=rtol_t.dtype, device=rtol_t.device)) \
            if atol else rtol_t
        iters = 0
        while True:
            self.step()
            if debug_iter is not None and iters % debug_iter == 0:
                logger.info(f"{name} residual {float(self.rnorm)} at the {iters}-th iteration")
            if (not torch.isnan(self.rnorm) and self.rnorm <= tol) or (maxiter is not None and iters >= maxiter):
                break
            iters += 1
            self.update()
        logger.info(f"{name} solver completed with residual {float(self.rnorm)} at the {iters}-th iteration")
        self.last_info = {"residual": float(self.rnorm), "iters": iters}
        return dict(self.last_info)

    def _solve_fused(self, rtol, atol, maxiter, precision) -> Dict[str, Any]:
        name = self.__class__.__name__
        from ..batched import BatchedPCG
        eng = self._fused_solver(precision)
        x, b = self.x.data, self.b.data
        if isinstance(eng, BatchedPCG):
            eng.load_instance(0, b=b, x0=x)
            [res] = eng.solve(rtol, atol, maxiter)
            x.copy_(eng.solution(0).to(x.dtype))
            rn = res["true_residual"]
            self.rnorm.data.fill_(res["residual"])
            self.bnorm.data.fill_(res["bnorm"])
            info = {"residual": res["residual"], "iters": res["iters"], "true_residual": rn,
                    "restarts": res["restarts"], "precision": precision, "status": res["status"]}
        elif precision == "mixed":
            s = eng.solve(b, x, self.r.data, self.z.data, self.p.data, rtol, atol, maxiter)
            rn = float(s.true_rr) ** 0.5
            self.rnorm.data.fill_(rn)
            self.bnorm.data.fill_(s.bnorm)
            info = {"residual": rn, "iters": max(s.iters - 1, 0), "true_residual": rn,
                    "replacements": s.replacements, "precision": "mixed",
                    "status": {1: "converged", 2: "maxiter", 3: "breakdown"}.get(s.done, "?")}
        else:
            s = eng.solve(b, x, self.r.data, self.z.data, self.p.data, rtol, atol, maxiter)
            rnorm = float(s.rr) ** 0.5
            iters = s.iters - 1
            self.rnorm.data.fill_(rnorm)
            self.bnorm.data.fill_(s.bnorm)
            self.rzsum.data.fill_(s.rz)
            true_res = eng.true_residual(b, x, self.q_scratch())
            info = {"residual": rnorm, "iters": iters, "true_residual": true_res, "precision": "native",
                    "status": {1: "converged", 2: "maxiter", 3: "breakdown"}.get(s.done, "?")}
        logger.info(f"{name} solver completed with residual {info['residual']} at the {info['iters']}-th iteration")
        self.last_info = info
        return dict(info)

    def q_scratch(self) -> torch.Tensor:
        if getattr(self, "_q_scratch", None) is None or self._q_scratch.shape != self.x.shape:
            self._q_scratch = torch.empty_like(self.x.data)
        return self._q_scratch
