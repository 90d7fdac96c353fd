"""Conjugate gradient, easier/numeric/solver/cg.py.

``CG.solve`` runs the fused PCG kernels when ``A`` is a compiled ``Linsys``
and ``M`` is None or ``Jacobi``: the reference's iteration and stopping test
(cg.py:130-161), evaluated on the device.  Any other operator or
preconditioner runs ``pcg_per_op``: the same iteration as a loop over the
package's device ops, calling ``A`` and ``M`` as given.
"""
from __future__ import annotations

from typing import Any, Callable, Dict, Optional

import torch
from torch import nn

from ... import _lib
from ... import module as esr
from ... import ops
from ...utils import logger
from ..linsys import Linsys
from ..preconditioner.jacobi import Jacobi


def _identity(x):
    return x


class _Dots:
    """FP64-accumulated dot products of one vector length (esr_dot), sharing
    one zeroed workspace (the kernel's arrival counter resets itself)."""

    def __init__(self, like: torch.Tensor) -> None:
        nbytes = int(_lib.lib().esr_dot_workspace_bytes(like.numel()))
        self.ws = torch.zeros(max(nbytes, 16), dtype=torch.uint8, device=like.device)

    def __call__(self, u: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
        return ops.dot(u.reshape(-1), v.reshape(-1), workspace=self.ws)


def pcg_per_op(A: Callable, M: Callable, b: torch.Tensor, x: torch.Tensor, r: torch.Tensor, z: torch.Tensor,
               p: torch.Tensor, rtol: float, atol: Optional[float], maxiter: Optional[int],
               on_iter: Callable[[int, float], None] = lambda it, rn: None):
    """Preconditioned CG for any operator ``A`` and preconditioner ``M``
    (callables on device tensors of x's shape), one device op at a time.

    Iteration and stopping test as the reference's (cg.py:74-137): after
    each update of x and r, stop when the recurrence residual norm is at
    most max(rtol * ||b||, atol) (a NaN norm never stops it) or the update
    count has reached ``maxiter``; otherwise precondition and form the next
    direction p = z + (r.z / r_old.z_old) p.  r.z is kept from one
    iteration to the next.  Dots accumulate in FP64; the scalars reach the
    vector updates in x's dtype.  ``x`` is updated in place and ``r``, ``z``,
    ``p`` hold the last residual, preconditioned residual and direction.
    Returns (residual norm, r.z, ||b||, update count)."""
    dot = _Dots(x)
    bnorm = float(dot(b, b).sqrt())
    tol = rtol * bnorm
    if atol:
        tol = max(tol, atol)
    r.copy_(b - A(x))
    z.copy_(M(r))
    p.copy_(z)
    rz = dot(r, z)
    it = 0
    while True:
        q = A(p)
        alpha = (rz / dot(p, q)).to(x.dtype)
        x.add_(alpha * p)
        r.sub_(alpha * q)
        rnorm = float(dot(r, r).sqrt())
        on_iter(it, rnorm)
        if (rnorm == rnorm and rnorm <= tol) or (maxiter is not None and it >= maxiter):
            return rnorm, float(rz), bnorm, it
        it += 1
        z.copy_(M(r))
        rz_next = dot(r, z)
        p.mul_((rz_next / rz).to(p.dtype)).add_(z)
        rz = rz_next


class _PlanCache:
    """The fused plan of a Linsys, kept while the operator's values are the
    ones it was built from.  The values are compared, not version counters:
    writes through ``tensor.data`` (the usual way to refill an esr.Tensor)
    leave the counters unchanged."""

    def __init__(self) -> None:
        self.plan = None
        self.key = None
        self.values = None

    def get(self, key, A, build):
        Ae, Av = A.Ae.data, A.Av.data
        same = (self.plan is not None and self.key == key and self.values is not None
                and self.values[0].shape == Ae.shape and self.values[1].shape == Av.shape
                and torch.equal(self.values[0], Ae) and torch.equal(self.values[1], Av))
        if not same:
            self.plan = build()
            self.key = key
            self.values = (Ae.clone(), Av.clone())
        return self.plan


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
        self._plans = _PlanCache()
        self._fused = None
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

        def build():
            jacobi = isinstance(self.M, Jacobi)
            if precision in ("mixed", "df64") and A.Av.dtype != torch.float64:
                raise ValueError(f"precision='{precision}' needs an FP64 system")
            if precision == "mixed":
                return MixedPCG(SellMatrix.from_linsys(A), jacobi=jacobi)
            if precision == "df64" or A.Av.dtype == torch.float64:
                from ..batched import BatchedPCG, LinsysInstance
                n = A.Av.shape[0]
                inst = LinsysInstance(n, A.reducer.idx.detach().cpu().numpy(), A.selector.idx.detach().cpu().numpy(),
                                      A.Ae.data, A.Av.data, self.b.data)
                eng = BatchedPCG([inst], jacobi=jacobi, precision="df64" if precision == "df64" else "fp64",
                                 device=self.x.device)
                eng.autotune()
                return eng
            return FusedPCG(SellMatrix.from_linsys(A), jacobi=jacobi)

        self._fused = self._plans.get((precision, isinstance(self.M, Jacobi)), A, build)
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

        def log(it, rn):
            if debug_iter is not None and it % debug_iter == 0:
                logger.info(f"{name} residual {rn} at the {it}-th iteration")
        rnorm, rz, bnorm, iters = pcg_per_op(self.A, self.M, self.b.data, self.x.data, self.r.data, self.z.data,
                                             self.p.data, rtol, atol, maxiter, log)
        self.rnorm.data.fill_(rnorm)
        self.rzsum.data.fill_(rz)
        self.bnorm.data.fill_(bnorm)
        logger.info(f"{name} solver completed with residual {rnorm} at the {iters}-th iteration")
        self.last_info = {"residual": rnorm, "iters": iters}
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
