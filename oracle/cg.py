"""Oracle: conjugate gradient (test infrastructure).

Restates easier/numeric/solver/cg.py (Init :49-53, Step :68-76,
Update :90-95, CG.solve :130-161) on torch CPU tensors, with an optional
diagonal (Jacobi) preconditioner M(r) = r / Av, or (``poly = (d, omega)``,
no reference counterpart) the polynomial-Jacobi preconditioner: d+1 damped
Jacobi sweeps y <- y + W (r - A y) on A z = r from y = 0, W = omega / Av,
i.e. the Neumann polynomial z = sum_{j<=d} (I - W A)^j W r (Saad,
"Iterative Methods for Sparse Linear Systems", 2nd ed., sec. 12.3).
"""
import torch

from .sparse import linsys_apply


def poly_jacobi(A, Av, r, d, omega):
    """z = sum_{j<=d} (I - W A)^j W r, W = omega / Av, by d+1 damped Jacobi
    sweeps from y = 0 (the first is y = W r)."""
    w = omega / Av
    y = w * r
    for _ in range(d):
        y = y + w * (r - A(y))
    return y


def cg(row, col, Ae, Av, b, x0=None, rtol=1e-5, atol=None, maxiter=None, jacobi=False, dtype=torch.float64,
       poly=None):
    """``dtype`` = the system's dtype (the reference computes in the module's
    dtype: FP64 by default, FP32 after ``Module.to(torch.float32)``)."""
    Ae, Av, b = (torch.as_tensor(a).to(dtype) for a in (Ae, Av, b))
    A = lambda v: linsys_apply(v, row, col, Ae, Av)  # noqa: E731
    M = (lambda r: r / Av) if jacobi else (lambda r: r)  # noqa: E731
    if poly is not None:
        M = lambda r: poly_jacobi(A, Av, r, poly[0], poly[1])  # noqa: E731
    x = torch.zeros_like(b) if x0 is None else torch.as_tensor(x0).to(dtype).clone()
    r = b - A(x)
    z = M(r)
    p = z.clone()
    bnorm = torch.linalg.vector_norm(b)
    tol = rtol * bnorm
    if atol:
        tol = max(tol, torch.tensor(atol, dtype=dtype))
    iters = 0
    while True:
        Ap = A(p)
        rz = (r * z).sum()
        alpha = rz / (p * Ap).sum()
        r = r - alpha * Ap
        x = x + alpha * p
        rnorm = torch.linalg.vector_norm(r)
        if (not torch.isnan(rnorm) and rnorm <= tol) or (maxiter is not None and iters >= maxiter):
            break
        iters += 1
        z1 = M(r)
        beta = (r * z1).sum() / rz
        p = z1 + beta * p
        z = z1
    return x, iters, float(rnorm)


def true_residual(row, col, Ae, Av, b, x):
    b = torch.as_tensor(b, dtype=torch.float64)
    return float(torch.linalg.vector_norm(b - linsys_apply(torch.as_tensor(x), row, col, Ae, Av)))
