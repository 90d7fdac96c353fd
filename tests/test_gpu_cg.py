"""Linsys SpMV and the fused (P)CG on the GPU against the reference's runs
(golden) and the oracle."""
import numpy as np
import pytest
import torch

import easier_gb300 as esr
from easier_gb300 import mesh, workloads
from easier_gb300.numeric import Linsys
from easier_gb300.numeric.preconditioner import Jacobi
from easier_gb300.numeric.solver import CG, GMRES
from easier_gb300.numeric.sparse import SellMatrix
from oracle import cg as ocg
from oracle import sparse as osp

pytestmark = pytest.mark.gpu


def _p1_module(row, col, Ae, Av, b):
    class P1(esr.Module):
        def __init__(self):
            super().__init__()
            n = len(Av)
            self.reducer = esr.Reducer(torch.as_tensor(row), n)
            self.selector = esr.Selector(torch.as_tensor(col))
            self.x = esr.Tensor(torch.zeros(n, dtype=torch.float64), mode="partition")
            self.b = esr.Tensor(torch.as_tensor(b, dtype=torch.float64), mode="partition")
            self.Av = esr.Tensor(torch.as_tensor(Av, dtype=torch.float64), mode="partition")
            self.Ae = esr.Tensor(torch.as_tensor(Ae, dtype=torch.float64), mode="partition")
            self.A = Linsys(self.Av, self.Ae, self.selector, self.reducer)
    return P1()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_spmv_bitwise_vs_oracle_fv_and_p1(dtype):
    m = mesh.triangular_mesh(40)
    a = mesh.poisson_fv(m)
    rng = np.random.default_rng(1)
    kappa = mesh.kappa_from_field(mesh.gaussian_random_field(60, 2))
    p1 = mesh.p1_system(60, kappa)
    for row, col, Ae, Av in ((m.src, m.dst, a.Af, a.Ac), (p1.row, p1.col, p1.Ae, p1.Av)):
        n = len(Av)
        x = torch.from_numpy(rng.standard_normal(n)).to(dtype)
        Ae_t, Av_t = torch.from_numpy(Ae).to(dtype), torch.from_numpy(Av).to(dtype)
        A = SellMatrix.from_arrays(n, row, col, Ae_t.cuda(), Av_t.cuda())
        y = A.spmv(x.cuda()).cpu()
        assert torch.equal(y, osp.linsys_apply(x, row, col, Ae_t, Av_t))
        # and through the per-op path of Linsys.forward
        mod = _p1_module(row, col, Ae, Av, np.zeros(n)).to(dtype)
        esr.compile([mod], "cuda")
        assert torch.equal(mod.A(x.cuda()).cpu(), y)


def test_cg_fv_n10_vs_reference(golden):
    g = golden("poisson_fv_n10_solve.npz")
    eqn = workloads.make_poisson_fv(10)
    sol = CG(eqn.A, eqn.b, eqn.x)
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    info = sol.solve(rtol=1e-8, maxiter=2000)
    assert abs(info["iters"] - int(g["cg_iters"])) <= 2
    x = eqn.x.collect().cpu().numpy()
    assert np.linalg.norm(x - g["cg_x"]) <= 1e-7 * np.linalg.norm(g["cg_x"])
    assert info["true_residual"] <= 2e-8 * np.linalg.norm(eqn.b.collect().cpu().numpy())


def test_cg_fv_n100_vs_reference(golden):
    """The tutorial's FV Poisson at N=100 (40,000 cells, 119,600 edges) on
    the fused CG, against the reference's own CG run: iterations within 2,
    solution within 1e-7, FP64 true residual at the tolerance."""
    g = golden("poisson_fv_n100_cg.npz")
    eqn = workloads.make_poisson_fv(100)
    sol = CG(eqn.A, eqn.b, eqn.x)
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    assert sol.fusable()
    info = sol.solve(rtol=1e-8, maxiter=5000)
    assert abs(info["iters"] - int(g["cg_iters"])) <= 2
    x = eqn.x.collect().cpu().numpy()
    assert np.linalg.norm(x - g["cg_x"]) <= 1e-7 * np.linalg.norm(g["cg_x"])
    assert info["true_residual"] <= 1.0001e-8 * np.linalg.norm(eqn.b.collect().cpu().numpy())


def test_cg_p1_vs_reference(golden):
    g = golden("linsys_p1_n12_cg.npz")
    eqn = _p1_module(g["row"], g["col"], g["Ae"], g["Av"], g["b"])
    sol = CG(eqn.A, eqn.b, eqn.x)
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    info = sol.solve(rtol=1e-10, maxiter=1000)
    assert abs(info["iters"] - int(g["iters"])) <= 1
    assert np.allclose(eqn.x.collect().cpu().numpy(), g["x"], rtol=1e-9, atol=1e-12)


def test_per_op_cg_matches_fused():
    eqn = workloads.P1Poisson(24, rhs_seed=3)
    sol = CG(eqn.A, eqn.b, eqn.x, M=Jacobi(eqn.A))
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    info_f = sol.solve(rtol=1e-8)
    x_f = eqn.x.collect().clone()
    eqn.x.data.zero_()
    info_p = sol.solve(rtol=1e-8, fused=False)
    assert abs(info_f["iters"] - info_p["iters"]) <= 2
    assert torch.allclose(eqn.x.collect(), x_f, rtol=1e-6, atol=1e-10)


def test_jacobi_pcg_grf_vs_oracle():
    n = 48
    kappa = mesh.kappa_from_field(mesh.gaussian_random_field(n, 9))
    s = mesh.p1_system(n, kappa)
    b = mesh.random_mode_rhs(n, 4)
    x_ref, it_ref, _ = ocg.cg(s.row, s.col, s.Ae, s.Av, b, rtol=1e-8, maxiter=5000, jacobi=True)
    eqn = _p1_module(s.row, s.col, s.Ae, s.Av, b)
    sol = CG(eqn.A, eqn.b, eqn.x, M=Jacobi(eqn.A))
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    info = sol.solve(rtol=1e-8, maxiter=5000)
    assert abs(info["iters"] - it_ref) <= 3
    x = eqn.x.collect().cpu().numpy()
    assert np.linalg.norm(x - x_ref.numpy()) <= 1e-6 * np.linalg.norm(x_ref.numpy())
    tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, b, x)
    assert tr <= 1.5e-8 * np.linalg.norm(b)


def test_mixed_precision_reaches_fp64_true_residual():
    eqn = workloads.P1Poisson(96, rhs_seed=1)
    sol = CG(eqn.A, eqn.b, eqn.x, M=Jacobi(eqn.A))
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    info = sol.solve(rtol=1e-8, precision="mixed")
    b = eqn.b.collect().cpu().numpy()
    s = mesh.p1_system(96)
    tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, b, eqn.x.collect().cpu().numpy())
    assert tr <= 1e-8 * np.linalg.norm(b)
    assert info["replacements"] >= 1 and info["status"] == "converged"
    eqn.x.data.zero_()
    info64 = sol.solve(rtol=1e-8)
    x64 = eqn.x.collect().cpu().numpy()
    assert info64["true_residual"] <= 1.5e-8 * np.linalg.norm(b)


def test_maxiter_and_status():
    eqn = workloads.P1Poisson(32, rhs_seed=2)
    sol = CG(eqn.A, eqn.b, eqn.x)
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    info = sol.solve(rtol=1e-12, maxiter=5)
    assert info["iters"] == 5 and info["status"] == "maxiter"


@pytest.mark.parametrize("fused", [False, True])
def test_gmres_vs_reference(golden, fused):
    g = golden("poisson_fv_n10_solve.npz")
    eqn = workloads.make_poisson_fv(10)
    sol = GMRES(eqn.A, eqn.b, eqn.x)
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    assert sol.fusable()
    info = sol.solve(rtol=1e-8, maxiter=2000, fused=fused)
    assert abs(info["iters"] - int(g["gmres_iters"])) <= 2
    x = eqn.x.collect().cpu().numpy()
    assert np.linalg.norm(x - g["gmres_x"]) <= 1e-6 * np.linalg.norm(g["gmres_x"])


def test_fused_gmres_matches_per_op_path():
    """Fused restart cycles (CUDA graph) vs the reference's modules run
    per-op on the GB300 kernels: same iteration count, same solution to
    the solve tolerance; Jacobi and identity M; a short restart."""
    for M_jacobi, restart in ((True, 20), (False, 7)):
        eqn = workloads.P1Poisson(20, rhs_seed=5)
        sol = GMRES(eqn.A, eqn.b, eqn.x, M=Jacobi(eqn.A) if M_jacobi else None, restart=restart)
        [eqn, sol] = esr.compile([eqn, sol], "cuda")
        assert sol.fusable()
        info_f = sol.solve(rtol=1e-8, maxiter=500)
        x_f = eqn.x.collect().clone()
        eqn.x.data.zero_()
        info_p = sol.solve(rtol=1e-8, maxiter=500, fused=False)
        x_p = eqn.x.collect()
        assert abs(info_f["iters"] - info_p["iters"]) <= 1, (info_f, info_p)
        assert torch.allclose(x_f, x_p, rtol=1e-6, atol=1e-9)
        b = eqn.b.collect().cpu().numpy()
        s = mesh.p1_system(20)
        tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, b, x_f.cpu().numpy())
        assert tr <= 1e-8 * np.linalg.norm(b) * 1.0001


def test_fused_gmres_maxiter():
    eqn = workloads.P1Poisson(40, rhs_seed=1)
    sol = GMRES(eqn.A, eqn.b, eqn.x, restart=5)
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    info = sol.solve(rtol=1e-12, maxiter=3)
    assert info["iters"] == 3 and info["residual"] > 0


def test_fp32_system_uses_single_system_kernels():
    """An FP32 Linsys solves on the single-system PCG kernels (float
    vectors, (hi, lo) float-pair dot accumulation) and reaches the FP32
    tolerance against the FP64 oracle."""
    from easier_gb300.numeric.sparse import FusedPCG
    eqn = workloads.P1Poisson(48, rhs_seed=7)
    eqn.to(torch.float32)
    sol = CG(eqn.A, eqn.b, eqn.x, M=Jacobi(eqn.A))
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    assert eqn.x.dtype == torch.float32 and sol.r.dtype == torch.float32
    info = sol.solve(rtol=1e-5, maxiter=5000)
    assert isinstance(sol._fused, FusedPCG) and info["status"] == "converged"
    s = mesh.p1_system(48)
    b = mesh.random_mode_rhs(48, 7)
    x_ref, it_ref, _ = ocg.cg(s.row, s.col, s.Ae, s.Av, b, rtol=1e-5, maxiter=5000, jacobi=True)
    _, it32, _ = ocg.cg(s.row, s.col, s.Ae, s.Av, b, rtol=1e-5, maxiter=5000, jacobi=True, dtype=torch.float32)
    # the FP32 recurrence (reference order, FP32 tensors) takes more
    # iterations than FP64 on this few-mode right hand side
    assert abs(info["iters"] - it32) <= max(3, it32 // 10), (info["iters"], it32, it_ref)
    x = eqn.x.collect().double().cpu().numpy()
    assert np.linalg.norm(x - x_ref.numpy()) <= 1e-3 * np.linalg.norm(x_ref.numpy())
    tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, b, x)
    assert tr <= 2e-5 * np.linalg.norm(b)


@pytest.mark.parametrize("solver", ["cg", "gmres"])
def test_fused_plan_follows_operator_values_changed_through_data(solver):
    """Refilling Ae/Av through ``.data`` (which leaves version counters
    alone) between two solves must rebuild the fused plan: scaling the
    operator by 2 halves the solution."""
    eqn = workloads.P1Poisson(16, rhs_seed=0)
    M = Jacobi(eqn.A)
    sol = CG(eqn.A, eqn.b, eqn.x, M=M) if solver == "cg" else GMRES(eqn.A, eqn.b, eqn.x, M=M, restart=10)
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    sol.solve(rtol=1e-11, maxiter=500)
    x1 = eqn.x.collect().clone()
    plan = sol._fused
    eqn.A.Ae.data.mul_(2)
    eqn.A.Av.data.mul_(2)
    eqn.x.data.zero_()
    sol.solve(rtol=1e-11, maxiter=500)
    assert sol._fused is not plan
    assert torch.allclose(eqn.x.collect(), x1 / 2, rtol=1e-8, atol=1e-14)
    # unchanged values keep the plan
    plan = sol._fused
    eqn.x.data.zero_()
    sol.solve(rtol=1e-11, maxiter=500)
    assert sol._fused is plan


def test_per_op_paths_take_any_operator_and_preconditioner():
    """A plain nn.Module operator (not a Linsys) and a callable
    preconditioner run the per-op CG and GMRES loops; both reach the
    tolerance on the FP64 true residual of the same system."""
    from torch import nn
    s = mesh.p1_system(20)
    for which in ("cg", "gmres"):
        eqn = workloads.P1Poisson(20, rhs_seed=2)

        class Op(nn.Module):
            def forward(self, v):
                return eqn.A(v)
        M = lambda r: r / eqn.A.Av  # noqa: E731
        sol = CG(Op(), eqn.b, eqn.x, M=M) if which == "cg" else GMRES(Op(), eqn.b, eqn.x, M=M, restart=15)
        [eqn, sol] = esr.compile([eqn, sol], "cuda")
        assert not sol.fusable()
        info = sol.solve(rtol=1e-9, maxiter=3000)
        b = eqn.b.collect().cpu().numpy()
        tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, b, eqn.x.collect().cpu().numpy())
        assert tr <= 1.05e-9 * np.linalg.norm(b), (which, info, tr)
