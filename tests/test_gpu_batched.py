"""Batched lockstep PCG on the GPU against the oracle's per-instance CG, and
the double-float (df64) path against the FP64 true residual."""
import numpy as np
import pytest
import torch

import easier_gb300 as esr
from easier_gb300 import workloads
from easier_gb300.numeric.batched import BatchedPCG, LinsysInstance, p1_instances
from easier_gb300.numeric.preconditioner import Jacobi
from easier_gb300.numeric.solver import CG
from oracle import cg as ocg

pytestmark = pytest.mark.gpu


def _oracle(insts, rtol):
    out = []
    for s in insts:
        x, it, _ = ocg.cg(s.row, s.col, s.Ae, s.Av, s.b, rtol=rtol, maxiter=20000, jacobi=True)
        out.append((x.numpy(), it))
    return out


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_batched_vs_oracle_per_instance(precision):
    insts = p1_instances(6, 6, 40, seed=11)
    ref = _oracle(insts, 1e-8)
    eng = BatchedPCG(insts, jacobi=True, precision=precision)
    res = eng.solve(rtol=1e-8, maxiter=20000)
    for i, (s, r, (x_ref, it_ref)) in enumerate(zip(insts, res, ref)):
        assert r["status"] == "converged", (i, r)
        slack = 3 if precision == "fp64" else max(5, it_ref // 20)
        assert abs(r["iters"] - it_ref) <= slack, (i, r["iters"], it_ref)
        x = eng.solution(i).cpu().numpy()
        tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, s.b, x)
        nb = np.linalg.norm(s.b)
        assert tr <= 1e-8 * nb * 1.0001, (i, tr / nb)
        assert abs(r["true_residual"] - tr) <= 1e-3 * tr + 1e-300
        assert np.linalg.norm(x - x_ref) <= 1e-6 * np.linalg.norm(x_ref)


def test_batched_maxiter_and_uneven_finish():
    insts = p1_instances(4, 8, 64, seed=2)
    eng = BatchedPCG(insts, jacobi=True, precision="fp64")
    res = eng.solve(rtol=1e-12, maxiter=10)
    assert all(r["status"] == "maxiter" and r["iters"] == 10 for r in res)
    eng.reset()
    res = eng.solve(rtol=1e-8)
    its = [r["iters"] for r in res]
    assert all(r["status"] == "converged" for r in res) and len(set(its)) > 1


def test_df64_single_system_through_cg_api():
    eqn = workloads.P1Poisson(64, rhs_seed=4)
    sol = CG(eqn.A, eqn.b, eqn.x, M=Jacobi(eqn.A))
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    info64 = sol.solve(rtol=1e-8)
    x64 = eqn.x.collect().clone()
    eqn.x.data.zero_()
    info = sol.solve(rtol=1e-8, precision="df64")
    assert info["status"] == "converged"
    assert abs(info["iters"] - info64["iters"]) <= max(5, info64["iters"] // 20)
    nb = float(torch.linalg.vector_norm(eqn.b.collect()))
    assert info["true_residual"] <= 1e-8 * nb * 1.0001
    x = eqn.x.collect()
    assert float(torch.linalg.vector_norm(x - x64)) <= 1e-6 * float(torch.linalg.vector_norm(x64))


def test_work_shapes_and_autotune_agree():
    insts = p1_instances(5, 20, 70, seed=7)
    eng = BatchedPCG(insts, jacobi=True, precision="fp64")
    runs = []
    for m, grid in ((1, 152), (3, 300), (16, 1216)):
        eng.set_shape(m, grid)
        eng.reset()
        runs.append(eng.solve(rtol=1e-8))
    for a, b in zip(runs[0], runs[1]):
        assert a["status"] == b["status"] == "converged" and abs(a["iters"] - b["iters"]) <= 2
    for a, b in zip(runs[0], runs[2]):
        assert abs(a["iters"] - b["iters"]) <= 2
    tune = eng.autotune(tiles=(1, 4), ctas_per_sm=(2, 4), iters=4, reps=1)
    assert len(tune["table"]) == 4 and tune["tiles_per_chunk"] in (1, 4)
    eng.reset()
    res = eng.solve(rtol=1e-8)
    assert all(r["status"] == "converged" for r in res)


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_one_graph_launch_solve_matches_polled_solve(precision):
    """The whole batched solve as one CUDA graph launch (device-side loop)
    gives the same iterations and solutions as the host-polled solve."""
    insts = p1_instances(5, 8, 48, seed=21)
    eng = BatchedPCG(insts, jacobi=True, precision=precision)
    ref = eng.solve(rtol=1e-8, maxiter=5000)
    x_ref = eng.solution().clone()
    eng.reset()
    res = eng.solve_graph(rtol=1e-8, maxiter=5000)
    assert [r["iters"] for r in res] == [r["iters"] for r in ref]
    assert all(r["status"] == "converged" for r in res)
    assert torch.allclose(eng.solution(), x_ref, rtol=0, atol=0)
    # replayed: same graph, same result
    eng.reset()
    res2 = eng.solve_graph(rtol=1e-8, maxiter=5000)
    assert [r["iters"] for r in res2] == [r["iters"] for r in ref]
    # a finite maxiter ends the device loop
    eng.reset()
    res3 = eng.solve_graph(rtol=1e-14, maxiter=7)
    assert all(r["status"] == "maxiter" and r["iters"] == 7 for r in res3)


@pytest.mark.parametrize("precision,degree", [("fp64", 4), ("df64", 4), ("df64", 2), ("df64", 3)])
def test_poly_jacobi_vs_oracle_per_instance(precision, degree):
    """Polynomial-Jacobi PCG (d+1 damped Jacobi sweeps per application)
    against the oracle's CG with the same preconditioner: iterations,
    FP64-verified residual, solution; and fewer iterations than Jacobi."""
    from easier_gb300.numeric.batched import POLY_OMEGA
    insts = p1_instances(5, 6, 40, seed=13)
    eng = BatchedPCG(insts, jacobi=True, precision=precision, poly_degree=degree)
    res = eng.solve(rtol=1e-8, maxiter=20000)
    jac = BatchedPCG(insts, jacobi=True, precision=precision).solve(rtol=1e-8, maxiter=20000)
    for i, (s, r) in enumerate(zip(insts, res)):
        x_ref, it_ref, _ = ocg.cg(s.row, s.col, s.Ae, s.Av, s.b, rtol=1e-8, maxiter=20000,
                                  poly=(degree, POLY_OMEGA))
        assert r["status"] == "converged", (i, r)
        slack = 2 if precision == "fp64" else max(3, it_ref // 20)
        assert abs(r["iters"] - it_ref) <= slack, (i, r["iters"], it_ref)
        assert r["iters"] < jac[i]["iters"], (i, r["iters"], jac[i]["iters"])
        x = eng.solution(i).cpu().numpy()
        tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, s.b, x)
        assert tr <= 1e-8 * np.linalg.norm(s.b) * 1.0001
        assert np.linalg.norm(x - x_ref.numpy()) <= 1e-6 * np.linalg.norm(x_ref.numpy())


@pytest.mark.parametrize("precision", ["fp64", "df64"])
@pytest.mark.parametrize("degree", [0, 4])
def test_residual_replacement_continues_to_the_new_solution(precision, degree):
    """An instance whose FP64 true residual misses the tolerance at the
    verification (here: its FP64 right-hand side changed after the
    recurrence converged) continues from r = b - A x and converges to the
    new system's solution; the other instances stay verified."""
    insts = p1_instances(3, 10, 30, seed=4)
    eng = BatchedPCG(insts, jacobi=True, precision=precision, poly_degree=degree)
    eng.start(1e-8, None, 20000)
    while eng.active() > 0:
        eng._group(8)
    rows = eng.pack.rows(1)
    eng.b64[rows] *= 1.001
    for _ in range(16):
        eng.verify()
        if eng.active() == 0:
            break
        while eng.active() > 0:
            eng._group(8)
    res = [eng._info(s) for s in eng.instances()]
    assert [r["status"] for r in res] == ["converged"] * 3
    assert res[1]["restarts"] >= 1 and res[0]["restarts"] == 0 and res[2]["restarts"] == 0
    s = insts[1]
    x = eng.solution(1).cpu().numpy()
    tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, s.b * 1.001, x)
    assert tr <= res[1]["tol"] * 1.0001, (tr, res[1]["tol"])
    x_ref, _, _ = ocg.cg(s.row, s.col, s.Ae, s.Av, s.b * 1.001, rtol=1e-10, maxiter=20000, jacobi=True)
    assert np.linalg.norm(x - x_ref.numpy()) <= 1e-6 * np.linalg.norm(x_ref.numpy())


def test_poly_jacobi_one_graph_launch_matches_polled_solve():
    insts = p1_instances(4, 8, 40, seed=9)
    eng = BatchedPCG(insts, jacobi=True, precision="df64", poly_degree=4)
    ref = eng.solve(rtol=1e-8, maxiter=5000)
    x_ref = eng.solution().clone()
    eng.reset()
    res = eng.solve_graph(rtol=1e-8, maxiter=5000)
    assert [r["iters"] for r in res] == [r["iters"] for r in ref]
    assert all(r["status"] == "converged" for r in res)
    assert torch.equal(eng.solution(), x_ref)
