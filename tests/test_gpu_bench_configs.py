"""Parity at the benchmarked configurations, against the oracle.

* Shallow water, N=2000 (16,000,000 cells), FP32 fast arithmetic on the
  temporally blocked kernel (the bench's engine), 5 steps at dt=2.5e-4,
  against the FP64 oracle step on the same mesh and initial state.
  Bar: relative max-norm error of the state vector (h, uh, vh) at most 1e-5.
* P1 Poisson 1000x1000 (998,001 unknowns), Jacobi-PCG to relative residual
  1e-8 in FP64 and in double-float, against the oracle's FP64 Jacobi-PCG.
* Four instances of the seeded 256-instance batch (GRF kappa, side
  N ~ U{32..512}, seed 0), FP64 and double-float, and four held-out
  instances (seed 1) with the GNN preconditioner, against oracle CG.

For the solves the bar is the solve tolerance: both solutions have FP64
true residuals at most 1e-8 ||b||, so ||A (x - x_oracle)|| <= 2e-8 ||b||
(computed in FP64 with the oracle's SpMV); iteration counts are compared
too, and the relative solution difference ||x - x_oracle|| / ||x_oracle||
is printed (run with -s to see it).
"""
import numpy as np
import pytest
import torch

import easier_gb300 as esr
from easier_gb300 import mesh, workloads
from oracle import cg as ocg
from oracle import mesh as omesh
from oracle import sparse as osp
from oracle import swe as oswe

pytestmark = pytest.mark.gpu

# instances of the seed-0 batch (256 instances, N ~ U{32..512}) compared with
# the oracle: the largest side (53: N=511), the largest kappa_max/kappa_min
# x N^2 (30: N=439), the smallest side (23: N=33) and the first (0);
# tests/test_inputs_seeded.py re-derives the choice
CONFIG3_PICKS = (53, 30, 23, 0)
# held-out seed-1 instances for the GNN: the largest side (130: N=512) and
# three more
CONFIG4_PICKS = (130, 1, 2, 3)


def _a_diff(row, col, Ae, Av, x, x_ref):
    d = torch.as_tensor(np.asarray(x, dtype=np.float64) - np.asarray(x_ref, dtype=np.float64))
    return float(torch.linalg.vector_norm(osp.linsys_apply(d, row, col, torch.as_tensor(Ae), torch.as_tensor(Av))))


def test_swe_n2000_fast_fp32_vs_fp64_oracle():
    n, steps, dt = 2000, 5, 2.5e-4
    eqn = workloads.make_swe(n, dt=dt, dtype=torch.float32)
    [eqn] = esr.compile([eqn], "cuda", precision="fast")
    eng = eqn.easier_fused_engine
    assert eng.tiled and eng.precision == "fast"
    h0 = eqn.h.collect().cpu().double()
    eng.step(steps)
    torch.cuda.synchronize()
    got = np.concatenate([getattr(eqn, k).collect().cpu().double().numpy() for k in ("h", "uh", "vh")])
    del eqn, eng
    torch.cuda.empty_cache()
    m = omesh.triangular_mesh(n)
    g = omesh.swe_geometry(m)
    p = oswe.SweProblem(m["src"], m["dst"], m["bcells"], g["sx"], g["sy"], g["alpha"], g["bsx"], g["bsy"],
                        g["area"], dt, torch.float64)
    z = torch.zeros_like(h0)
    ref = np.concatenate([t.numpy() for t in p.run(h0, z, z.clone(), steps)])
    err = np.abs(got - ref).max() / np.abs(ref).max()
    print(f"\nSWE N=2000 fast FP32 vs FP64 oracle after {steps} steps: relative max-norm error {err:.3e}")
    assert err <= 1e-5


@pytest.mark.parametrize("precision", ["native", "df64"])
def test_p1_1000_jacobi_pcg_vs_oracle(precision):
    from easier_gb300.numeric.preconditioner import Jacobi
    from easier_gb300.numeric.solver import CG
    n = 1000
    eqn = workloads.P1Poisson(n, rhs_seed=0)
    sol = CG(eqn.A, eqn.b, eqn.x, M=Jacobi(eqn.A))
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    info = sol.solve(rtol=1e-8, precision=precision)
    x = eqn.x.collect().cpu().numpy()
    b = eqn.b.collect().cpu().numpy()
    s = mesh.p1_system(n)
    x_ref, it_ref, _ = ocg.cg(s.row, s.col, s.Ae, s.Av, b, rtol=1e-8, jacobi=True)
    x_ref = x_ref.numpy()
    bn = np.linalg.norm(b)
    tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, b, x)
    rel = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
    print(f"\nP1-1000 {precision}: {info['iters']} iterations (oracle {it_ref}), true rel. residual {tr / bn:.3e}, "
          f"||x - x_oracle|| / ||x_oracle|| = {rel:.3e}")
    assert tr <= 1e-8 * bn * 1.0001
    assert _a_diff(s.row, s.col, s.Ae, s.Av, x, x_ref) <= 2e-8 * bn
    slack = 3 if precision == "native" else max(5, it_ref // 8)
    assert abs(info["iters"] - it_ref) <= slack


def _batched_vs_oracle(insts, label, **engine_kw):
    from easier_gb300.numeric.batched import BatchedPCG
    eng = BatchedPCG(insts, jacobi=True, **engine_kw)
    res = eng.solve(rtol=1e-8)
    out = []
    for i, (si, ri) in enumerate(zip(insts, res)):
        assert ri["status"] == "converged", (label, i, ri)
        x = eng.solution(i).cpu().numpy()
        x_ref, it_ref, _ = ocg.cg(si.row, si.col, si.Ae, si.Av, si.b, rtol=1e-8, jacobi=True)
        x_ref = x_ref.numpy()
        bn = np.linalg.norm(si.b)
        tr = ocg.true_residual(si.row, si.col, si.Ae, si.Av, si.b, x)
        rel = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        side = int(round(np.sqrt(si.n))) + 1
        print(f"\n{label} instance N={side}: {ri['iters']} iterations (oracle Jacobi-PCG {it_ref}), "
              f"true rel. residual {tr / bn:.3e}, ||x - x_oracle|| / ||x_oracle|| = {rel:.3e}")
        assert tr <= 1e-8 * bn * 1.0001
        assert _a_diff(si.row, si.col, si.Ae, si.Av, x, x_ref) <= 2e-8 * bn
        out.append((ri["iters"], it_ref))
    return out


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_batched_config_instances_vs_oracle(precision):
    from easier_gb300.numeric.batched import p1_instance, p1_sides
    sides = p1_sides(256, 32, 512, seed=0)
    insts = [p1_instance(i, int(sides[i]), seed=0) for i in CONFIG3_PICKS]
    for got, ref in _batched_vs_oracle(insts, f"batched {precision}", precision=precision):
        slack = 3 if precision == "fp64" else max(5, ref // 8)
        assert abs(got - ref) <= slack


def test_gnn_flexible_cg_held_out_instances_vs_oracle():
    from easier_gb300.numeric.batched import p1_instance, p1_sides
    from easier_gb300.numeric.preconditioner.gnn import GnnWeights
    sides = p1_sides(256, 32, 512, seed=1)
    insts = [p1_instance(i, int(sides[i]), seed=1) for i in CONFIG4_PICKS]
    _batched_vs_oracle(insts, "GNN flexible CG", precision="df64", gnn=GnnWeights.load())
