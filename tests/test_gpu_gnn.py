"""GNN preconditioner on the GPU: the tcgen05 layer kernels against the
torch FP32 restatement (BF16 rounding emulated), and flexible CG with it
(Jacobi equivalence at zero output, fallback on a non-SPD network)."""
import numpy as np
import pytest
import torch

from easier_gb300.numeric.batched import BatchedPCG, join_df64, p1_instances, split_df64
from easier_gb300.numeric.preconditioner.gnn import GnnNet, GnnWeights, edge_inputs, reference_apply
from oracle import cg as ocg

pytestmark = pytest.mark.gpu


def _random_weights(seed):
    torch.manual_seed(seed)
    net = GnnNet()
    with torch.no_grad():
        net.dec.weight.normal_(0, 0.3)
        net.dec.bias.fill_(0.05)
        for lin in net.layers:
            lin.weight.mul_(2.0)
    return GnnWeights.from_net(net)


def _sign_flip_weights():
    """y = -2 r/sigma: z = -r / Av, a negative-definite preconditioner."""
    w = GnnWeights.zeros_output(0)
    w.enc_w[:] = 0
    w.enc_b[:] = 0
    w.enc_w[0, 0], w.enc_w[1, 0] = 1.0, -1.0
    w.layer_w[:] = 0
    w.layer_b[:] = 0
    w.dec_w[:] = 0
    w.dec_w[0], w.dec_w[1] = -2.0, 2.0
    w.dec_b = 0.0
    return w


@pytest.mark.parametrize("precision", ["fp64", "df64"])
@pytest.mark.parametrize("which", ["random", "sign_flip"])
def test_layer_kernels_match_torch(precision, which):
    insts = p1_instances(3, 9, 40, seed=5)
    weights = _random_weights(1) if which == "random" else _sign_flip_weights()
    eng = BatchedPCG(insts, jacobi=True, precision=precision, gnn=weights)
    rng = np.random.default_rng(2)
    r64 = torch.zeros(eng.pack.n, dtype=torch.float64)
    for i in range(len(insts)):
        rows = eng.pack.rows(i)
        r64[rows] = torch.from_numpy(rng.standard_normal(insts[i].n))
    r_dev = r64.cuda()
    r_in = split_df64(r_dev) if precision == "df64" else r_dev
    z = eng.apply_preconditioner(r_in)
    z64 = (join_df64(z) if precision == "df64" else z).cpu()
    net = weights.to_net()
    pad = torch.ones(eng.pack.n, dtype=torch.bool)
    for i, s in enumerate(insts):
        rows = eng.pack.rows(i)
        pad[rows] = False
        w, ln = edge_inputs(s.row, s.col, s.Ae, s.Av, s.edge_len)
        Av = torch.from_numpy(s.Av)
        ref = reference_apply(net, r64[rows], Av, torch.from_numpy(s.row), torch.from_numpy(s.col),
                              torch.from_numpy(w), torch.from_numpy(ln), bf16=True).double()
        # compare the network part sigma*y/Av (the Jacobi part is exact)
        jac = r64[rows] / Av
        got, want = z64[rows] - jac, ref - jac
        err = float((got - want).norm() / want.norm())
        assert err < 3e-2, (i, err)
    assert torch.all(z64[pad] == 0)


def test_fcg_zero_output_is_jacobi_pcg():
    insts = p1_instances(4, 10, 60, seed=8)
    jac = BatchedPCG(insts, jacobi=True, precision="fp64").solve(rtol=1e-8)
    fcg = BatchedPCG(insts, jacobi=True, precision="fp64", gnn=GnnWeights.zeros_output(2)).solve(rtol=1e-8)
    for a, b in zip(jac, fcg):
        assert b["status"] == "converged" and b["true_residual"] <= 1e-8 * b["bnorm"] * 1.0001
        assert abs(a["iters"] - b["iters"]) <= max(3, a["iters"] // 50), (a["iters"], b["iters"])
        assert b["fallbacks"] == 0


def _check_solutions(eng, insts, res):
    for i, (s, r) in enumerate(zip(insts, res)):
        assert r["status"] == "converged", r
        x = eng.solution(i).cpu().numpy()
        tr = ocg.true_residual(s.row, s.col, s.Ae, s.Av, s.b, x)
        assert tr <= 1e-8 * np.linalg.norm(s.b) * 1.0001


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_fcg_clips_a_negative_correction(precision):
    """z = -r/Av from the network: theta holds z.r at half the Jacobi value
    (z = invdiag r / 2), the solve goes on as scaled Jacobi."""
    insts = p1_instances(3, 10, 40, seed=6)
    eng = BatchedPCG(insts, jacobi=True, precision=precision, gnn=_sign_flip_weights(), stall_window=1 << 30)
    res = eng.solve(rtol=1e-8)
    assert all(r["clips"] >= 1 and r["fallbacks"] == 0 and r["mode"] == "gnn" for r in res)
    _check_solutions(eng, insts, res)
    # with the stall window on, a window of clipped iterations switches to Jacobi
    eng = BatchedPCG(insts, jacobi=True, precision=precision, gnn=_sign_flip_weights(), stall_window=16)
    res = eng.solve(rtol=1e-8)
    for r in res:
        if r["iters"] > 16:
            assert r["fallbacks"] == 1 and r["fallback_iter"] == 16 and r["mode"] == "jacobi", r
    _check_solutions(eng, insts, res)


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_fcg_falls_back_to_jacobi_on_nonfinite_output(precision):
    w = GnnWeights.zeros_output(1)
    w.dec_b = float("nan")
    insts = p1_instances(3, 10, 40, seed=6)
    eng = BatchedPCG(insts, jacobi=True, precision=precision, gnn=w)
    res = eng.solve(rtol=1e-8)
    assert all(r["fallbacks"] == 1 and r["fallback_iter"] == 1 and r["mode"] == "jacobi" for r in res)
    _check_solutions(eng, insts, res)
    jac = BatchedPCG(insts, jacobi=True, precision=precision).solve(rtol=1e-8)
    for a, b in zip(jac, res):
        assert abs(a["iters"] - b["iters"]) <= max(3, a["iters"] // 50)


def test_trained_weights_converge_if_present():
    from easier_gb300.numeric.preconditioner.gnn import WEIGHTS_FILE
    if not WEIGHTS_FILE.exists():
        pytest.skip("no trained weights")
    insts = p1_instances(6, 20, 80, seed=1)
    eng = BatchedPCG(insts, jacobi=True, precision="df64", gnn=GnnWeights.load())
    res = eng.solve(rtol=1e-8)
    _check_solutions(eng, insts, res)


def test_bounded_wait_gives_up_and_context_survives():
    """The GNN kernels' mbarrier wait is bounded: a wait that nothing
    completes returns with ESR_DEV_WAIT_TIMEOUT; later work still runs."""
    from easier_gb300 import _lib, ops
    ops.device_status(clear=True)
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("esr_wait_selftest", 1 << 12, _lib.ptr(flag), _lib.stream_handle())
    assert int(flag.item()) == 1
    assert ops.device_status(clear=True) & _lib.DEV_WAIT_TIMEOUT
    # the context is intact: a batched solve right after
    insts = p1_instances(2, 8, 12, seed=2)
    res = BatchedPCG(insts, jacobi=True, precision="fp64").solve(rtol=1e-8)
    assert all(r["status"] == "converged" for r in res)
    assert ops.device_status(clear=True) == 0
