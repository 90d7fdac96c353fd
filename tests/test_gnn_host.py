"""GNN preconditioner host side: weight export round trip, BF16 emulation,
edge/node inputs of the packed batch, and that training lowers the A-norm
error of one application below Jacobi's on exact (residual, error) pairs."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch

from easier_gb300 import mesh
from easier_gb300.numeric.batched import LinsysInstance, PackedBatch, p1_edge_length, p1_instances
from easier_gb300.numeric.preconditioner.gnn import (GnnNet, GnnWeights, edge_inputs, node_input,
                                                      reference_apply)
from easier_gb300.numeric.preconditioner.train_gnn import Graphs, a_apply, train


def test_weights_roundtrip(tmp_path):
    torch.manual_seed(0)
    net = GnnNet()
    with torch.no_grad():
        net.dec.weight.normal_()
    w = GnnWeights.from_net(net)
    assert w.layer_w.dtype == np.uint16 and w.layer_w.shape == (4, 32, 96)
    w.save(tmp_path / "w.npz")
    w2 = GnnWeights.load(tmp_path / "w.npz")
    assert np.array_equal(w.layer_w, w2.layer_w) and np.array_equal(w.enc_w, w2.enc_w)
    net2 = w2.to_net()
    # the reloaded net is the BF16-rounded one: identical under bf16 emulation
    s = mesh.p1_system(9)
    row, col = torch.as_tensor(s.row), torch.as_tensor(s.col)
    wv, ln = edge_inputs(s.row, s.col, s.Ae, s.Av, p1_edge_length(9, s.row, s.col))
    r = torch.randn(s.nunk, dtype=torch.float64)
    Av = torch.as_tensor(s.Av)
    z1 = reference_apply(net, r, Av, row, col, torch.as_tensor(wv), torch.as_tensor(ln), bf16=True)
    z2 = reference_apply(net2, r, Av, row, col, torch.as_tensor(wv), torch.as_tensor(ln), bf16=True)
    assert torch.allclose(z1, z2, rtol=1e-5, atol=1e-6)
    # and close to the FP32 network
    z3 = reference_apply(net, r, Av, row, col, torch.as_tensor(wv), torch.as_tensor(ln), bf16=False)
    assert float((z1 - z3).norm() / z3.norm()) < 5e-2


def test_zero_decoder_is_jacobi():
    w = GnnWeights.zeros_output(3)
    net = w.to_net()
    s = mesh.p1_system(12)
    r = torch.randn(s.nunk, dtype=torch.float64)
    wv, ln = edge_inputs(s.row, s.col, s.Ae, s.Av, None)
    z = reference_apply(net, r, torch.as_tensor(s.Av), torch.as_tensor(s.row), torch.as_tensor(s.col),
                        torch.as_tensor(wv), torch.as_tensor(ln))
    assert torch.allclose(z, (r / torch.as_tensor(s.Av)).float(), rtol=1e-6, atol=0)


def test_packed_edge_and_node_inputs():
    insts = p1_instances(3, 5, 12, seed=4)
    pk = PackedBatch(insts, edge_features=True)
    assert pk.edge_feat.shape == (int(pk.slice_ptr[-1]), 2)
    for i, s in enumerate(insts):
        rows = pk.rows(i)
        assert np.allclose(pk.node_lk[rows], node_input(s.Av).astype(np.float32))
        # per-row multiset of (w, len) equals the instance's couplings
        w, ln = edge_inputs(s.row, s.col, s.Ae, s.Av, s.edge_len)
        r0 = int(pk.row0[i])
        for u in range(0, s.n, max(1, s.n // 7)):
            g = r0 + u
            sl, lane = g // 32, g % 32
            b, e = int(pk.slice_ptr[sl]), int(pk.slice_ptr[sl + 1])
            slots = [b + 32 * k + lane for k in range((e - b) // 32)]
            got = sorted((round(float(pk.edge_feat[t, 0]), 5), round(float(pk.edge_feat[t, 1]), 5))
                         for t in slots if pk.col[t] >= 0)
            want = sorted((round(float(a), 5), round(float(c), 5)) for a, c in zip(w[s.row == u], ln[s.row == u]))
            assert got == want
    # lengths of the P1 grid: 1 for axis neighbours, sqrt(2) for the diagonal
    el = insts[0].edge_len
    assert set(np.round(el, 6)) <= {1.0, round(np.sqrt(2), 6)}


def _pairs(s, k, rng):
    """k exact (r, e = A^-1 r) pairs with smooth errors (A^-1 of noise)."""
    A = sp.csr_matrix((s.Ae, (s.row, s.col)), shape=(s.n, s.n)) + sp.diags(s.Av)
    out = []
    for _ in range(k):
        e = spla.spsolve(A.tocsc(), rng.standard_normal(s.n))
        out.append((torch.as_tensor(A @ e, dtype=torch.float32), torch.as_tensor(e, dtype=torch.float32)))
    return out


def test_training_beats_jacobi_on_exact_pairs():
    rng = np.random.default_rng(0)
    insts = p1_instances(2, 10, 14, seed=9)
    snaps = [_pairs(s, 6, rng) for s in insts]
    dev = torch.device("cpu")
    graphs = Graphs(insts, dev)
    torch.manual_seed(0)
    net = GnnNet()
    G = graphs.batch([0])
    r, e = snaps[0][0]
    z0 = r / G["Av"]
    d0 = z0 - e
    jac = float((d0 * a_apply(G, d0)).sum() / (e * a_apply(G, e)).sum())
    hist = train(net, graphs, snaps, steps=120, minibatch=4, lr=3e-3, device=dev, log=lambda m: None)
    assert np.mean(hist[:5]) > np.mean(hist[-10:])
    assert np.mean(hist[-10:]) < jac
