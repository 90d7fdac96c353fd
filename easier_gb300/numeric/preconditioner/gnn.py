"""GNN preconditioner for flexible CG (no reference counterpart).

Network (the contract between this module, its trainer and the CUDA
kernels of ``csrc/gnn.cu``), per node i of one system, sigma = rms(r):

    h0_i = relu(enc_w [r_i / sigma, lk_i] + enc_b)                  32
    for l in 1..4:
        A_i = sum_j w_ij h_j,  L_i = sum_j len_ij h_j   (j over row i's couplings)
        h_i = h_i + relu(W_l [h_i, A_i, L_i] + b_l)                  96 -> 32
    y_i = dec_w . h_i + dec_b
    z_i = (r_i + sigma y_i) / Av_i

Node input lk_i = log(Av_i / 4): the log of the kappa-weighted mean over
the node's triangles on the P1 grid (Av_i = 4 for kappa = 1).  Edge inputs:
w_ij = Ae_ij / sqrt(Av_i Av_j) (normalised coupling) and len_ij (edge
length in grid units).  With the network's output at zero the
preconditioner is Jacobi.  On the device the features are BF16 and the
MLPs run on the tensor cores; ``GnnNet.forward(..., bf16=True)`` rounds at
the same points for parity tests.
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path
from typing import Optional

import numpy as np
import torch
from torch import nn

HIDDEN = 32
LAYERS = 4
WEIGHTS_FILE = Path(__file__).resolve().parent / "gnn_p1_weights.npz"


def _bf16(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.bfloat16).to(torch.float32)


class GnnNet(nn.Module):
    def __init__(self, hidden: int = HIDDEN, layers: int = LAYERS):
        super().__init__()
        self.enc = nn.Linear(2, hidden)
        self.layers = nn.ModuleList([nn.Linear(3 * hidden, hidden) for _ in range(layers)])
        self.dec = nn.Linear(hidden, 1)
        with torch.no_grad():  # start at Jacobi: zero output
            self.dec.weight.zero_()
            self.dec.bias.zero_()

    def forward(self, rhat: torch.Tensor, lk: torch.Tensor, row: torch.Tensor, col: torch.Tensor,
                w: torch.Tensor, ln: torch.Tensor, bf16: bool = False) -> torch.Tensor:
        """y for every node; (row, col) = couplings (i receives from j)."""
        q = _bf16 if bf16 else (lambda t: t)
        x = torch.stack([rhat, lk], dim=-1)
        if bf16:
            h = q(torch.relu(x @ _bf16(self.enc.weight).t() + self.enc.bias))
        else:
            h = torch.relu(self.enc(x))
        n = h.shape[0]
        for lin in self.layers:
            hj = h[col]
            A = torch.zeros_like(h).index_add_(0, row, w[:, None] * hj)
            L = torch.zeros_like(h).index_add_(0, row, ln[:, None] * hj)
            u = q(torch.cat([h, A, L], dim=-1))
            if bf16:
                out = u @ _bf16(lin.weight).t() + lin.bias
            else:
                out = lin(u)
            h = q(h + torch.relu(out))
        if bf16:
            return h @ _bf16(self.dec.weight).t().squeeze(-1) + self.dec.bias
        return self.dec(h).squeeze(-1)


@dataclass
class GnnWeights:
    """Exported weights: BF16 values (stored as float32 / uint16 bits)."""
    enc_w: np.ndarray    # [32, 2] float32 (BF16-rounded)
    enc_b: np.ndarray    # [32]
    layer_w: np.ndarray  # [4, 32, 96] uint16 BF16 bits
    layer_b: np.ndarray  # [4, 32] float32
    dec_w: np.ndarray    # [32] float32 (BF16-rounded)
    dec_b: float

    @classmethod
    def from_net(cls, net: GnnNet) -> "GnnWeights":
        with torch.no_grad():
            lw = torch.stack([l.weight.detach().float().cpu() for l in net.layers])
            bits = lw.to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
            return cls(enc_w=_bf16(net.enc.weight.detach().float().cpu()).numpy(),
                       enc_b=net.enc.bias.detach().float().cpu().numpy(),
                       layer_w=bits.copy(),
                       layer_b=torch.stack([l.bias.detach().float().cpu() for l in net.layers]).numpy(),
                       dec_w=_bf16(net.dec.weight.detach().float().cpu()).reshape(-1).numpy(),
                       dec_b=float(net.dec.bias.detach().float().cpu()[0]))

    def to_net(self) -> GnnNet:
        net = GnnNet()
        with torch.no_grad():
            net.enc.weight.copy_(torch.from_numpy(self.enc_w))
            net.enc.bias.copy_(torch.from_numpy(self.enc_b))
            lw = torch.from_numpy(self.layer_w.view(np.int16).copy()).view(torch.bfloat16).float()
            for k, lin in enumerate(net.layers):
                lin.weight.copy_(lw[k])
                lin.bias.copy_(torch.from_numpy(self.layer_b[k]))
            net.dec.weight.copy_(torch.from_numpy(self.dec_w).reshape(1, -1))
            net.dec.bias.fill_(self.dec_b)
        return net

    def save(self, path) -> None:
        np.savez(path, enc_w=self.enc_w, enc_b=self.enc_b, layer_w=self.layer_w, layer_b=self.layer_b,
                 dec_w=self.dec_w, dec_b=np.array([self.dec_b], np.float32))

    @classmethod
    def load(cls, path=None) -> "GnnWeights":
        d = np.load(WEIGHTS_FILE if path is None else path)
        return cls(d["enc_w"].astype(np.float32), d["enc_b"].astype(np.float32), d["layer_w"].astype(np.uint16),
                   d["layer_b"].astype(np.float32), d["dec_w"].astype(np.float32), float(d["dec_b"][0]))

    @classmethod
    def zeros_output(cls, seed: int = 0) -> "GnnWeights":
        """Random hidden layers with a zero decoder: the preconditioner is
        exactly Jacobi (used before training and in tests)."""
        torch.manual_seed(seed)
        return cls.from_net(GnnNet())

    def device_tensors(self, dev) -> dict:
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        return {"enc_w": t(self.enc_w.astype(np.float32)), "enc_b": t(self.enc_b.astype(np.float32)),
                "layer_w": t(self.layer_w.view(np.int16)), "layer_b": t(self.layer_b.astype(np.float32)),
                "dec_w": t(self.dec_w.astype(np.float32))}


def node_input(Av: np.ndarray) -> np.ndarray:
    """lk_i = log(Av_i / 4)."""
    return np.log(np.maximum(Av, 1e-300) / 4.0)


def edge_inputs(row: np.ndarray, col: np.ndarray, Ae: np.ndarray, Av: np.ndarray,
                edge_len: Optional[np.ndarray]):
    """(w, len) per coupling."""
    w = Ae / np.sqrt(Av[row] * Av[col])
    ln = np.ones_like(w) if edge_len is None else np.asarray(edge_len, np.float64)
    return w, ln


def reference_apply(net: GnnNet, r: torch.Tensor, Av: torch.Tensor, row, col, w, ln,
                    bf16: bool = True) -> torch.Tensor:
    """z = (r + sigma y) / Av for one system, in FP32 on the tensors' device
    (the torch restatement of the device preconditioner)."""
    r32 = r.to(torch.float32)
    n = r32.shape[0]
    sigma = torch.sqrt((r.to(torch.float64) ** 2).sum() / max(n, 1)).to(torch.float32)
    rhat = r32 / sigma if float(sigma) > 0 else torch.zeros_like(r32)
    lk = torch.log(Av.to(torch.float64) / 4.0).to(torch.float32)
    y = net(rhat, lk, row, col, w.to(torch.float32), ln.to(torch.float32), bf16=bf16)
    return (r32 + sigma * y) / Av.to(torch.float32)
