"""Trains the GNN preconditioner (``gnn.py``) for the batched flexible CG.

Data: (residual, error) pairs harvested from batched Jacobi-PCG runs on a
seeded batch of P1 Poisson instances (side N ~ U{nmin..nmax}, GRF kappa,
random-mode right hand side).  A first solve to a tight tolerance gives x*;
a second, identical solve records the residual r_k and iterate x_k every
`stride` iterations of every running instance (stride chosen so that about
`pairs` pairs are kept); the error is e_k = x* - x_k = A^-1 r_k.

Loss: the A-norm relative error of one preconditioner application,
||M(r) - e||_A^2 / ||e||_A^2, averaged over a minibatch of pairs (Adam,
cosine learning-rate decay).  Runs on one GPU:

    python -m easier_gb300.numeric.preconditioner.train_gnn --out weights.npz
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np
import torch

from ..batched import BatchedPCG, p1_instances
from .gnn import GnnNet, GnnWeights, WEIGHTS_FILE, edge_inputs, node_input


def harvest(instances, pairs: int, device, rtol: float = 1e-8, log=print):
    eng = BatchedPCG(instances, jacobi=True, precision="fp64", device=device, use_graph=False)
    res = eng.solve(rtol=1e-10, maxiter=20000)
    xstar = eng.solution().clone()
    good = np.array([r["status"] == "converged" for r in res])
    iters = np.array([r["iters"] for r in res])
    # the second run stops at rtol: about 80% of the tight solve's iterations
    stride = max(1, int(round(0.8 * iters[good].sum() / max(pairs, 1))))
    eng.reset()
    eng.start(rtol, None, None)
    pk = eng.pack
    snaps = [[] for _ in instances]
    k = 0
    while eng.active() > 0:
        eng._iterate_call(stride)
        k += stride
        st = eng.instances()
        for i, s in enumerate(st):
            if s.done == 0 and good[i]:
                rows = pk.rows(i)
                snaps[i].append((eng.r[rows].float().clone(), (xstar[rows] - eng.x[rows]).float()))
    npairs = sum(len(s) for s in snaps)
    log(f"harvest: {len(instances)} instances ({int(good.sum())} with x*), stride {stride}, {npairs} pairs, "
        f"max iters {iters[good].max()}")
    return snaps


class Graphs:
    """Per-instance COO couplings and inputs on the device."""

    def __init__(self, instances, device):
        self.items = []
        for s in instances:
            row = torch.as_tensor(np.asarray(s.row, np.int64), device=device)
            col = torch.as_tensor(np.asarray(s.col, np.int64), device=device)
            Ae = np.asarray(s.Ae, np.float64)
            Av = np.asarray(s.Av, np.float64)
            w, ln = edge_inputs(np.asarray(s.row), np.asarray(s.col), Ae, Av, s.edge_len)
            self.items.append({
                "n": int(s.n), "row": row, "col": col,
                "Ae": torch.as_tensor(Ae, device=device, dtype=torch.float32),
                "Av": torch.as_tensor(Av, device=device, dtype=torch.float32),
                "w": torch.as_tensor(w, device=device, dtype=torch.float32),
                "ln": torch.as_tensor(ln, device=device, dtype=torch.float32),
                "lk": torch.as_tensor(node_input(Av), device=device, dtype=torch.float32)})

    def batch(self, picks):
        """Concatenate instances (with repeats) into one graph."""
        rows, cols, Aes, Avs, ws, lns, lks, pid = [], [], [], [], [], [], [], []
        off = 0
        for p, i in enumerate(picks):
            g = self.items[i]
            rows.append(g["row"] + off)
            cols.append(g["col"] + off)
            for dst, key in ((Aes, "Ae"), (Avs, "Av"), (ws, "w"), (lns, "ln"), (lks, "lk")):
                dst.append(g[key])
            pid.append(torch.full((g["n"],), p, dtype=torch.int64, device=g["row"].device))
            off += g["n"]
        cat = torch.cat
        return dict(row=cat(rows), col=cat(cols), Ae=cat(Aes), Av=cat(Avs), w=cat(ws), ln=cat(lns), lk=cat(lks),
                    pid=cat(pid), n=off)


def a_apply(G, v):
    return torch.zeros_like(v).index_add_(0, G["row"], G["Ae"] * v[G["col"]]) + G["Av"] * v


def train(net, graphs, snaps, steps: int, minibatch: int, lr: float, device, log=print, seed: int = 0):
    gen = np.random.default_rng(seed)
    pool = [(i, t) for i, s in enumerate(snaps) for t in range(len(s))]
    opt = torch.optim.Adam(net.parameters(), lr=lr)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, steps)
    t0 = time.perf_counter()
    hist = []
    for step in range(steps):
        pick = [pool[k] for k in gen.integers(0, len(pool), minibatch)]
        G = graphs.batch([i for i, _ in pick])
        r = torch.cat([snaps[i][t][0] for i, t in pick])
        e = torch.cat([snaps[i][t][1] for i, t in pick])
        npair = len(pick)
        rr = torch.zeros(npair, device=device).index_add_(0, G["pid"], r * r)
        cnt = torch.zeros(npair, device=device).index_add_(0, G["pid"], torch.ones_like(r))
        sigma = torch.sqrt(rr / cnt)[G["pid"]]
        y = net(r / sigma, G["lk"], G["row"], G["col"], G["w"], G["ln"])
        z = (r + sigma * y) / G["Av"]
        # scale-free: e and z are per-pair homogeneous of degree 1 in r
        d = z - e
        num = torch.zeros(npair, device=device).index_add_(0, G["pid"], d * a_apply(G, d))
        den = torch.zeros(npair, device=device).index_add_(0, G["pid"], e * a_apply(G, e))
        loss = (num / den).mean()
        opt.zero_grad(set_to_none=True)
        loss.backward()
        torch.nn.utils.clip_grad_norm_(net.parameters(), 1.0)
        opt.step()
        sched.step()
        hist.append(float(loss.detach()))
        if step % 100 == 0 or step == steps - 1:
            log(f"step {step}: loss {np.mean(hist[-100:]):.4f} ({time.perf_counter() - t0:.0f} s)")
    return hist


def evaluate(weights, count: int, nmin: int, nmax: int, seed: int, device, log=print):
    """Jacobi-PCG vs GNN flexible CG (df64) on a held-out seeded batch:
    per-instance iterations and whole-batch solve time."""
    insts = p1_instances(count, nmin, nmax, seed=seed)
    out = {}
    for name, kw in (("jacobi", {}), ("gnn", {"gnn": weights}),
                     ("gnn_nostall", {"gnn": weights, "stall_window": 1 << 30})):
        eng = BatchedPCG(insts, jacobi=True, precision="df64", device=device, **kw)
        eng.autotune()
        eng.run(1e-8)
        eng.reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = eng.solve(rtol=1e-8)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        its = np.array([r["iters"] for r in res])
        ok = all(r["status"] == "converged" for r in res)
        fb = sum(r["fallbacks"] for r in res)
        fbi = [r["fallback_iter"] for r in res if r["fallbacks"]]
        clips = sum(r["clips"] for r in res)
        out[name] = {"seconds": dt, "iters_mean": float(its.mean()), "iters_max": int(its.max()), "converged": ok,
                     "fallbacks": fb, "fallback_iter_median": float(np.median(fbi)) if fbi else None}
        log(f"eval {name}: {dt:.3f} s, iters mean {its.mean():.1f} max {its.max()}, converged {ok}, "
            f"fallbacks {fb} (median at iteration {out[name]['fallback_iter_median']}), theta clips {clips}")
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(WEIGHTS_FILE))
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--nmin", type=int, default=32)
    ap.add_argument("--nmax", type=int, default=512)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--pairs", type=int, default=50000)
    ap.add_argument("--steps", type=int, default=1500)
    ap.add_argument("--minibatch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--eval-count", type=int, default=64)
    ap.add_argument("--eval-seed", type=int, default=1)
    args = ap.parse_args(argv)
    dev = torch.device("cuda")
    torch.manual_seed(args.seed)
    t0 = time.perf_counter()
    insts = p1_instances(args.count, args.nmin, args.nmax, seed=args.seed)
    print(f"instances: {time.perf_counter() - t0:.1f} s", flush=True)
    snaps = harvest(insts, args.pairs, dev, log=lambda m: print(m, flush=True))
    graphs = Graphs(insts, dev)
    net = GnnNet().to(dev)
    train(net, graphs, snaps, args.steps, args.minibatch, args.lr, dev, log=lambda m: print(m, flush=True))
    w = GnnWeights.from_net(net.cpu())
    w.save(args.out)
    print(f"saved {args.out} ({time.perf_counter() - t0:.0f} s total)", flush=True)
    del snaps, graphs
    torch.cuda.empty_cache()
    if args.eval_count > 0:
        evaluate(w, args.eval_count, args.nmin, args.nmax, args.eval_seed, dev, log=lambda m: print(m, flush=True))


if __name__ == "__main__":
    main()
