"""Oracle: Selector / Reducer / Linsys / orderings (test infrastructure).

Selector.forward = t[idx]  (easier/core/module.py:364-371)
Reducer.forward  = out.scatter_reduce_(0, idx, t, op, include_self=False)
                   (easier/core/module.py:441-461)
Linsys.forward   = reducer(selector(x) * Ae) + x * Av  (easier/numeric/linsys.py:23-24)
stable CSR       = the edge order of sparse_encoding.py:244-338 at world size 1
"""
from collections import deque

import numpy as np
import torch


def select(x, idx):
    return torch.as_tensor(x)[torch.as_tensor(idx, dtype=torch.int64)]


def reduce(t, idx, n, op="sum", out=None):
    t = torch.as_tensor(t)
    idx = torch.as_tensor(idx, dtype=torch.int64)
    if out is None:
        out = torch.zeros((n,) + tuple(t.shape[1:]), dtype=t.dtype)
    else:
        out = torch.as_tensor(out).clone()
    ix = idx[(...,) + (None,) * (t.dim() - 1)].expand(-1, *t.shape[1:])
    return out.scatter_reduce_(0, ix, t, op, include_self=False)


def linsys_apply(x, row, col, Ae, Av):
    x = torch.as_tensor(x)
    n = x.shape[0]
    return reduce(select(x, col) * torch.as_tensor(Ae), row, n) + x * torch.as_tensor(Av)


def stable_csr(idx, n):
    """rowptr [n+1] and perm with a stable ascending sort of idx."""
    idx = np.asarray(idx, dtype=np.int64)
    perm = np.argsort(idx, kind="stable")
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, idx + 1, 1)
    return np.cumsum(rowptr), perm


def rcm(n, src, dst):
    """Reverse Cuthill-McKee, pure Python (small graphs): undirected simple
    graph; components in (degree, index) order of their first unplaced
    vertex; pseudo-peripheral start by repeated BFS while the eccentricity
    grows (<= 16 rounds); neighbours by (degree, index); order reversed."""
    adj = [set() for _ in range(n)]
    for a, b in zip(src, dst):
        if a != b:
            adj[a].add(b)
            adj[b].add(a)
    deg = [len(s) for s in adj]
    key = lambda v: (deg[v], v)  # noqa: E731
    nbrs = [sorted(s, key=key) for s in adj]

    def bfs_last(s):
        level = {s: 0}
        q = deque([s])
        order = [s]
        while q:
            v = q.popleft()
            for w in nbrs[v]:
                if w not in level:
                    level[w] = level[v] + 1
                    q.append(w)
                    order.append(w)
        ecc = max(level.values())
        return min((v for v in order if level[v] == ecc), key=key), ecc

    placed = [False] * n
    out = []
    for r in sorted(range(n), key=key):
        if placed[r]:
            continue
        start = r
        cand, ecc = bfs_last(start)
        for _ in range(16):
            cand2, ecc2 = bfs_last(cand)
            if ecc2 <= ecc:
                break
            start, ecc, cand = cand, ecc2, cand2
        head = len(out)
        out.append(start)
        placed[start] = True
        while head < len(out):
            v = out[head]
            head += 1
            for w in nbrs[v]:
                if not placed[w]:
                    placed[w] = True
                    out.append(w)
    return np.array(out[::-1], dtype=np.int64)


def bandwidth(order, src, dst):
    inv = np.empty(len(order), np.int64)
    inv[order] = np.arange(len(order))
    return int(np.abs(inv[np.asarray(src)] - inv[np.asarray(dst)]).max()) if len(src) else 0
