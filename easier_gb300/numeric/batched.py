"""Batched (P)CG: many independent ``Linsys`` instances solved in lockstep.

The instances are packed as one block-diagonal SELL-32 system.  Each
instance's rows are padded to a multiple of 256 (identity rows, zero right
hand side), so every 256-row CTA of the device kernels belongs to exactly one
instance and every per-instance dot product is finished by the last CTA of
that instance (``include/esr_gb300.h``, ``esr_bcg_*``).  Per instance the
iteration and stopping test are those of easier/numeric/solver/cg.py:68-161
(Jacobi ``M`` or none).  Converged instances are re-checked on the FP64 true
residual ``b - A x``; an instance that fails restarts from it.

Two arithmetic precisions:

``"fp64"``  FP64 matrix, vectors and dots (the reference's precision);
``"df64"``  double-float pairs (two FP32 numbers per value, ~48 significand
            bits) for the matrix, vectors and dots, on the FP32 pipes, with the
            FP64 true residual deciding convergence.

A single system is a batch of one (``CG.solve(precision="df64")``).
"""
from __future__ import annotations

import atexit
import ctypes
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import torch

from .. import _lib, mesh

ROWS_PER_BLOCK = 256
STATUS = {0: "running", 1: "converged", 2: "maxiter", 3: "breakdown"}
# damping of the polynomial-Jacobi sweeps: fewest iterations on the P1
# Poisson family at degrees 2 and 4 (the classical 2/3 takes ~5% more
# iterations there, 1.0 ~20% more)
POLY_OMEGA = 0.8


@dataclass
class LinsysInstance:
    """One system in Linsys form: A x = reducer(x[col] * Ae) + x * Av with the
    Reducer index ``row``; ``b`` the right hand side, ``x0`` the start (zero
    when None).  Arrays are numpy or torch (any device)."""
    n: int
    row: np.ndarray
    col: np.ndarray
    Ae: object
    Av: object
    b: object
    x0: object = None
    edge_len: object = None  # per coupling, grid units (GNN edge input); 1 when None


def _np(a, dtype):
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(a, dtype=dtype))


def split_df64(t: torch.Tensor) -> torch.Tensor:
    """FP64 tensor -> [..., 2] FP32 pairs (hi, lo) with hi + lo == t to ~48 bits."""
    t = t.to(torch.float64)
    hi = t.to(torch.float32)
    lo = (t - hi.to(torch.float64)).to(torch.float32)
    return torch.stack([hi, lo], dim=-1).contiguous()


def join_df64(t: torch.Tensor) -> torch.Tensor:
    return t[..., 0].to(torch.float64) + t[..., 1].to(torch.float64)


class PackedBatch:
    """Host packing of instances into one block-diagonal SELL-32 system.

    Slices never span instances (256-row blocks, 32-row slices), so each
    instance's SELL layout is built on its own and the layouts concatenated
    with row/slot offsets.  Entries of a row keep the reference's edge order
    (stable sort of the Reducer index).  Without edge features, couplings
    whose Ae is exactly 0 are left out: they add exactly nothing to a row's
    sum of finite products (P1 grids: the hypotenuse couplings of right
    triangles, a third of all), so the SpMV moves and multiplies less for
    the same result (for finite vectors: the reference's 0 * Inf = NaN is
    not reproduced).  The GNN's message passing keeps them as graph edges."""

    def __init__(self, instances: Sequence[LinsysInstance], edge_features: bool = False):
        if len(instances) == 0:
            raise ValueError("empty batch")
        nblk = [max(1, -(-int(s.n) // ROWS_PER_BLOCK)) for s in instances]
        self.ninst = len(instances)
        self.sizes = np.array([int(s.n) for s in instances], np.int64)
        self.inst_block0 = np.zeros(self.ninst + 1, np.int32)
        self.inst_block0[1:] = np.cumsum(nblk)
        self.nblocks = int(self.inst_block0[-1])
        self.n = self.nblocks * ROWS_PER_BLOCK
        self.row0 = self.inst_block0[:-1].astype(np.int64) * ROWS_PER_BLOCK
        self.block_inst = np.repeat(np.arange(self.ninst, dtype=np.int32), nblk)
        sp_parts, col_parts, val_parts, w_parts, len_parts = [], [], [], [], []
        self.node_lk = np.zeros(self.n, np.float32) if edge_features else None
        self.diag = np.ones(self.n, np.float64)
        self.b = np.zeros(self.n, np.float64)
        self.x0 = np.zeros(self.n, np.float64)
        base = 0
        for i, s in enumerate(instances):
            n, r0, npad = int(s.n), int(self.row0[i]), nblk[i] * ROWS_PER_BLOCK
            row, col = _np(s.row, np.int64), _np(s.col, np.int64)
            Ae, Av = _np(s.Ae, np.float64), _np(s.Av, np.float64)
            if row.shape != col.shape or row.shape != Ae.shape or Av.shape != (n,):
                raise ValueError(f"instance {i}: inconsistent Linsys arrays")
            if not edge_features:
                keep = Ae != 0.0
                if not keep.all():
                    row, col, Ae = row[keep], col[keep], Ae[keep]
            rowptr, perm = mesh.csr_from_index(row, npad)
            slice_ptr, c, src_pos = mesh.sell_layout(npad, rowptr, perm, col, n)
            valid = src_pos >= 0
            val = np.where(valid, Ae[np.where(valid, src_pos, 0)], 0.0)
            sp_parts.append(slice_ptr[:-1] + base)
            col_parts.append(np.where(c >= 0, c + r0, -1).astype(np.int32))
            val_parts.append(val)
            if edge_features:
                from .preconditioner.gnn import node_input
                widths = np.diff(slice_ptr) // 32
                srow = (np.repeat(np.arange(len(widths), dtype=np.int64) * 32, widths * 32)
                        + np.arange(int(slice_ptr[-1]), dtype=np.int64) % 32)
                cc = np.where(valid, c, 0)
                rr = np.minimum(srow, max(n - 1, 0))
                w = np.where(valid, val / np.sqrt(Av[rr] * Av[cc]) if n else 0.0, 0.0)
                el = np.ones(len(val)) if s.edge_len is None else _np(s.edge_len, np.float64)[np.where(valid, src_pos, 0)]
                w_parts.append(w.astype(np.float32))
                len_parts.append(np.where(valid, el, 0.0).astype(np.float32))
                self.node_lk[r0:r0 + n] = node_input(Av).astype(np.float32)
            base += int(slice_ptr[-1])
            self.diag[r0:r0 + n] = Av
            self.b[r0:r0 + n] = _np(s.b, np.float64)
            if s.x0 is not None:
                self.x0[r0:r0 + n] = _np(s.x0, np.float64)
        if self.n >= 2 ** 31:
            raise ValueError("batch too large for int32 column indices")
        self.slice_ptr = np.concatenate(sp_parts + [np.array([base], np.int64)])
        self.col = np.concatenate(col_parts)
        self.val = np.concatenate(val_parts)
        self.edge_feat = (np.stack([np.concatenate(w_parts), np.concatenate(len_parts)], axis=1)
                          if edge_features else None)

    def rows(self, i: int) -> slice:
        r0 = int(self.row0[i])
        return slice(r0, r0 + int(self.sizes[i]))


def chunk_layout(inst_block0: np.ndarray, tiles_per_chunk: int):
    """Chunks of up to ``tiles_per_chunk`` consecutive tiles of one instance:
    chunk_tile0 [nchunks+1], chunk_inst [nchunks], inst_chunk0 [ninst+1]."""
    m = int(tiles_per_chunk)
    if m < 1:
        raise ValueError("tiles_per_chunk must be >= 1")
    ntiles = np.diff(inst_block0.astype(np.int64))
    nch = -(-ntiles // m)
    inst_chunk0 = np.zeros(len(ntiles) + 1, np.int64)
    inst_chunk0[1:] = np.cumsum(nch)
    chunk_inst = np.repeat(np.arange(len(ntiles), dtype=np.int64), nch)
    j = np.arange(int(inst_chunk0[-1])) - inst_chunk0[chunk_inst]
    chunk_tile0 = np.empty(int(inst_chunk0[-1]) + 1, np.int64)
    chunk_tile0[:-1] = inst_block0[chunk_inst].astype(np.int64) + j * m
    chunk_tile0[-1] = int(inst_block0[-1])
    return chunk_tile0.astype(np.int32), chunk_inst.astype(np.int32), inst_chunk0.astype(np.int32)


# Iterations between the GNN stall checks (no decrease of r.r over the
# window, or the network's correction cut in more than half of it -> the
# instance falls back to Jacobi-PCG).  Where the network does not help, the
# first check decides; a short window keeps the failed GNN iterations (each
# costing several Jacobi iterations) few.
GNN_STALL_WINDOW = 16


class BatchedPCG:
    """Lockstep (P)CG over a packed batch on one GPU.

    ``run`` enqueues iterations in groups of up to ``graph_iters``, each group
    one CUDA graph (1 compaction + 2 persistent launches per iteration in
    df64, 3 in FP64, 5 more with the GNN);
    between groups the host reads the 4-byte running-instance counter.
    The work shape -- 256-row tiles per CTA work unit (``tiles_per_chunk``)
    and persistent CTAs (``grid``) -- is set by ``autotune`` or by hand.

    ``poly_degree = d > 0`` replaces Jacobi by the polynomial-Jacobi
    preconditioner z = sum_{j<=d} (I - W A)^j W r, W = ``poly_omega``/diag:
    d+1 damped Jacobi sweeps on A z = r from z = 0, d SpMV sweeps per
    iteration (an even d keeps M SPD for any omega > 0)."""

    def __init__(self, instances: Sequence[LinsysInstance], jacobi: bool = True, precision: str = "df64",
                 device="cuda", graph_iters: int = 32, use_graph: bool = True, tiles_per_chunk: int = 4,
                 grid: Optional[int] = None, gnn=None, stall_window: int = None, gnn_ctas_per_sm: int = 2,
                 poly_degree: int = 0, poly_omega: float = POLY_OMEGA):
        if precision not in ("fp64", "df64"):
            raise ValueError("precision must be 'fp64' or 'df64'")
        dev = torch.device(device)
        if dev.type != "cuda":
            raise ValueError("BatchedPCG runs on a CUDA device")
        if gnn is not None and not jacobi:
            raise ValueError("the GNN preconditioner falls back to Jacobi: jacobi must be True")
        _drain_pending()
        poly_degree = int(poly_degree)
        if poly_degree:
            if not 2 <= poly_degree <= 16:
                raise ValueError("poly_degree must be 0 or in [2, 16]")
            if gnn is not None or not jacobi:
                raise ValueError("the polynomial preconditioner needs jacobi=True and no GNN")
            if not poly_omega > 0.0:
                raise ValueError("poly_omega must be positive")
        pk = PackedBatch(instances, edge_features=gnn is not None)
        self.pack = pk
        self.dev = dev
        self.precision = precision
        self.graph_iters = int(graph_iters)
        self.use_graph = use_graph
        self.jacobi = jacobi
        self.poly_degree = poly_degree
        self.poly_omega = float(poly_omega) if poly_degree else None
        n = pk.n
        t = lambda a: torch.from_numpy(a).to(dev)
        self.slice_ptr = t(pk.slice_ptr)
        self.col = t(pk.col)
        self.block_inst = t(pk.block_inst)
        self.inst_block0 = t(pk.inst_block0)
        self.val64 = t(pk.val)
        self.diag64 = t(pk.diag)
        self.b64 = t(pk.b)
        inv64 = ((self.poly_omega if poly_degree else 1.0) / self.diag64) if jacobi else None
        df = precision == "df64"
        conv = split_df64 if df else (lambda a: a.contiguous())
        self.val = conv(self.val64)
        self.diag = conv(self.diag64)
        self.invdiag = conv(inv64) if jacobi else None
        self.b = conv(self.b64)
        self.x = conv(t(pk.x0))
        self.r, self.z, self.p, self.q = (torch.zeros_like(self.x) for _ in range(4))
        self.poly_tmp = torch.zeros((2,) + tuple(self.x.shape), dtype=self.x.dtype, device=dev) \
            if poly_degree else None
        self.x64 = torch.zeros(n, dtype=torch.float64, device=dev)
        self.r64 = torch.zeros(n, dtype=torch.float64, device=dev)
        # sized for the finest chunking (one tile per chunk)
        nbytes = int(_lib.lib().esr_bcg_workspace_bytes(pk.ninst, pk.nblocks, pk.nblocks))
        self.ws = torch.zeros(nbytes, dtype=torch.uint8, device=dev)
        self.sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
        self._graphs = {}
        self._one_graphs = {}
        self.kernel_launches = 0
        self.polls = 0
        self.tuning = None
        self.gnn_desc = None
        if gnn is not None:
            self._gnn = gnn.device_tensors(dev)
            self._gnn["node_lk"] = t(pk.node_lk)
            self._gnn["edge_feat"] = t(pk.edge_feat)
            self._gnn["inst_rows"] = t(pk.sizes.astype(np.int32))
            self._gnn["h0"] = torch.zeros(n * 32, dtype=torch.bfloat16, device=dev)
            self._gnn["h1"] = torch.zeros(n * 32, dtype=torch.bfloat16, device=dev)
            g = self._gnn
            self.gnn_desc = _lib.Gnn(_lib.ptr(g["node_lk"]), _lib.ptr(g["edge_feat"]), _lib.ptr(g["inst_rows"]),
                                     _lib.ptr(g["h0"]), _lib.ptr(g["h1"]), _lib.ptr(g["enc_w"]), _lib.ptr(g["enc_b"]),
                                     _lib.ptr(g["layer_w"]), _lib.ptr(g["layer_b"]), _lib.ptr(g["dec_w"]),
                                     float(gnn.dec_b), int(gnn_ctas_per_sm * self.sm_count),
                                     int(GNN_STALL_WINDOW if stall_window is None else stall_window), 0)
        self.set_shape(tiles_per_chunk, grid if grid is not None else 4 * self.sm_count)

    def set_shape(self, tiles_per_chunk: int, grid: int):
        """Work unit of the persistent kernels (tiles per chunk) and their
        CTA count."""
        ct0, cinst, ic0 = chunk_layout(self.pack.inst_block0, tiles_per_chunk)
        self.tiles_per_chunk = int(tiles_per_chunk)
        self.grid = int(grid)
        self.nchunks = len(cinst)
        self.chunk_tile0 = torch.from_numpy(ct0).to(self.dev)
        self.chunk_inst = torch.from_numpy(cinst).to(self.dev)
        self.inst_chunk0 = torch.from_numpy(ic0).to(self.dev)
        pk = self.pack
        self.desc = _lib.Batch(pk.n, pk.ninst, pk.nblocks, ROWS_PER_BLOCK, 1 if self.precision == "df64" else 0,
                               self.nchunks, self.grid, _lib.ptr(self.slice_ptr), _lib.ptr(self.col),
                               _lib.ptr(self.val), _lib.ptr(self.diag), _lib.ptr(self.invdiag),
                               _lib.ptr(self.val64), _lib.ptr(self.diag64), _lib.ptr(self.block_inst),
                               _lib.ptr(self.inst_block0), _lib.ptr(self.chunk_tile0), _lib.ptr(self.chunk_inst),
                               _lib.ptr(self.inst_chunk0),
                               ctypes.pointer(self.gnn_desc) if self.gnn_desc is not None else None,
                               _lib.ptr(self.poly_tmp), self.poly_degree, 0)
        self._graphs = {}
        self._free_graphs()

    def bytes_per_row_iteration(self) -> float:
        """Algorithmic HBM bytes of one lockstep iteration per active packed
        row (8-byte values in both precisions): the SpMV streams col and val
        (per stored slot) and diag; 14 vector touches: df64 gathers z, reads
        p, q and writes p, q (one sweep); FP64 gathers p and writes q, then
        reads z, p and writes p (two sweeps); both then read x, r, p, q,
        invdiag and write x, r, z.  Each polynomial sweep streams the matrix
        and diag again, reads y_in, r, W and writes y_out."""
        slots = self.pack.slice_ptr[-1] / self.pack.n
        return slots * 12 + 8 * 14 + 8 / 32 + self.poly_degree * (slots * 12 + 8 * 5 + 8 / 32)

    def load_packed(self, b64: Optional[torch.Tensor] = None, x0: Optional[torch.Tensor] = None):
        """Replace the packed right hand side and/or start vector (FP64,
        length n, padding rows zero)."""
        conv = split_df64 if self.precision == "df64" else (lambda a: a)
        if b64 is not None:
            self.b64.copy_(b64)
            self.b.copy_(conv(self.b64))
        if x0 is not None:
            self.x.copy_(conv(x0.to(self.dev, torch.float64)))

    # ------------------------------------------------------------- calls --
    def _stream(self):
        return _lib.stream_handle(self.dev)

    def _iterate_call(self, k: int):
        _lib.call("esr_bcg_iterate", ctypes.byref(self.desc), _lib.ptr(self.x), _lib.ptr(self.r), _lib.ptr(self.z),
                  _lib.ptr(self.p), _lib.ptr(self.q), int(k), _lib.ptr(self.ws), self._stream())

    def _group(self, k: int):
        per_it = (2 if self.precision == "df64" else 3) + (5 if self.gnn_desc is not None else 0) + self.poly_degree
        self.kernel_launches += 1 + per_it * k
        if not self.use_graph:
            self._iterate_call(k)
            return
        g = self._graphs.get(k)
        if g is None:
            s = torch.cuda.Stream(self.dev)
            s.wait_stream(torch.cuda.current_stream(self.dev))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self._iterate_call(k)
            torch.cuda.current_stream(self.dev).wait_stream(s)
            self._graphs[k] = g
        g.replay()

    def active(self) -> int:
        a = ctypes.c_int32()
        _lib.call("esr_bcg_status", _lib.ptr(self.ws), self.pack.ninst, self.nchunks, ctypes.byref(a), None,
                  self._stream())
        self.polls += 1
        return int(a.value)

    def instances(self) -> List[_lib.BcgInst]:
        a = ctypes.c_int32()
        out = (_lib.BcgInst * self.pack.ninst)()
        _lib.call("esr_bcg_status", _lib.ptr(self.ws), self.pack.ninst, self.nchunks, ctypes.byref(a), out,
                  self._stream())
        return list(out)

    def reset(self, x0: Optional[torch.Tensor] = None):
        """Start vector for the next solve: the packed x0 (default) or a
        packed FP64 tensor of length n."""
        src = torch.from_numpy(self.pack.x0).to(self.dev) if x0 is None else x0.to(self.dev, torch.float64)
        self.x.copy_(split_df64(src) if self.precision == "df64" else src)

    def load_instance(self, i: int, b: Optional[torch.Tensor] = None, x0: Optional[torch.Tensor] = None):
        """Replace instance i's right hand side and/or start vector (FP64,
        length = the instance's size) in the packed device vectors."""
        rows = self.pack.rows(i)
        conv = split_df64 if self.precision == "df64" else (lambda a: a)
        if b is not None:
            b = b.to(self.dev, torch.float64)
            self.b64[rows] = b
            self.b[rows] = conv(b)
        if x0 is not None:
            self.x[rows] = conv(x0.to(self.dev, torch.float64))

    # ---------------------------------------------------------- autotune --
    def autotune(self, tiles=(2, 4, 8, 16, 32, 64), ctas_per_sm=(2, 3, 4, 6, 8), iters: int = 8,
                 reps: int = 2) -> dict:
        """Times ``iters`` lockstep iterations (every instance running) for
        each (tiles per chunk, persistent CTAs per SM) pair on this batch and
        keeps the fastest.  Leaves x untouched; the next ``run`` starts from
        scratch.  Results are cached per batch signature in-process."""
        key = (self.precision, self.pack.n, self.pack.ninst, int(self.pack.slice_ptr[-1]), self.jacobi,
               self.poly_degree)
        hit = _TUNE_CACHE.get(key)
        if hit is not None:
            self.set_shape(hit["tiles_per_chunk"], hit["grid"])
            self.tuning = dict(hit, cached=True)
            return self.tuning
        x_keep = self.x.clone()
        stream = torch.cuda.current_stream(self.dev)
        table = []
        for m in tiles:
            for c in ctas_per_sm:
                self.set_shape(m, c * self.sm_count)
                self.start(0.0, None, None)
                self._iterate_call(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                best = float("inf")
                for _ in range(reps):
                    e0.record(stream)
                    self._iterate_call(iters)
                    e1.record(stream)
                    e1.synchronize()
                    best = min(best, e0.elapsed_time(e1) / iters)
                table.append({"tiles_per_chunk": m, "ctas_per_sm": c, "ms_per_iter": best,
                              "units_per_cta": self.nchunks / self.grid})
        self.x.copy_(x_keep)
        # (the timing has every instance running; rules that favour finer
        # chunks for the tail of a batch cost more on single systems than
        # they gain on batches: the fastest shape wins)
        win = min(table, key=lambda r: r["ms_per_iter"])
        res = {"tiles_per_chunk": win["tiles_per_chunk"], "grid": win["ctas_per_sm"] * self.sm_count,
               "ms_per_iter": win["ms_per_iter"], "table": table}
        _TUNE_CACHE[key] = res
        self.set_shape(res["tiles_per_chunk"], res["grid"])
        self.tuning = dict(res, cached=False)
        return self.tuning

    # ------------------------------------------------------------- solve --
    def start(self, rtol: float, atol: Optional[float], maxiter: Optional[int]):
        _lib.call("esr_bcg_init", ctypes.byref(self.desc), _lib.ptr(self.b64), _lib.ptr(self.b), _lib.ptr(self.x),
                  _lib.ptr(self.r), _lib.ptr(self.z), _lib.ptr(self.p), float(rtol), float(atol) if atol else 0.0,
                  -1 if maxiter is None else int(maxiter), _lib.ptr(self.ws), self._stream())
        self.kernel_launches += 1

    def apply_preconditioner(self, r: torch.Tensor, z: Optional[torch.Tensor] = None) -> torch.Tensor:
        """z = M(r) with the GNN preconditioner for every instance (packed
        vectors in the engine's precision); overwrites the solver state."""
        if self.gnn_desc is None:
            raise ValueError("no GNN preconditioner attached")
        z = torch.empty_like(r) if z is None else z
        _lib.call("esr_gnn_apply", ctypes.byref(self.desc), _lib.ptr(r), _lib.ptr(z), _lib.ptr(self.ws),
                  self._stream())
        self.kernel_launches += 6
        return z

    def verify(self):
        _lib.call("esr_bcg_verify", ctypes.byref(self.desc), _lib.ptr(self.b64), _lib.ptr(self.x),
                  _lib.ptr(self.x64), _lib.ptr(self.r64), _lib.ptr(self.r), _lib.ptr(self.z), _lib.ptr(self.p),
                  _lib.ptr(self.ws), self._stream())
        self.kernel_launches += 4

    def run(self, rtol: float = 1e-8, atol: Optional[float] = None, maxiter: Optional[int] = None,
            max_rounds: int = 16) -> int:
        """Device part of a solve; returns the number of verification rounds."""
        self.start(rtol, atol, maxiter)
        k = min(8, self.graph_iters)
        rounds = 0
        while True:
            active = self.active()
            while active > 0:
                self._group(k)
                k = min(self.graph_iters, 2 * k)
                active = self.active()
            self.verify()
            rounds += 1
            if self.active() == 0 or rounds >= max_rounds:
                if self.gnn_desc is not None:
                    from .. import ops
                    bits = ops.device_status(clear=True)
                    if bits & _lib.DEV_WAIT_TIMEOUT:
                        raise RuntimeError("a GNN tensor-core wait timed out on the device")
                return rounds

    # ------------------------------------------------- one-launch solve --
    def solve_graph(self, rtol: float = 1e-8, atol: Optional[float] = None, maxiter: int = 100000,
                    k: Optional[int] = None) -> List[dict]:
        """The whole solve as ONE CUDA graph launch (esr_bcg_graph_create):
        init, then a device-side loop of k-iteration bodies with the FP64
        verification, until no instance runs.  maxiter must be finite (it
        also bounds the device loop).  The graph is built once per
        (rtol, atol, maxiter, k) and work shape."""
        k = int(k or self.graph_iters)
        key = (float(rtol), float(atol or 0.0), int(maxiter), k, self.tiles_per_chunk, self.grid)
        g = self._one_graphs.get(key)
        if g is None:
            h = ctypes.c_void_p()
            _lib.call("esr_bcg_graph_create", ctypes.byref(self.desc), _lib.ptr(self.b64), _lib.ptr(self.b),
                      _lib.ptr(self.x), _lib.ptr(self.r), _lib.ptr(self.z), _lib.ptr(self.p), _lib.ptr(self.q),
                      _lib.ptr(self.x64), _lib.ptr(self.r64), float(rtol), float(atol) if atol else 0.0,
                      int(maxiter), k, _lib.ptr(self.ws), ctypes.byref(h))
            g = self._one_graphs[key] = h
        _lib.call("esr_bcg_graph_launch", g, self._stream())
        self.kernel_launches += 1
        return [self._info(s) for s in self.instances()]

    def _free_graphs(self):
        graphs = getattr(self, "_one_graphs", {})
        self._one_graphs = {}
        if graphs:
            _destroy_graphs(list(graphs.values()), self.dev)
        _drain_pending()

    def __del__(self):
        # the collector can run this while some stream is being captured
        # into a CUDA graph, where a synchronisation or a graph teardown
        # would invalidate that capture: the handles wait for a safe point
        # (the next engine call that frees graphs, or interpreter exit)
        graphs, captured = getattr(self, "_one_graphs", {}), getattr(self, "_graphs", {})
        if graphs or captured:  # (the torch graphs are released there too)
            _PENDING_GRAPHS.append((list(graphs.values()), getattr(self, "dev", None), list(captured.values())))
            self._one_graphs, self._graphs = {}, {}

    def solve(self, rtol: float = 1e-8, atol: Optional[float] = None, maxiter: Optional[int] = None,
              max_rounds: int = 16) -> List[dict]:
        """Solves every instance to ``||r|| <= max(rtol*||b||, atol)`` and
        returns one dict per instance: status, iters (reference counting:
        step() calls - 1), the final recurrence residual, the FP64 true
        residual and the number of residual replacements."""
        self.run(rtol, atol, maxiter, max_rounds)
        return [self._info(s) for s in self.instances()]

    @staticmethod
    def _info(s) -> dict:
        status = STATUS.get(s.done, "?")
        if s.done == 1 and s.verified != 1:
            status = "unverified"
        tr = float(s.true_rr) ** 0.5 if s.true_rr >= 0 else float("nan")
        return {"status": status, "iters": max(int(s.iters) - 1, 0), "residual": float(s.rr) ** 0.5,
                "true_residual": tr, "bnorm": float(s.bnorm), "tol": float(s.tol), "restarts": int(s.restarts),
                "mode": "gnn" if s.mode == 1 else "jacobi", "fallbacks": int(s.fallbacks),
                "fallback_iter": int(s.gnn_iters), "clips": int(s.clips)}

    def solution(self, i: Optional[int] = None) -> torch.Tensor:
        """FP64 solution of instance i (all packed rows when None)."""
        x = join_df64(self.x) if self.precision == "df64" else self.x
        return x if i is None else x[self.pack.rows(i)]


_TUNE_CACHE: dict = {}
_PENDING_GRAPHS: list = []  # (graph handles, device, torch graphs) of collected engines


def _destroy_graphs(handles, dev) -> None:
    try:  # no launch of them may still be running
        torch.cuda.synchronize(dev)
    except Exception:  # interpreter shutdown
        pass
    for h in handles:
        try:
            _lib.call("esr_bcg_graph_destroy", h)
        except Exception:  # interpreter shutdown
            pass


def _drain_pending() -> None:
    while _PENDING_GRAPHS:
        handles, dev, captured = _PENDING_GRAPHS.pop()
        _destroy_graphs(handles, dev)
        del captured


atexit.register(_drain_pending)


def p1_sides(count: int, nmin: int, nmax: int, seed: int = 0) -> np.ndarray:
    """Mesh sides of a seeded batch: N ~ U{nmin..nmax}."""
    return np.random.default_rng(seed).integers(nmin, nmax + 1, count)


def p1_instance(i: int, n: int, seed: int = 0, corr_len: float = 0.1, variance: float = 1.0) -> LinsysInstance:
    """Instance i of a seeded batch, of side n: kappa = exp(g) with g a
    Gaussian random field (field seed 100003 * seed + 2i), 16-mode random
    right hand side (seed 100003 * seed + 2i + 1)."""
    kappa = mesh.kappa_from_field(mesh.gaussian_random_field(n, seed * 100_003 + 2 * i, corr_len, variance))
    s = mesh.p1_system(n, kappa)
    b = mesh.random_mode_rhs(n, seed * 100_003 + 2 * i + 1)
    return LinsysInstance(s.nunk, s.row, s.col, s.Ae, s.Av, b, edge_len=p1_edge_length(n, s.row, s.col))


def p1_instances(count: int, nmin: int, nmax: int, seed: int = 0, corr_len: float = 0.1,
                 variance: float = 1.0) -> List[LinsysInstance]:
    """Seeded batch of P1 Poisson instances: side N ~ U{nmin..nmax},
    kappa = exp(g) with g a Gaussian random field (correlation length
    corr_len, variance), 16-mode random right hand side."""
    return [p1_instance(i, int(n), seed, corr_len, variance) for i, n in enumerate(p1_sides(count, nmin, nmax, seed))]


def p1_edge_length(n: int, row: np.ndarray, col: np.ndarray) -> np.ndarray:
    """Length (grid units) of each coupling of the P1 grid system: unknown
    u = (j-1)*(n-1) + (i-1) sits at node (i, j)."""
    m = max(n - 1, 1)
    di = (col % m) - (row % m)
    dj = (col // m) - (row // m)
    return np.sqrt((di * di + dj * dj).astype(np.float64))


def main(argv: Optional[Sequence[str]] = None) -> None:
    """Solve P1 Poisson systems on the batched engine and print one line per
    solve: ``--grid N`` one constant-coefficient system (16-mode right hand
    side, seed 0), else a seeded batch (``--count/--nmin/--nmax/--seed``);
    ``--shape TILES,GRID`` fixes the work shape (default: autotune)."""
    import argparse
    import time
    ap = argparse.ArgumentParser(prog="python -m easier_gb300.numeric.batched")
    ap.add_argument("--grid", type=int, default=None)
    ap.add_argument("--count", type=int, default=16)
    ap.add_argument("--nmin", type=int, default=32)
    ap.add_argument("--nmax", type=int, default=512)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", choices=["fp64", "df64"], default="df64")
    ap.add_argument("--shape", default=None)
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--repeat", type=int, default=2)
    args = ap.parse_args(argv)
    if args.grid:
        s = mesh.p1_system(args.grid)
        insts = [LinsysInstance(s.nunk, s.row, s.col, s.Ae, s.Av, mesh.random_mode_rhs(args.grid, 0))]
    else:
        insts = p1_instances(args.count, args.nmin, args.nmax, args.seed)
    eng = BatchedPCG(insts, jacobi=True, precision=args.precision)
    if args.shape:
        t, g = (int(v) for v in args.shape.split(","))
        eng.set_shape(t, g)
    else:
        eng.autotune()
    for _ in range(args.repeat):
        eng.reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = eng.solve(rtol=args.rtol)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        ok = sum(r["status"] == "converged" for r in res)
        print(f"{len(res)} systems, {ok} converged, {dt * 1e3:.1f} ms, max iterations {max(r['iters'] for r in res)}, "
              f"replacements {sum(r['restarts'] for r in res)}, shape {eng.tiles_per_chunk},{eng.grid}", flush=True)


if __name__ == "__main__":
    main()
