"""SELL-32 matrices built from a ``Linsys`` and the fused PCG driver.

``SellMatrix.from_linsys`` turns ``A(x) = reducer(selector(x)*Ae) + x*Av``
into the slot-major SELL-32 layout of ``include/esr_gb300.h`` (rows = the
Reducer index, columns = the Selector index, entries of a row in the
reference's edge order).  ``FusedPCG`` runs (P)CG on it with the device-side
stopping test, launching iterations in chunks captured in a CUDA graph.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch

from .. import _lib, mesh


class SellMatrix:
    def __init__(self, n: int, slice_ptr: torch.Tensor, col: torch.Tensor, val: torch.Tensor, diag: torch.Tensor,
                 src_pos: Optional[torch.Tensor] = None):
        self.n = n
        self.slice_ptr = slice_ptr
        self.col = col
        self.val = val
        self.diag = diag
        self.src_pos = src_pos
        self.dtype = val.dtype
        self.device = val.device
        self.nnz = int((col >= 0).sum().item()) if col.numel() else 0
        self.desc = _lib.Sell(n, col.numel(), _lib.dtype_code(val.dtype), 0, _lib.ptr(slice_ptr), _lib.ptr(col),
                              _lib.ptr(val), _lib.ptr(diag))

    @staticmethod
    def layout(n: int, row_idx: np.ndarray, col_idx: np.ndarray):
        rowptr, perm = mesh.csr_from_index(row_idx, n)
        return mesh.sell_layout(n, rowptr, perm, col_idx, n)

    @classmethod
    def from_arrays(cls, n: int, row_idx: np.ndarray, col_idx: np.ndarray, Ae: torch.Tensor, Av: torch.Tensor,
                    dtype: Optional[torch.dtype] = None, layout=None) -> "SellMatrix":
        dev = Av.device
        dtype = dtype or Av.dtype
        slice_ptr, col, src_pos = layout if layout is not None else cls.layout(n, row_idx, col_idx)
        sp = torch.from_numpy(slice_ptr).to(dev)
        c = torch.from_numpy(col).to(dev)
        pos = torch.from_numpy(src_pos).to(dev)
        valid = pos >= 0
        ae = Ae.to(dev)
        val = torch.where(valid, ae[torch.where(valid, pos, torch.zeros_like(pos))],
                          torch.zeros(1, dtype=ae.dtype, device=dev)).to(dtype).contiguous()
        return cls(n, sp, c, val, Av.to(dtype).contiguous(), pos)

    @classmethod
    def from_linsys(cls, A, dtype: Optional[torch.dtype] = None) -> "SellMatrix":
        """The Linsys's current values; couplings whose Ae is exactly 0 are
        left out (they add exactly nothing to a row's sum of finite
        products; the solvers rebuild their plan when Ae changes).  For a
        vector x with an Inf or NaN the results differ from the
        reference's reducer(selector(x) * Ae), where 0 * Inf gives NaN:
        the packed SpMV is the reference's Linsys for finite x only (a
        solver that meets a non-finite value stops with a breakdown
        status either way)."""
        sel, red = A.selector, A.reducer
        n = A.Av.shape[0]
        if red.n != n:
            raise ValueError(f"Linsys reducer has n={red.n} rows but Av has {n}")
        row = red.idx.detach().cpu().numpy().astype(np.int64)
        col = sel.idx.detach().cpu().numpy().astype(np.int64)
        Ae = A.Ae.data
        keep = (Ae != 0).cpu().numpy()
        if not keep.all():
            row, col = row[keep], col[keep]
            Ae = Ae[torch.from_numpy(keep).to(Ae.device)]
        return cls.from_arrays(n, row, col, Ae, A.Av.data, dtype)

    def astype(self, dtype: torch.dtype) -> "SellMatrix":
        return SellMatrix(self.n, self.slice_ptr, self.col, self.val.to(dtype), self.diag.to(dtype), self.src_pos)

    def spmv(self, x: torch.Tensor, y: Optional[torch.Tensor] = None) -> torch.Tensor:
        """y = A x, bitwise the reference's Linsys.forward."""
        if y is None:
            y = torch.empty_like(x)
        _lib.call("esr_spmv", ctypes.byref(self.desc), _lib.ptr(x), _lib.ptr(y), _lib.stream_handle(self.device))
        return y

    def bytes_per_spmv(self) -> int:
        s = self.val.element_size()
        return self.col.numel() * (4 + s) + self.slice_ptr.numel() * 8 + self.n * (3 * s)


class FusedPCG:
    """Jacobi- or un-preconditioned CG on a SELL matrix (cg.py algorithm)."""

    def __init__(self, A: SellMatrix, jacobi: bool = False, chunk: int = 32, use_graph: bool = True):
        self.A = A
        self.n = A.n
        self.dev = A.device
        self.dtype = A.dtype
        self.invdiag = (1.0 / A.diag).contiguous() if jacobi else None
        self.ws = torch.zeros(int(_lib.lib().esr_cg_workspace_bytes(self.n)), dtype=torch.uint8, device=self.dev)
        self.q = torch.empty(self.n, dtype=self.dtype, device=self.dev)
        self.chunk = chunk
        self.use_graph = use_graph
        self._graphs = {}
        self.kernel_launches = 0

    def bytes_per_iteration(self) -> int:
        """Algorithmic HBM bytes of one iteration: the SpMV streams col, val,
        slice_ptr and diag, gathers p and writes q; the update reads x, r, p,
        q, invdiag and writes x, r, z; the p-update reads z, p and writes p."""
        s = self.A.val.element_size()
        return self.A.col.numel() * (4 + s) + self.A.slice_ptr.numel() * 8 + self.n * 14 * s

    def _iterate_call(self, x, r, z, p, k):
        _lib.call("esr_cg_iterate", ctypes.byref(self.A.desc), _lib.ptr(x), _lib.ptr(r), _lib.ptr(z), _lib.ptr(p),
                  _lib.ptr(self.q), _lib.ptr(self.invdiag), int(k), _lib.ptr(self.ws), _lib.stream_handle(self.dev))

    def _chunk(self, x, r, z, p, k):
        key = (x.data_ptr(), r.data_ptr(), z.data_ptr(), p.data_ptr(), k)
        if not self.use_graph:
            self._iterate_call(x, r, z, p, k)
            return
        g = self._graphs.get(key)
        if g is None:
            # capture on a side stream, as torch requires
            s = torch.cuda.Stream(self.dev)
            s.wait_stream(torch.cuda.current_stream(self.dev))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self._iterate_call(x, r, z, p, k)
            torch.cuda.current_stream(self.dev).wait_stream(s)
            self._graphs[key] = g
        g.replay()

    def scalars(self) -> _lib.CgScalars:
        out = _lib.CgScalars()
        _lib.call("esr_cg_read_scalars", _lib.ptr(self.ws), ctypes.byref(out), _lib.stream_handle(self.dev))
        return out

    def solve(self, b, x, r, z, p, rtol: float, atol: Optional[float], maxiter: Optional[int]) -> _lib.CgScalars:
        """Runs to convergence; x is updated in place.  Returns the final
        device scalars (iters = number of step() calls)."""
        _lib.call("esr_cg_init", ctypes.byref(self.A.desc), _lib.ptr(b), _lib.ptr(x), _lib.ptr(r), _lib.ptr(z),
                  _lib.ptr(p), _lib.ptr(self.invdiag), float(rtol), float(atol) if atol else 0.0,
                  -1 if maxiter is None else int(maxiter), _lib.ptr(self.ws), _lib.stream_handle(self.dev))
        self.kernel_launches += 1
        k = max(1, min(self.chunk, 8))
        while True:
            self._chunk(x, r, z, p, k)
            self.kernel_launches += 3 * k
            s = self.scalars()
            if s.done:
                return s
            k = min(self.chunk, 2 * k)

    def true_residual(self, b, x, r_scratch) -> float:
        out = torch.empty(1, dtype=torch.float64, device=self.dev)
        _lib.call("esr_true_residual", ctypes.byref(self.A.desc), _lib.ptr(b), _lib.ptr(x), _lib.ptr(r_scratch),
                  _lib.ptr(out), _lib.ptr(self.ws), _lib.stream_handle(self.dev))
        return float(out.item())


class MixedPCG:
    """FP32-SpMV / FP64-vector PCG with FP64 true-residual replacement.

    The SpMV runs on the FP32 pipes (FP32 matrix values and an FP32 copy of
    the search direction for the gathers); x, r, z, p, q and every dot
    product stay FP64 (an FP32 recurrence loses too much at the conditioning
    of these systems), and after every chunk of iterations the FP64 true
    residual b - A64 x replaces r (the search direction is kept, so CG does
    not restart) and decides convergence.
    """

    def __init__(self, A64: SellMatrix, jacobi: bool = True, chunk: int = 32, use_graph: bool = True):
        self.A64 = A64
        self.A32 = A64.astype(torch.float32)
        n, dev = A64.n, A64.device
        self.n, self.dev = n, dev
        self.invdiag = (1.0 / A64.diag).contiguous() if jacobi else None
        f64 = dict(dtype=torch.float64, device=dev)
        self.q = torch.empty(n, **f64)
        self.p32 = torch.empty(n, dtype=torch.float32, device=dev)
        self.ws = torch.zeros(int(_lib.lib().esr_cg_workspace_bytes(n)), dtype=torch.uint8, device=dev)
        self.chunk = chunk
        self.use_graph = use_graph
        self._graphs = {}
        self.kernel_launches = 0

    def bytes_per_iteration(self) -> int:
        """FP32 SpMV (col, val32, p32 gather, diag32) plus FP64 vectors: the
        update reads x, r, p, q, invdiag and writes x, r, z; the p-update
        reads z, p and writes p and p32; the chunk's true residual is
        amortised over ``chunk`` iterations."""
        A, n = self.A32, self.n
        spmv = A.col.numel() * 8 + A.slice_ptr.numel() * 8 + n * (4 + 4 + 8 + 8)
        vec = n * 8 * 8 + n * (8 * 3 + 4)
        tr = (self.A64.col.numel() * 12 + n * 8 * 4) / self.chunk
        return int(spmv + vec + tr)

    def _iterate_call(self, b, x, r, z, p):
        _lib.call("esr_cg_mixed_iterate", ctypes.byref(self.A64.desc), ctypes.byref(self.A32.desc), _lib.ptr(b),
                  _lib.ptr(x), _lib.ptr(r), _lib.ptr(z), _lib.ptr(p), _lib.ptr(self.p32), _lib.ptr(self.q),
                  _lib.ptr(self.invdiag), int(self.chunk), _lib.ptr(self.ws), _lib.stream_handle(self.dev))

    def _chunk(self, b, x, r, z, p):
        if not self.use_graph:
            self._iterate_call(b, x, r, z, p)
            return
        key = (b.data_ptr(), x.data_ptr(), r.data_ptr(), z.data_ptr(), p.data_ptr())
        g = self._graphs.get(key)
        if g is None:
            s = torch.cuda.Stream(self.dev)
            s.wait_stream(torch.cuda.current_stream(self.dev))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self._iterate_call(b, x, r, z, p)
            torch.cuda.current_stream(self.dev).wait_stream(s)
            self._graphs[key] = g
        g.replay()

    def scalars(self) -> _lib.CgScalars:
        out = _lib.CgScalars()
        _lib.call("esr_cg_read_scalars", _lib.ptr(self.ws), ctypes.byref(out), _lib.stream_handle(self.dev))
        return out

    def solve(self, b, x, r, z, p, rtol: float, atol: Optional[float], maxiter: Optional[int]) -> _lib.CgScalars:
        _lib.call("esr_cg_mixed_init", ctypes.byref(self.A64.desc), ctypes.byref(self.A32.desc), _lib.ptr(b),
                  _lib.ptr(x), _lib.ptr(r), _lib.ptr(z), _lib.ptr(p), _lib.ptr(self.p32), _lib.ptr(self.invdiag),
                  float(rtol), float(atol) if atol else 0.0, -1 if maxiter is None else int(maxiter),
                  _lib.ptr(self.ws), _lib.stream_handle(self.dev))
        self.kernel_launches += 2
        s = self.scalars()
        while not s.done:
            self._chunk(b, x, r, z, p)
            self.kernel_launches += 3 * self.chunk + 1
            s = self.scalars()
        return s


class FusedGMRES:
    """Restarted GMRES on a SELL matrix with M = Jacobi or identity
    (gmres.py algorithm): one CUDA graph per restart cycle, one 64-byte read
    of the device scalars per cycle for the host's stopping test."""

    def __init__(self, A: SellMatrix, restart: int, jacobi: bool = False, use_graph: bool = True):
        self.A = A
        self.n = A.n
        self.dev = A.device
        self.dtype = A.dtype
        self.restart = int(restart)
        self.invdiag = (1.0 / A.diag).contiguous() if jacobi else None
        nbytes = int(_lib.lib().esr_gmres_workspace_bytes(self.n, self.restart))
        if nbytes < 0:
            raise ValueError("fused GMRES supports restart <= 64")
        self.ws = torch.zeros(nbytes, dtype=torch.uint8, device=self.dev)
        self.V = torch.empty((self.restart, self.n), dtype=self.dtype, device=self.dev)
        self.w2 = torch.empty((2, self.n), dtype=self.dtype, device=self.dev)
        self.use_graph = use_graph
        self._graphs = {}
        self.kernel_launches = 0

    def launches_per_cycle(self) -> int:
        R = self.restart
        return 1 + R + R * (R + 1) // 2 + 3

    def scalars(self) -> _lib.GmresScalars:
        out = _lib.GmresScalars()
        _lib.call("esr_gmres_read", _lib.ptr(self.ws), ctypes.byref(out), _lib.stream_handle(self.dev))
        return out

    def _cycle_call(self, b, x, r):
        _lib.call("esr_gmres_cycle", ctypes.byref(self.A.desc), _lib.ptr(self.invdiag), _lib.ptr(b), _lib.ptr(x),
                  _lib.ptr(r), _lib.ptr(self.V), _lib.ptr(self.w2), self.restart, _lib.ptr(self.ws),
                  _lib.stream_handle(self.dev))

    def _cycle(self, b, x, r):
        self.kernel_launches += self.launches_per_cycle()
        if not self.use_graph:
            self._cycle_call(b, x, r)
            return
        key = (b.data_ptr(), x.data_ptr(), r.data_ptr())
        g = self._graphs.get(key)
        if g is None:
            s = torch.cuda.Stream(self.dev)
            s.wait_stream(torch.cuda.current_stream(self.dev))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self._cycle_call(b, x, r)
            torch.cuda.current_stream(self.dev).wait_stream(s)
            self._graphs[key] = g
        g.replay()

    def solve(self, b, x, r, rtol: float, atol: Optional[float], maxiter: Optional[int], log=None):
        """The reference's loop (gmres.py:229-266): residual, stopping test,
        one restart cycle per iteration.  Returns (scalars, iters)."""
        st = _lib.stream_handle(self.dev)
        _lib.call("esr_gmres_init", ctypes.byref(self.A.desc), _lib.ptr(b), float(rtol),
                  float(atol) if atol else 0.0, _lib.ptr(self.ws), st)
        _lib.call("esr_gmres_residual", ctypes.byref(self.A.desc), _lib.ptr(b), _lib.ptr(x), _lib.ptr(r),
                  _lib.ptr(self.ws), st)
        self.kernel_launches += 2
        iters = 0
        while True:
            s = self.scalars()
            if log is not None:
                log(iters, s.rnorm)
            if (s.rnorm == s.rnorm and s.rnorm <= s.tol) or (maxiter is not None and iters >= maxiter):
                return s, iters
            iters += 1
            self._cycle(b, x, r)
