"""Fused engine for the shallow-water step.

``compile`` offers every module to ``try_install``.  A module qualifies when
it has the shallow-water layout of tutorial/shallow_water_equation/
swe_main.py:13-84 (cell tensors h, uh, vh, area; edge tensors sx, sy, alpha;
wall tensors bsx, bsy; Selectors gather_src, gather_dst, gather_b; Reducers
scatter(dst, nc) and scatter_b(bcells, nc); a float ``dt``) with consistent
indices, and when one fused step reproduces one step of its own ``forward``
(run on the per-op path) bit for bit on a random state.  The fused engine
then replaces ``forward``; anything that does not qualify keeps the per-op
path.

Data layout built here (world size 1):
  * cells renumbered by reverse Cuthill-McKee over the edge graph, so the
    neighbours a warp gathers sit close together (L1/L2 reuse);
  * each cell's in-edges in the reference's edge order (a stable sort by
    destination, the order sparse_encoding.py:244-338 gives the edge group),
    then its wall faces, in ``width`` face slots stored slot-major;
  * the state (h, uh, vh) packed per cell in one [nc, 4] buffer; the
    module's ``h``/``uh``/``vh`` become views of it, in RCM order, with
    ``elempart`` recording the original index of every row, so
    ``Tensor.collect()`` returns the original order as in the reference.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional

import numpy as np
import torch

from . import _lib, mesh
from . import module as _m
from .utils import logger

CELL = ("h", "uh", "vh", "area")
EDGE = ("sx", "sy", "alpha")
WALL = ("bsx", "bsy")
SELECTORS = ("gather_src", "gather_dst", "gather_b")
REDUCERS = ("scatter", "scatter_b")


def bind(m) -> Optional[dict]:
    """Role binding of a shallow-water module, or None."""
    try:
        t = {k: getattr(m, k) for k in CELL + EDGE + WALL}
        s = {k: getattr(m, k) for k in SELECTORS}
        r = {k: getattr(m, k) for k in REDUCERS}
        dt = getattr(m, "dt")
    except AttributeError:
        return None
    if not all(isinstance(v, _m.Tensor) and v.is_partition for v in t.values()):
        return None
    if not all(isinstance(v, _m.Selector) for v in s.values()) or not all(isinstance(v, _m.Reducer) for v in r.values()):
        return None
    if not isinstance(dt, (float, int)) or isinstance(dt, bool):
        return None
    dtype = t["h"].dtype
    if dtype not in (torch.float32, torch.float64) or any(v.dtype != dtype for v in t.values()):
        return None
    if any(v.dim() != 1 for v in t.values()):
        return None
    nc = t["h"].shape[0]
    ne = s["gather_src"].idx.shape[0]
    nbc = s["gather_b"].idx.shape[0]
    if any(t[k].shape[0] != nc for k in CELL) or any(t[k].shape[0] != ne for k in EDGE) \
            or any(t[k].shape[0] != nbc for k in WALL):
        return None
    if s["gather_dst"].idx.shape[0] != ne or r["scatter"].idx.shape[0] != ne or r["scatter_b"].idx.shape[0] != nbc:
        return None
    if r["scatter"].n != nc or r["scatter_b"].n != nc or r["scatter"].reduce != "sum" or r["scatter_b"].reduce != "sum":
        return None
    if not torch.equal(r["scatter"].idx, s["gather_dst"].idx) or not torch.equal(r["scatter_b"].idx, s["gather_b"].idx):
        return None
    if s["gather_src"]._idx_max >= nc:
        return None
    return dict(tensors=t, selectors=s, reducers=r, nc=nc, ne=ne, nbc=nbc, dtype=dtype)


class SweEngine:
    """The fused step of one shallow-water module."""

    def __init__(self, module, binding: dict, reorder: str = "rcm"):
        self.m = module
        self.b = binding
        self.reorder = reorder
        self.dtype = binding["dtype"]
        self.device = binding["tensors"]["h"].device
        self.nc = binding["nc"]
        self._graph = None
        self._build_layout()

    # ----------------------------------------------------------- layout --
    def _build_layout(self) -> None:
        b = self.b
        nc, ne, nbc = b["nc"], b["ne"], b["nbc"]
        src = b["selectors"]["gather_src"].idx.cpu().numpy().astype(np.int64)
        dst = b["selectors"]["gather_dst"].idx.cpu().numpy().astype(np.int64)
        bcell = b["selectors"]["gather_b"].idx.cpu().numpy().astype(np.int64)
        if self.reorder == "rcm" and nc > 1:
            order = mesh.rcm_order(nc, src, dst)
        else:
            order = np.arange(nc, dtype=np.int64)
        inv = np.empty(nc, np.int64)
        inv[order] = np.arange(nc, dtype=np.int64)
        nd = inv[dst]
        rowptr, perm = mesh.csr_from_index(nd, nc)
        nb = inv[bcell]
        browptr, bperm = mesh.csr_from_index(nb, nc)
        deg = np.diff(rowptr)
        bdeg = np.diff(browptr)
        total = deg + bdeg
        wmax = int(total.max()) if nc else 0
        if wmax > 4:
            raise NotImplementedError(f"a cell has {wmax} faces; the fused kernel handles at most 4")
        width = 3 if wmax <= 3 else 4
        # slot position of every sorted edge / wall face
        cell_of_edge = nd[perm]
        k_edge = np.arange(ne, dtype=np.int64) - rowptr[cell_of_edge]
        cell_of_wall = nb[bperm]
        k_wall = deg[cell_of_wall] + (np.arange(nbc, dtype=np.int64) - browptr[cell_of_wall])
        nbr = np.full((width, nc), -2, np.int32)
        nbr[k_edge, cell_of_edge] = inv[src[perm]].astype(np.int32)
        nbr[k_wall, cell_of_wall] = -1
        # where each slot's values come from: edge e -> e, wall face b -> ne + b
        pos = np.full((width, nc), -1, np.int64)
        pos[k_edge, cell_of_edge] = perm
        pos[k_wall, cell_of_wall] = ne + bperm
        self.width = width
        self.order_np = order
        self.order = torch.from_numpy(order).to(self.device)
        self.nbr = torch.from_numpy(nbr).to(self.device)
        self.slot_pos = torch.from_numpy(pos).to(self.device)
        self._fill_geometry()
        self._pack_state()
        self.ws = torch.empty(3 * 4 * nc, dtype=self.dtype, device=self.device)

    def _fill_geometry(self) -> None:
        t = self.b["tensors"]
        pos = self.slot_pos
        valid = pos >= 0
        safe = torch.where(valid, pos, torch.zeros_like(pos))
        zero = torch.zeros(1, dtype=self.dtype, device=self.device)
        fx = torch.cat([t["sx"].data, t["bsx"].data])
        fy = torch.cat([t["sy"].data, t["bsy"].data])
        al = torch.cat([t["alpha"].data, torch.zeros(self.b["nbc"], dtype=self.dtype, device=self.device)])
        self.sx = torch.where(valid, fx[safe], zero).contiguous()
        self.sy = torch.where(valid, fy[safe], zero).contiguous()
        self.alpha = torch.where(valid, al[safe], zero).contiguous()
        area = t["area"]
        if area.elempart is None:
            area.data = area.data[self.order].contiguous()
            area.elempart = self.order
        self.area = area.data
        self._geom_versions = self._versions()
        self._mesh = _lib.SweMesh(self.nc, self.width, _lib.dtype_code(self.dtype), _lib.ptr(self.nbr),
                                  _lib.ptr(self.sx), _lib.ptr(self.sy), _lib.ptr(self.alpha), _lib.ptr(self.area))

    def _versions(self):
        t = self.b["tensors"]
        return tuple((t[k].data.data_ptr(), t[k]._version) for k in EDGE + WALL + ("area",))

    def _pack_state(self) -> None:
        t = self.b["tensors"]
        state = torch.zeros((self.nc, 4), dtype=self.dtype, device=self.device)
        for j, k in enumerate(("h", "uh", "vh")):
            v = t[k]
            state[:, j] = v.data if v.elempart is not None else v.data[self.order]
        self.state = state
        for j, k in enumerate(("h", "uh", "vh")):
            t[k].data = state[:, j]
            t[k].elempart = self.order
        self._state_ptrs = tuple(t[k].data.data_ptr() for k in ("h", "uh", "vh"))

    def reorder_other_cell_tensors(self) -> None:
        """Other partitioned tensors of the module with nc rows (e.g. the
        centroid coordinates x, y) follow the cell renumbering."""
        bound = set(id(v) for v in self.b["tensors"].values())
        for _, p in self.m.named_parameters(recurse=False):
            if isinstance(p, _m.Tensor) and id(p) not in bound and p.is_partition and p.easier_data_ready \
                    and p.dim() >= 1 and p.shape[0] == self.nc and p.elempart is None:
                p.data = p.data[self.order].contiguous()
                p.elempart = self.order

    # ---------------------------------------------------------- running --
    def _sync_inputs(self) -> None:
        if self._versions() != self._geom_versions:
            self._fill_geometry()
        t = self.b["tensors"]
        if tuple(t[k].data.data_ptr() for k in ("h", "uh", "vh")) != self._state_ptrs:
            raise RuntimeError("the shallow-water state tensors were replaced after compile(); write into them in place")

    def step(self, steps: int = 1) -> None:
        """`steps` fused steps on torch's current stream."""
        self._sync_inputs()
        _lib.call("esr_swe_step", ctypes.byref(self._mesh), float(self.m.dt), _lib.ptr(self.state), int(steps),
                  _lib.ptr(self.ws), _lib.stream_handle(self.device))

    def forward(self):
        self.step(1)

    def delta(self, state: torch.Tensor) -> torch.Tensor:
        """One `delta` evaluation on a [nc, 4] state (RCM order)."""
        out = torch.empty_like(state)
        _lib.call("esr_swe_delta", ctypes.byref(self._mesh), _lib.ptr(state), _lib.ptr(out),
                  _lib.stream_handle(self.device))
        return out

    def describe(self) -> str:
        return f"nc={self.nc} width={self.width} dtype={str(self.dtype).replace('torch.', '')} reorder={self.reorder}"

    def workload_bytes_per_step(self) -> int:
        """Algorithmic HBM bytes of one step (4 stage kernels), counting
        every array each kernel must touch once."""
        s = 8 if self.dtype == torch.float64 else 4
        nc, w = self.nc, self.width
        geom = nc * (w * (4 + 3 * s) + s)          # slots + area, every stage
        st = 4 * s * nc                             # one [nc,4] state array
        k1 = geom + st + 2 * st                     # s0 in; S1, A out
        k2 = geom + 3 * st + 2 * st                 # S1, s0, A in; S2, A out
        k3 = k2
        k4 = geom + 3 * st + st                     # S1, s0, A in; s0 out
        return k1 + k2 + k3 + k4


def _shared_with_others(m, modules) -> bool:
    mine = set(id(o) for o in _m.get_easier_objects([m]) if not isinstance(o, _m.Module))
    for other in modules:
        if other is m:
            continue
        for o in _m.get_easier_objects([other]):
            if not isinstance(o, _m.Module) and id(o) in mine:
                return True
    return False


def _verify(m, eng: SweEngine, binding: dict) -> bool:
    """One fused step vs one per-op step of the module's own forward, from
    the same random state; bitwise equality required."""
    t = binding["tensors"]
    nc, dtype, dev = binding["nc"], binding["dtype"], eng.device
    g = torch.Generator(device="cpu").manual_seed(1234)
    h0 = (1.0 + 0.05 * torch.rand(nc, generator=g, dtype=torch.float64)).to(dtype).to(dev)
    u0 = (0.01 * torch.randn(nc, generator=g, dtype=torch.float64)).to(dtype).to(dev)
    v0 = (0.01 * torch.randn(nc, generator=g, dtype=torch.float64)).to(dtype).to(dev)
    saved = {k: (t[k].data, t[k].elempart) for k in ("h", "uh", "vh", "area")}
    state_saved = eng.state.clone()
    order = eng.order
    try:
        # per-op path, original order
        area_orig = torch.empty_like(t["area"].data)
        area_orig[order] = t["area"].data
        t["area"].data, t["area"].elempart = area_orig, None
        for k, v in zip(("h", "uh", "vh"), (h0, u0, v0)):
            t[k].data, t[k].elempart = v.clone(), None
        type(m).forward(m)
        ref = [t[k].data.clone() for k in ("h", "uh", "vh")]
    finally:
        for k, (d, e) in saved.items():
            t[k].data, t[k].elempart = d, e
    # fused path, RCM order
    eng.state[:, 0] = h0[order]
    eng.state[:, 1] = u0[order]
    eng.state[:, 2] = v0[order]
    eng._fill_geometry()
    eng.step(1)
    out = eng.state[:, :3].clone()
    eng.state.copy_(state_saved)
    torch.cuda.synchronize(dev)
    ok = True
    for j, k in enumerate(("h", "uh", "vh")):
        fused = torch.empty_like(ref[j])
        fused[order] = out[:, j]
        if not torch.equal(fused, ref[j]):
            diff = (fused - ref[j]).abs().max().item()
            logger.warning(f"fused shallow-water step differs from the module's forward on {k} (max |diff| {diff:.3e});"
                           " keeping the per-op path")
            ok = False
    return ok


def try_install(m, modules: List) -> Optional[SweEngine]:
    binding = bind(m)
    if binding is None:
        return None
    reorder = "none" if _shared_with_others(m, modules) else "rcm"
    try:
        eng = SweEngine(m, binding, reorder=reorder)
    except NotImplementedError as e:
        logger.info(f"{type(m).__name__}: not fused ({e})")
        return None
    if not _verify(m, eng, binding):
        # undo the renumbering of the bound tensors
        for k in ("h", "uh", "vh", "area"):
            v = binding["tensors"][k]
            if v.elempart is not None:
                v.data = v.collect().to(v.device)
                v.elempart = None
        return None
    eng.reorder_other_cell_tensors()
    m.forward = eng.forward
    m.easier_fused_engine = eng
    return eng
