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

Two kernels, same arithmetic, bitwise-equal results:

* **tiled** (FP32, 3 faces per cell; the default there): one launch per
  step.  Cells are grouped in compact tiles of <= ``tile_cells`` cells by
  recursive BFS bisection; each CTA holds its tile plus the 4 rings of
  in-neighbours the 4 stages depend on in shared memory and recomputes the
  halo instead of exchanging stage states through HBM.
* **staged** (FP64, or wider cells): one launch per stage, stage states in
  HBM.

Data layout (world size 1):
  * cells renumbered by reverse Cuthill-McKee over the edge graph (staged) or
    tile-major with RCM order inside each tile (tiled);
  * each cell's in-edges in the reference's edge order (a stable sort by
    destination, the order sparse_encoding.py:244-338 gives the edge group),
    then its wall faces, in face slots stored slot-major;
  * the state (h, uh, vh) packed per cell in [nc, 4] buffers; the module's
    ``h``/``uh``/``vh`` are views of the current buffer, with ``elempart``
    recording the original index of every row, so ``Tensor.collect()``
    returns the original order as in the reference.
"""
from __future__ import annotations

import atexit
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
STATE = ("h", "uh", "vh")

TILE_CELLS = 4096       # tile size cap (kernel limit: 4096 own cells)
TILE_MIN_CELLS = 256
TILE_TARGET = 3500      # large meshes: measured best at N=2000 (3,300-3,900 within 4%)
# Target tile size; None = auto: one tile per SM while the mesh is small,
# TILE_TARGET on large meshes.  Tiles of <= 1024 / 2048 own cells run 4 / 2
# CTAs per SM.
DEFAULT_TILE_CELLS: Optional[int] = None
TILE_MAX_L3 = 6144      # kernel limit on tile + 3 halo rings
TILE_SMEM = 227 * 1024  # shared memory per CTA
DEFAULT_MODE = "auto"   # "auto" (tiled for FP32), "tiled" or "staged"
# Numbering before the tile partition of a tiled layout: "rcm" (reverse
# Cuthill-McKee, then tile-major) or "tiles" (the module's own order, then
# tile-major: the partition alone, without the RCM pass).  Measured at
# N=2000: the same kernel time (0.454 vs 0.457 ms), 2 s less compile.
TILED_REORDER = "tiles"
# numbering of a staged (FP64) layout: "none" (the module's own order; built
# on the device) or "rcm" (reverse Cuthill-McKee, a host pass).  Measured at
# N=2000 on the tutorial mesh: the same step time (21.3 / 8.29 ms exact /
# fast), 0.37 instead of 5.7 s of setup.
STAGED_REORDER = "none"
# build the tiled layout of a CUDA engine on the GPU (esr_bisect_partition_device
# and torch sorts); False: the host functions (same arrays for the same
# partition; the host partition itself differs, see esr_bisect_partition_device)
LAYOUT_ON_DEVICE = True
# Fast arithmetic on large meshes: tiles for the pipelined tile kernel
# (<= 2048 own cells, <= 4096 local cells)
PIPE_TILE_TARGET = 2000  # measured at N=2000: 0.427-0.429 ms; 1,900: 0.434; 2,048: 0.431; 1,800: 0.437
PIPE_LIMITS = dict(max_own=2048, max_local=4096)
# pieces a host-resident state moves in per step (step_host)
HOST_CHUNKS = 8
# tile kernel: "auto" (pipelined where the layout allows), "blocked",
# "pipelined" (its shape from the tile size), "pipelined_512", "pipelined_768"
DEFAULT_TILE_KERNEL = "auto"
_TILE_KERNELS = {"auto": 0, "blocked": 1, "pipelined": 2, "pipelined_512": 3, "pipelined_768": 4}
DEFAULT_PRECISION = "exact"  # "exact" (bitwise the reference) or "fast"
# compile-time check of the fast arithmetic: one step from a random state,
# max |fused - per-op| per component over max |h|
FAST_STEP_RTOL = {torch.float32: 2e-6, torch.float64: 1e-13}


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
    return dict(tensors=t, selectors=s, reducers=r, nc=nc, ne=ne, nbc=nbc, dtype=dtype, dt_attr="dt")


def find_roles(m) -> Optional[dict]:
    """Role binding of a shallow-water module whose attributes are not named
    like the tutorial's, found from its structure and checked on its own
    forward.

    Structure: two sum Reducers onto the same n cells (the longer index =
    the interior edges' destinations, the shorter = the wall cells), a
    Selector with each of their indices (gather of the destination cell /
    of the wall cell) and one more Selector over the edges (the source
    cell); three float edge tensors, two wall tensors, cell tensors and a
    float step size among the module's attributes.  The three cell tensors
    forward() writes are the state.  Every assignment of the remaining
    roles (state order, area, the edge and wall tensors' order, dt) is then
    run through one step of the staged fused kernel in exact arithmetic and
    compared bit for bit with one step of forward() from the same random
    state; the binding is the first assignment that matches, or None."""
    import itertools
    sels = [v for v in m._modules.values() if isinstance(v, _m.Selector)]
    reds = [v for v in m._modules.values() if isinstance(v, _m.Reducer)]
    if len(sels) != 3 or len(reds) != 2 or any(r.reduce != "sum" for r in reds) or reds[0].n != reds[1].n:
        return None
    if any(getattr(x, "easier_index_status", None) != "rewritten" for x in sels + reds):
        return None
    nc = reds[0].n
    scat, scat_b = sorted(reds, key=lambda r: -r.idx.shape[0])
    ne, nbc = scat.idx.shape[0], scat_b.idx.shape[0]
    if ne == nbc:
        return None
    g_dst = [x for x in sels if x.idx.shape[0] == ne and torch.equal(x.idx, scat.idx)]
    g_b = [x for x in sels if x.idx.shape[0] == nbc and torch.equal(x.idx, scat_b.idx)]
    if not g_dst or not g_b:
        return None
    g_src = [x for x in sels if x is not g_dst[0] and x is not g_b[0] and x.idx.shape[0] == ne]
    if len(g_src) != 1 or g_src[0]._idx_max >= nc:
        return None
    params = [v for v in m._parameters.values() if isinstance(v, _m.Tensor) and v.is_partition and v.dim() == 1]
    dtype = next((v.dtype for v in params if v.shape[0] == nc), None)
    if dtype not in (torch.float32, torch.float64):
        return None
    of = lambda n: [v for v in params if v.shape[0] == n and v.dtype == dtype]  # noqa: E731
    cells, edges, walls = of(nc), of(ne), of(nbc)
    dts = [(k, v) for k, v in vars(m).items() if isinstance(v, float) and not k.startswith("_")]
    if len(cells) < 4 or len(edges) != 3 or len(walls) != 2 or not dts or cells[0].device.type != "cuda":
        return None
    dev = cells[0].device
    saved = [(v, v.data) for v in cells]
    gen = torch.Generator(device="cpu").manual_seed(4321)
    try:
        # which cell tensors forward() writes: the state
        for v in cells:
            v.data = (1.0 + 0.05 * torch.rand(nc, generator=gen, dtype=torch.float64)).to(dtype).to(dev)
        before = [v.data.clone() for v in cells]
        type(m).forward(m)
        state = [v for v, b in zip(cells, before) if not torch.equal(v.data, b)]
        if len(state) != 3:
            return None
        for v, d in saved:
            v.data = d
        # the reference step: forward() from a random state
        inputs = [(1.0 + 0.05 * torch.rand(nc, generator=gen, dtype=torch.float64)).to(dtype).to(dev)
                  for _ in state]
        for v, x in zip(state, inputs):
            v.data = x.clone()
        type(m).forward(m)
        ref = [v.data.clone() for v in state]
    except Exception:  # not a forward we can run this way
        return None
    finally:
        for v, d in saved:
            v.data = d
    src = g_src[0].idx.cpu().numpy().astype(np.int64)
    dst = g_dst[0].idx.cpu().numpy().astype(np.int64)
    bcell = g_b[0].idx.cpu().numpy().astype(np.int64)
    lay = cell_layout(nc, src, dst, bcell, reorder="none")
    pos = torch.from_numpy(lay["pos"]).to(dev)
    nbr = torch.from_numpy(lay["nbr"]).to(dev)
    valid = pos >= 0
    safe = torch.where(valid, pos, torch.zeros_like(pos))
    zero = torch.zeros(1, dtype=dtype, device=dev)
    ws = torch.empty(3 * 4 * nc, dtype=dtype, device=dev)
    others = [v for v in cells if not any(v is x for x in state)]
    for order in itertools.permutations(range(3)):
        for area in others:
            for e in itertools.permutations(edges):
                for w in itertools.permutations(walls):
                    fx = torch.where(valid, torch.cat([e[0].data, w[0].data])[safe], zero).contiguous()
                    fy = torch.where(valid, torch.cat([e[1].data, w[1].data])[safe], zero).contiguous()
                    al = torch.where(valid, torch.cat([e[2].data, torch.zeros(nbc, dtype=dtype, device=dev)])[safe],
                                     zero).contiguous()
                    ar = area.data.contiguous()
                    mesh_d = _lib.SweMesh(nc, lay["width"], _lib.dtype_code(dtype), _lib.ptr(nbr), _lib.ptr(fx),
                                          _lib.ptr(fy), _lib.ptr(al), _lib.ptr(ar), _lib.ptr(ar), 1, 0)
                    for dt_name, dt in dts:
                        st = torch.zeros((nc, 4), dtype=dtype, device=dev)
                        for j in range(3):
                            st[:, j] = inputs[order[j]]
                        _lib.call("esr_swe_step", ctypes.byref(mesh_d), float(dt), _lib.ptr(st), 1, _lib.ptr(ws),
                                  _lib.stream_handle(dev))
                        if all(torch.equal(st[:, j], ref[order[j]]) for j in range(3)):
                            t = dict(zip(STATE, (state[i] for i in order)))
                            t.update(area=area, sx=e[0], sy=e[1], alpha=e[2], bsx=w[0], bsy=w[1])
                            return dict(tensors=t, selectors=dict(gather_src=g_src[0], gather_dst=g_dst[0],
                                                                  gather_b=g_b[0]),
                                        reducers=dict(scatter=scat, scatter_b=scat_b), nc=nc, ne=ne, nbc=nbc,
                                        dtype=dtype, dt_attr=dt_name)
    return None


class SweEngine:
    """The fused step of one shallow-water module."""

    def __init__(self, module, binding: dict, reorder: str = "rcm", mode: str = "auto",
                 tile_cells: Optional[int] = None, precision: str = "exact"):
        if precision not in ("exact", "fast"):
            raise ValueError(f"precision must be 'exact' or 'fast', not {precision!r}")
        self.precision = precision
        self.m = module
        self.b = binding
        self.reorder = reorder
        self.dtype = binding["dtype"]
        self.device = binding["tensors"]["h"].device
        self.nc = binding["nc"]
        self.tile_cells = min(tile_cells or DEFAULT_TILE_CELLS or self._auto_tile_cells(), TILE_CELLS)
        self.mode = mode
        self.tile_kernel = DEFAULT_TILE_KERNEL
        self._host_plan = None
        self._host_stage = None
        self._dt_attr = binding.get("dt_attr", "dt")
        self._build_layout()

    def _auto_tile_cells(self) -> int:
        """Largest tiles (least halo work) while there are enough of them to
        give every SM one."""
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count if self.device.type == "cuda" else 1
        target = PIPE_TILE_TARGET if self.precision == "fast" else TILE_TARGET
        return max(TILE_MIN_CELLS, min(target, -(-self.nc // sms)))

    @staticmethod
    def _pipe_fits(st: dict) -> bool:
        return all(st[k] <= v for k, v in PIPE_LIMITS.items())

    # ----------------------------------------------------------- layout --
    def _build_layout(self) -> None:
        b = self.b
        nc = b["nc"]
        sel = b["selectors"]
        idx = [sel[k].idx for k in ("gather_src", "gather_dst", "gather_b")]
        ph = self.setup_phases = _Phases(self.device)
        want_tiles = self.mode in ("tiled", "auto") and self.dtype == torch.float32
        tiles = None
        tile_cells = self.tile_cells
        pipe_tries = 0
        while True:
            # self.reorder "rcm": renumbering allowed (the layout picks the order)
            reorder = self.reorder if self.reorder != "rcm" else (TILED_REORDER if want_tiles else STAGED_REORDER)
            self.layout_order = reorder
            # the tiled layout of a CUDA engine is built on the GPU (partition,
            # slots, rings); RCM numberings are a host pass
            on_gpu = self.device.type == "cuda" and reorder != "rcm" and LAYOUT_ON_DEVICE
            src, dst, bcell = ([a.to(self.device, torch.int64) for a in idx] if on_gpu else
                               [a.cpu().numpy().astype(np.int64) for a in idx])
            lay = cell_layout(nc, src, dst, bcell, reorder=reorder,
                              tile_cells=tile_cells if want_tiles else None)
            ph.mark("partition_and_slots")
            if lay["part"] is None:
                break
            tiles = tile_layout(lay["nbr"], lay["part"])
            ph.mark("tile_lists")
            if self.precision == "fast" and reorder != "rcm":
                # a few over-wide tiles: cut them rather than shrink every tile
                for _ in range(2):
                    if tiles["stats"]["max_own"] > PIPE_LIMITS["max_own"]:
                        break
                    split = split_wide_tiles(lay, tiles, PIPE_LIMITS["max_local"])
                    if split is None:
                        break
                    lay = cell_layout(nc, src, dst, bcell, reorder=reorder, part=split)
                    tiles = tile_layout(lay["nbr"], lay["part"])
                    ph.mark("wide_tile_split")
            st = tiles["stats"]
            if st["max_own"] <= TILE_CELLS and st["max_l3"] <= TILE_MAX_L3 and st["smem"] <= TILE_SMEM:
                # fast arithmetic: smaller tiles until the pipelined kernel takes them
                if self.precision != "fast" or self._pipe_fits(st) or pipe_tries >= 4:
                    break
                pipe_tries += 1
                tile_cells = max(TILE_MIN_CELLS, int(tile_cells * 0.85))
                continue
            # halo too large for one CTA: smaller tiles, else the staged kernel
            tiles = None
            if tile_cells > 512:
                tile_cells //= 2
                continue
            want_tiles = False
        self.tile_cells = tile_cells
        order, nbr, pos, width = lay["order"], lay["nbr"], lay["pos"], lay["width"]
        tiled = tiles is not None
        self.order = _to(order, self.device)
        self.width = width
        self.nbr = _to(nbr, self.device)
        self.slot_pos = _to(pos, self.device)
        self.tiled = tiled
        if tiled:
            self._build_tiles(tiles)
        ph.mark("record_order")
        self._fill_geometry()
        ph.mark("geometry_records")
        nbuf = 2 if tiled else 1
        self.bufs = [torch.zeros((nc, 4), dtype=self.dtype, device=self.device) for _ in range(nbuf)]
        self.cur = 0
        self._pack_state()
        self.ws = None if tiled else torch.empty(3 * 4 * nc, dtype=self.dtype, device=self.device)
        ph.mark("state_buffers")

    def _build_tiles(self, lay: dict) -> None:
        st = lay["stats"]
        dev = self.device
        self.tile_meta = _to(lay["meta"], dev).reshape(-1).contiguous()
        self.tile_off3 = _to(lay["off3"], dev)
        self.tile_offh = _to(lay["offh"], dev)
        halo = _to(lay["halo"], dev)
        self.tile_halo = halo if halo.numel() else torch.zeros(1, dtype=torch.int32, device=dev)
        self.tile_lnbr = _to(lay["lnbr"], dev)
        self.tile_gsrc = _to(lay["slot_src"], dev)
        self.tile_area_src = _to(lay["area_src"], dev)
        self.tile_fast_order = _to(_slots_by_neighbour(lay["meta"], lay["off3"], lay["lnbr"]), dev)
        self.ntiles = st["ntiles"]
        self.tile_stats = st

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
        self.inv_area = (1.0 / self.area).contiguous()
        exact = 1 if self.precision == "exact" else 0
        self._geom_versions = self._versions()
        self._mesh = _lib.SweMesh(self.nc, self.width, _lib.dtype_code(self.dtype), _lib.ptr(self.nbr),
                                  _lib.ptr(self.sx), _lib.ptr(self.sy), _lib.ptr(self.alpha), _lib.ptr(self.area),
                                  _lib.ptr(self.inv_area), exact, 0)
        if self.tiled:
            src = self.tile_gsrc
            # one 16-byte record per tile face slot: sx, sy, alpha, lnbr bits;
            # fast arithmetic: sx / area, sy / area of the slot's cell
            fx, fy = self.sx.reshape(-1)[src], self.sy.reshape(-1)[src]
            if not exact:
                inv = self.inv_area[src % self.nc]
                fx, fy = fx * inv, fy * inv
            self.t_slots = torch.stack([fx, fy, self.alpha.reshape(-1)[src], self.tile_lnbr.view(torch.float32)],
                                       dim=1)
            if not exact:  # order the cell's faces by neighbour (the sums' order is free)
                self.t_slots = self.t_slots[self.tile_fast_order]
            self.t_slots = self.t_slots.contiguous()
            self.t_area = self.area[self.tile_area_src].contiguous()
            self.t_inv_area = self.inv_area[self.tile_area_src].contiguous()
            st = self.tile_stats
            self._tiles = _lib.SweTiles(self.nc, self.ntiles, _lib.F32, st["max_local"], st["max_l3"],
                                        st["max_own"], st["max_halo3"], _lib.ptr(self.tile_meta),
                                        _lib.ptr(self.tile_off3), _lib.ptr(self.tile_offh), _lib.ptr(self.tile_halo),
                                        _lib.ptr(self.t_slots), _lib.ptr(self.t_area), _lib.ptr(self.t_inv_area),
                                        exact, st["slot_info"])

    def set_precision(self, precision: str) -> None:
        """Switch between 'exact' and 'fast' arithmetic (same layout)."""
        if precision not in ("exact", "fast"):
            raise ValueError(f"precision must be 'exact' or 'fast', not {precision!r}")
        self.precision = precision
        self._fill_geometry()

    def _versions(self):
        t = self.b["tensors"]
        return tuple((t[k].data.data_ptr(), t[k]._version) for k in EDGE + WALL + ("area",))

    @property
    def state(self) -> torch.Tensor:
        return self.bufs[self.cur]

    def _bind_views(self) -> None:
        t = self.b["tensors"]
        for j, k in enumerate(STATE):
            t[k].data = self.state[:, j]
            t[k].elempart = self.order
        self._state_ptrs = tuple(t[k].data.data_ptr() for k in STATE)

    def _pack_state(self) -> None:
        t = self.b["tensors"]
        for j, k in enumerate(STATE):
            v = t[k]
            self.state[:, j] = v.data if v.elempart is not None else v.data[self.order]
        self._bind_views()

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
        if tuple(t[k].data.data_ptr() for k in STATE) != self._state_ptrs:
            raise RuntimeError("the shallow-water state tensors were replaced after compile(); write into them in place")

    def step(self, steps: int = 1) -> None:
        """`steps` fused steps on torch's current stream."""
        self._sync_inputs()
        stream = _lib.stream_handle(self.device)
        if self.tiled:
            a, b = self.bufs[self.cur], self.bufs[1 - self.cur]
            _lib.call("esr_swe_tile_step_with", ctypes.byref(self._tiles), _TILE_KERNELS[self.tile_kernel],
                      self.dt, _lib.ptr(a), _lib.ptr(b), int(steps), stream)
            if steps % 2:
                self.cur = 1 - self.cur
                self._bind_views()
        else:
            _lib.call("esr_swe_step", ctypes.byref(self._mesh), self.dt, _lib.ptr(self.state), int(steps),
                      _lib.ptr(self.ws), stream)

    def forward(self):
        self.step(1)

    def delta(self, state: torch.Tensor) -> torch.Tensor:
        """One `delta` evaluation on a [nc, 4] state (engine order)."""
        out = torch.empty_like(state)
        _lib.call("esr_swe_delta", ctypes.byref(self._mesh), _lib.ptr(state), _lib.ptr(out),
                  _lib.stream_handle(self.device))
        return out

    def step_host(self, host: torch.Tensor, steps: int = 1, chunks: int = HOST_CHUNKS) -> None:
        """Advance a state kept in host memory: ``host`` is FP32 (h, uh, vh)
        [nc, 3] in the engine's cell numbering (``self.order``), updated in
        place (pinned memory lets the copies overlap).  Every step uploads
        it, runs one fused step and brings the result back, in ``chunks``
        pieces so that uploads and downloads share the host link both ways
        (esr_swe_host_step); with the pipelined kernel the step's tiles also
        run in groups as their chunks land.  Returns once ``host`` holds the
        result; the engine's device state then holds it too."""
        if not self.tiled:
            raise NotImplementedError("host-resident stepping needs the tiled FP32 layout")
        if (host.dtype != torch.float32 or tuple(host.shape) != (self.nc, 3) or host.is_cuda
                or not host.is_contiguous()):
            raise ValueError(f"host state must be a contiguous CPU float32 tensor of shape ({self.nc}, 3)")
        self._sync_inputs()  # (may rebuild the geometry records the plan points to)
        key = (self.t_slots.data_ptr(), self.bufs[0].data_ptr(), self.bufs[1].data_ptr(), int(chunks))
        if self._host_plan is None or self._host_plan[0] != key:
            self._free_host_plan()
            if self._host_stage is None:
                self._host_stage = torch.empty((self.nc, 3), dtype=torch.float32, device=self.device)
                self._host_tiles = torch.empty(self.ntiles, dtype=torch.int32, device=self.device)
            h = ctypes.c_void_p()
            _lib.call("esr_swe_host_plan_create", ctypes.byref(self._tiles), _lib.ptr(self.bufs[0]),
                      _lib.ptr(self.bufs[1]), _lib.ptr(self._host_stage), _lib.ptr(self._host_tiles), int(chunks),
                      ctypes.byref(h))
            self._host_plan = (key, h)
        stream = torch.cuda.current_stream(self.device)
        _lib.call("esr_swe_host_step", self._host_plan[1], self.dt, _lib.ptr(host), int(steps),
                  _lib.stream_handle(self.device))
        stream.synchronize()
        self.cur = 1
        self._bind_views()

    def _free_host_plan(self) -> None:
        if getattr(self, "_host_plan", None) is not None:
            _destroy_host_plan(self._host_plan[1])
        self._host_plan = None
        _drain_host_plans()

    def __del__(self):
        # the destroy synchronises the plan's copy streams, which must not
        # happen while some stream is being captured into a CUDA graph: the
        # collector queues the plan for the next safe point instead
        plan = getattr(self, "_host_plan", None)
        if plan is not None:
            _PENDING_HOST_PLANS.append(plan[1])
            self._host_plan = None

    def launches_per_step(self) -> int:
        return 1 if self.tiled else 4

    def tile_threads(self) -> int:
        """Threads per CTA of the tiled step (1024 / that many CTAs per SM)."""
        return int(_lib.lib().esr_swe_tile_threads(ctypes.byref(self._tiles))) if self.tiled else 0

    def describe(self) -> str:
        s = (f"nc={self.nc} width={self.width} dtype={str(self.dtype).replace('torch.', '')} "
             f"kernel={'tiled' if self.tiled else 'staged'} precision={self.precision} "
             f"reorder={self.layout_order if not self.tiled else ('rcm+tiles' if self.layout_order == 'rcm' else 'tiles')}")
        if self.tiled:
            st = self.tile_stats
            s += (f" tiles={st['ntiles']} own<={st['max_own']} L3/own={st['l3_over_own']:.3f}"
                  f" local/own={st['local_over_own']:.3f} smem={st['smem']}"
                  f" cta={self.tile_threads()} kernel={self.tile_kernel_name()}")
        return s

    @property
    def dt(self) -> float:
        """The module's step size (read at every step, as its forward does)."""
        return float(getattr(self.m, self._dt_attr))

    def tile_kernel_name(self) -> str:
        """The tile kernel step() runs: 'pipelined_512', 'pipelined_768' or
        'blocked'."""
        if not self.tiled:
            return ""
        k = _TILE_KERNELS[self.tile_kernel]
        if k in (0, 2):
            auto = int(_lib.lib().esr_swe_tile_kernel(ctypes.byref(self._tiles)))
            k = auto if k == 0 or auto != 1 else 2
        return {1: "blocked", 2: "pipelined", 3: "pipelined_512", 4: "pipelined_768"}.get(k, "?")

    def touched_bytes_per_step(self) -> int:
        """HBM bytes one step must move in this layout, each array once."""
        s = 8 if self.dtype == torch.float64 else 4
        nc, w = self.nc, self.width
        if self.tiled:
            st = self.tile_stats
            l3 = st["l3_over_own"] * nc
            loc = st["local_over_own"] * nc
            geom = l3 * (48 + (4 if self.precision == "exact" else 0))
            halo_idx = (loc - nc) * 4
            return int(geom + halo_idx + loc * 16 + nc * 16 + self.ntiles * 48)
        geom = nc * (w * (4 + 3 * s) + s)
        st = 4 * s * nc
        k1 = geom + st + 2 * st
        k2 = geom + 3 * st + 2 * st
        k4 = geom + 3 * st + st
        return k1 + 2 * k2 + k4

    def bytes_model(self) -> str:
        """The byte count touched_bytes_per_step() makes, in words."""
        if self.tiled:
            return ("per step: three 16-byte face records of every cell of halo level <= 3 (sx, sy, alpha, local "
                    "neighbour" + ("; plus its area" if self.precision == "exact" else "; sx, sy pre-divided by the "
                    "area") + "), the 16-byte state of every cell of level <= 4 and the 4-byte global index of "
                    "each halo cell, the 16-byte new state of every cell, 48 bytes of tile metadata")
        return ("per stage launch: face slots (neighbour index, sx, sy, alpha) and area of every cell, the stage "
                "state in, the base state and the delta sum in and out, the stage state out")

    def traffic_key(self) -> str:
        """Key of this kernel variant's measured DRAM bytes per launch."""
        return f"swe_tiled_{self.tile_kernel_name()}_{self.precision}"


_PENDING_HOST_PLANS: list = []  # host-stepping plans of collected engines


def _destroy_host_plan(handle) -> None:
    try:
        _lib.call("esr_swe_host_plan_destroy", handle)
    except Exception:  # interpreter shutdown
        pass


def _drain_host_plans() -> None:
    while _PENDING_HOST_PLANS:
        _destroy_host_plan(_PENDING_HOST_PLANS.pop())


atexit.register(_drain_host_plans)


class _Phases:
    """Wall time of the setup phases (the device synchronised at each
    boundary, so asynchronous work is charged to its own phase)."""

    def __init__(self, device):
        import time
        self._time = time.perf_counter
        self._dev = device if device.type == "cuda" else None
        self.times = {}
        self._sync()
        self._t = self._time()

    def _sync(self):
        if self._dev is not None:
            torch.cuda.synchronize(self._dev)

    def mark(self, name: str) -> None:
        self._sync()
        t = self._time()
        self.times[name] = self.times.get(name, 0.0) + (t - self._t)
        self._t = t


def _to(a, dev) -> torch.Tensor:
    return a.to(dev) if isinstance(a, torch.Tensor) else torch.from_numpy(a).to(dev)


def slot_width(nc: int, nd: np.ndarray, nb: np.ndarray) -> int:
    total = np.bincount(nd, minlength=nc) + np.bincount(nb, minlength=nc)
    wmax = int(total.max()) if total.size else 0
    if wmax > 4:
        raise NotImplementedError(f"a cell has {wmax} faces; the fused kernels handle at most 4")
    return 3 if wmax <= 3 else 4


def cell_layout(nc: int, src: np.ndarray, dst: np.ndarray, bcell: np.ndarray, reorder: str = "rcm",
                tile_cells: Optional[int] = None, part=None) -> dict:
    """Cell numbering and face slots of the fused step.

    order[new] = original cell.  RCM numbering, or (tile_cells given and 3
    faces per cell) tile-major numbering with RCM order inside each tile,
    tiles from recursive BFS bisection.  nbr [width, nc]: neighbour (new
    numbering), -1 wall, -2 empty; slots hold a cell's in-edges in the
    reference's edge order, then its wall faces.  pos [width, nc]: source of
    each slot's values (edge e -> e, wall face b -> ne + b, none -> -1).
    ``part`` (reorder 'tiles' or 'none'): the tile of every cell, instead of
    the bisection."""
    if isinstance(src, torch.Tensor) and src.is_cuda:
        return _cell_layout_device(nc, src, dst, bcell, reorder, tile_cells, part)
    if part is not None and reorder == "rcm":
        raise ValueError("a given partition needs the module's own numbering")
    ne, nbc = src.shape[0], bcell.shape[0]
    order = mesh.rcm_order(nc, src, dst) if (reorder == "rcm" and nc > 1) else np.arange(nc, dtype=np.int64)
    inv = np.empty(nc, np.int64)
    inv[order] = np.arange(nc, dtype=np.int64)
    width = slot_width(nc, inv[dst], inv[bcell])
    if (tile_cells is not None or part is not None) and width == 3 and nc > 0:
        if part is None:
            part, _ = mesh.bisect_partition(nc, inv[src], inv[dst], tile_cells)
        part = np.asarray(part, dtype=np.int64)
        tmajor = np.argsort(part, kind="stable")
        order = order[tmajor]
        part = part[tmajor]
        inv[order] = np.arange(nc, dtype=np.int64)
    else:
        part = None
    nd = inv[dst]
    rowptr, perm = mesh.csr_from_index(nd, nc)
    nb = inv[bcell]
    browptr, bperm = mesh.csr_from_index(nb, nc)
    deg = np.diff(rowptr)
    cell_of_edge = nd[perm]
    k_edge = np.arange(ne, dtype=np.int64) - rowptr[cell_of_edge]
    cell_of_wall = nb[bperm]
    k_wall = deg[cell_of_wall] + (np.arange(nbc, dtype=np.int64) - browptr[cell_of_wall])
    nbr = np.full((width, nc), -2, np.int32)
    nbr[k_edge, cell_of_edge] = inv[src[perm]].astype(np.int32)
    nbr[k_wall, cell_of_wall] = -1
    pos = np.full((width, nc), -1, np.int64)
    pos[k_edge, cell_of_edge] = perm
    pos[k_wall, cell_of_wall] = ne + bperm
    return dict(order=order, nbr=nbr, pos=pos, width=width, part=part)


def _cell_layout_device(nc: int, src: torch.Tensor, dst: torch.Tensor, bcell: torch.Tensor, reorder: str,
                        tile_cells: Optional[int], part=None) -> dict:
    """cell_layout on the GPU (CUDA tensors in and out) for the module's own
    numbering ('tiles' or 'none'; RCM is a host pass): the partition from
    esr_bisect_partition_device, the rest the same torch operations as the
    numpy ones (a stable sort is the stable CSR of esr_csr_from_index)."""
    if reorder == "rcm":
        raise ValueError("the device cell layout keeps the module's numbering ('tiles' or 'none')")
    dev = src.device
    src, dst, bcell = (a.to(dev, torch.int64) for a in (src, dst, bcell))
    ne, nbc = src.shape[0], bcell.shape[0]
    ar = torch.arange(nc, dtype=torch.int64, device=dev)
    order, inv = ar, ar
    total = torch.bincount(dst, minlength=nc) + torch.bincount(bcell, minlength=nc)
    wmax = int(total.max()) if nc else 0
    if wmax > 4:
        raise NotImplementedError(f"a cell has {wmax} faces; the fused kernels handle at most 4")
    width = 3 if wmax <= 3 else 4
    if (tile_cells is not None or part is not None) and width == 3 and nc > 0:
        if part is None:
            part, _ = mesh.bisect_partition(nc, src, dst, tile_cells)
        part = torch.as_tensor(part, device=dev).to(torch.int64)
        order = torch.sort(part, stable=True).indices
        part = part[order]
        inv = torch.empty_like(order)
        inv[order] = ar
    else:
        part = None
    nd, nb = inv[dst], inv[bcell]
    rowptr, perm = mesh._stable_csr_device(nd, nc)
    browptr, bperm = mesh._stable_csr_device(nb, nc)
    rowptr, perm, browptr, bperm = (a.to(torch.int64) for a in (rowptr, perm, browptr, bperm))
    deg = rowptr[1:] - rowptr[:-1]
    cell_of_edge = nd[perm]
    k_edge = torch.arange(ne, dtype=torch.int64, device=dev) - rowptr[cell_of_edge]
    cell_of_wall = nb[bperm]
    k_wall = deg[cell_of_wall] + (torch.arange(nbc, dtype=torch.int64, device=dev) - browptr[cell_of_wall])
    nbr = torch.full((width, nc), -2, dtype=torch.int32, device=dev)
    nbr[k_edge, cell_of_edge] = inv[src[perm]].to(torch.int32)
    nbr[k_wall, cell_of_wall] = -1
    pos = torch.full((width, nc), -1, dtype=torch.int64, device=dev)
    pos[k_edge, cell_of_edge] = perm
    pos[k_wall, cell_of_wall] = ne + bperm
    return dict(order=order, nbr=nbr, pos=pos, width=width, part=part)


def split_wide_tiles(lay: dict, tiles: dict, limit: int):
    """The partition (in the module's numbering) of `lay` with every tile
    whose local list (tile and four rings) exceeds `limit` cells cut in two
    by a BFS bisection of its own cells (the halves become new tiles after
    the others); None when no tile exceeds it.  A long, thin tile -- which a
    bisection cut along an irregular BFS level can leave -- has a halo near
    its own size; its halves have about half of it each."""
    meta = tiles["meta"]
    nl = np.asarray(meta[:, 5].cpu() if isinstance(meta, torch.Tensor) else meta[:, 5]).astype(np.int64)
    wide = np.nonzero(nl > limit)[0]
    if wide.size == 0:
        return None
    meta_np = np.asarray(meta.cpu() if isinstance(meta, torch.Tensor) else meta)
    part = lay["part"]
    dev = part.device if isinstance(part, torch.Tensor) else None
    new = part.cpu().numpy().copy() if dev is not None else np.asarray(part).copy()
    nbr = lay["nbr"]
    next_id = int(meta_np.shape[0])
    for t in wide:
        b, n0 = int(meta_np[t, 0]), int(meta_np[t, 1])
        sub = nbr[:, b:b + n0]
        sub = sub.cpu().numpy() if isinstance(sub, torch.Tensor) else np.asarray(sub)
        c = np.broadcast_to(np.arange(n0, dtype=np.int64), sub.shape)
        inside = (sub >= b) & (sub < b + n0)
        half, _ = mesh.bisect_partition(n0, c[inside], sub[inside].astype(np.int64) - b, (n0 + 1) // 2)
        new[b + np.nonzero(half == 1)[0]] = next_id
        next_id += 1
    order = lay["order"]
    order = order.cpu().numpy() if isinstance(order, torch.Tensor) else np.asarray(order)
    out = np.empty_like(new)
    out[order] = new
    return torch.from_numpy(out).to(dev) if dev is not None else out


def _isin_sorted(keys: torch.Tensor, sorted_keys: torch.Tensor) -> torch.Tensor:
    if sorted_keys.numel() == 0:
        return torch.zeros(keys.shape, dtype=torch.bool, device=keys.device)
    p = torch.searchsorted(sorted_keys, keys).clamp_(max=sorted_keys.numel() - 1)
    return sorted_keys[p] == keys


def _tile_layout_device(nbr: torch.Tensor, part: torch.Tensor) -> dict:
    """esr_swe_tile_layout on the GPU, the same arrays (as CUDA tensors).
    Ring L of a tile is the set of (tile, cell) keys reached from ring L-1
    through a face slot, minus the tile's own cells and rings L-1 and L-2
    (a neighbour is at most one ring away), deduplicated and sorted by one
    torch.unique; positions in the local lists come from sorted-key
    searches."""
    dev = nbr.device
    nbr = nbr.to(torch.int32).contiguous()
    nc = nbr.shape[1]
    if nc == 0:
        raise ValueError("empty layout")
    part = part.to(dev, torch.int64).contiguous()
    if int(part.min()) < 0 or bool((part[1:] < part[:-1]).any()):
        raise ValueError("part must be non-decreasing tile ids")
    if bool(((nbr < -2) | (nbr >= nc)).any()):
        raise ValueError("face slot out of range")
    ntiles = int(part[-1]) + 1
    i64 = dict(dtype=torch.int64, device=dev)
    n0 = torch.bincount(part, minlength=ntiles)
    if bool((n0 == 0).any()):
        raise ValueError("tile ids skip a value")
    tbeg = torch.cumsum(n0, 0) - n0
    g64 = nbr.to(torch.int64)
    K = nc  # key of (tile t, cell g): t * nc + g

    def ring(cells, tiles, exclude):
        g = g64[:, cells]
        t = tiles.unsqueeze(0).expand(3, -1)
        gs = g.clamp(min=0)
        keep = (g >= 0) & (part[gs] != t)
        keys = t * K + gs
        for ex in exclude:
            keep &= ~_isin_sorted(keys, ex)
        return torch.unique(keys[keep])

    rings = [ring(torch.arange(nc, **i64), part, [])]
    for _ in range(3):
        r = rings[-1]
        rings.append(ring(r % K, r // K, rings[-1:] + rings[-2:-1]))
    counts = [torch.bincount(r // K, minlength=ntiles) for r in rings]
    cum = [n0]
    for c in counts:
        cum.append(cum[-1] + c)
    meta = torch.zeros((ntiles, 8), dtype=torch.int32, device=dev)
    meta[:, 0] = tbeg.to(torch.int32)
    for q in range(5):
        meta[:, 1 + q] = cum[q].to(torch.int32)
    n3, nL = cum[3], cum[4]
    nh = nL - n0
    off3 = torch.cumsum(n3, 0) - n3
    offh = torch.cumsum(nh, 0) - nh
    tot3, toth = int(n3.sum()), int(nh.sum())
    # halo: each tile's rings 1..4 in order, each ascending; the local index
    # of ring L's i-th entry of tile t is cum[L-1][t] + (i - first entry of t)
    halo = torch.zeros(toth + 1, dtype=torch.int64, device=dev)  # + 1: a safe index for tiles without halo
    keys, local = [], []
    for L, (r, c) in enumerate(zip(rings, counts), start=1):
        t = r // K
        first = torch.cumsum(c, 0) - c
        li = cum[L - 1][t] + (torch.arange(r.numel(), **i64) - first[t])
        halo[offh[t] + (li - n0[t])] = r % K
        keys.append(r)
        local.append(li)
    keys, srt = torch.sort(torch.cat(keys))
    local = torch.cat(local)[srt]
    # the face slots of every tile's cells of level <= 3
    tile = torch.repeat_interleave(torch.arange(ntiles, **i64), n3)
    j = torch.arange(tot3, **i64) - off3[tile]
    n0t = n0[tile]
    cell = torch.where(j < n0t, tbeg[tile] + j, halo[offh[tile] + (j - n0t).clamp(min=0)])
    lnbr = torch.empty(3 * tot3, dtype=torch.int32, device=dev)
    slot_src = torch.empty(3 * tot3, **i64)
    for k in range(3):
        g = g64[k, cell]
        gs = g.clamp(min=0)
        own = part[gs] == tile
        key = tile * K + gs
        p = torch.searchsorted(keys, key).clamp_(max=max(keys.numel() - 1, 0))
        hl = local[p] if keys.numel() else torch.zeros_like(key)
        lp = torch.where(g < 0, g, torch.where(own, gs - tbeg[tile], hl))
        if bool(((g >= 0) & ~own & ((keys[p] != key) if keys.numel() else True)).any()):
            raise RuntimeError("tile layout: a neighbour of a level-3 cell is outside the local list")
        d = 3 * off3[tile] + k * n3[tile] + j
        lnbr[d] = lp.to(torch.int32)
        slot_src[d] = k * nc + cell
    halo = halo[:toth].to(torch.int32)
    max_own, max_l3, max_local = int(n0.max()), int(n3.max()), int(nL.max())
    stats = dict(ntiles=ntiles, max_own=max_own, max_l3=max_l3, max_local=max_local,
                 max_halo3=int((n3 - n0).max()), slot_info=int(_one_boundary_slot(meta, lnbr)),
                 mean_own=float(n0.double().mean()), l3_over_own=float(tot3 / nc),
                 local_over_own=float(int(nL.sum()) / nc), smem=(3 * max_local + 6 * max_l3) * 4)
    return dict(meta=meta, off3=off3, offh=offh, halo=halo, lnbr=lnbr, slot_src=slot_src, area_src=cell,
                stats=stats)


def _local_slots(meta, off3):
    """[3, total] positions 3 * off3[t] + k * n3[t] + j of the records of
    every tile's cells of level <= 3 (torch or numpy, as given)."""
    if isinstance(meta, torch.Tensor):
        dev = meta.device
        n3 = meta[:, 4].to(torch.int64)
        total = int(n3.sum())
        tile = torch.repeat_interleave(torch.arange(n3.shape[0], device=dev), n3)
        j = torch.arange(total, device=dev) - torch.repeat_interleave(torch.cumsum(n3, 0) - n3, n3)
        o3 = off3.to(dev, torch.int64) if off3 is not None else (torch.cumsum(n3, 0) - n3)
        return 3 * o3[tile] + torch.arange(3, device=dev)[:, None] * n3[tile] + j
    n3 = meta[:, 4].astype(np.int64)
    total = int(n3.sum())
    tile = np.repeat(np.arange(n3.shape[0], dtype=np.int64), n3)
    j = np.arange(total, dtype=np.int64) - np.repeat(np.cumsum(n3) - n3, n3)
    o3 = off3.astype(np.int64) if off3 is not None else np.concatenate([[0], np.cumsum(n3)[:-1]])
    return 3 * o3[tile] + np.arange(3, dtype=np.int64)[:, None] * n3[tile] + j


def _slots_by_neighbour(meta: np.ndarray, off3: np.ndarray, lnbr: np.ndarray) -> np.ndarray:
    """Record order of the fast-arithmetic tile layout: each cell's three
    face records sorted by local neighbour index (walls and empty slots
    first).  Neighbouring lanes of a warp then read neighbour states at more
    regular offsets: fewer shared-memory bank conflicts (modelled on the
    N=400 mesh: 4.1 -> 3.2 wavefronts per (h, uh) load of a warp)."""
    if isinstance(lnbr, torch.Tensor):
        order = torch.arange(lnbr.shape[0], dtype=torch.int64, device=lnbr.device)
        if lnbr.shape[0] == 0:
            return order
        idx = _local_slots(meta, off3)
        k = torch.sort(lnbr[idx].to(torch.int64), dim=0, stable=True).indices
        order[idx] = torch.gather(idx, 0, k)
        return order
    order = np.arange(lnbr.shape[0], dtype=np.int64)
    if lnbr.shape[0] == 0:
        return order
    # every level-<=3 cell of every tile: its three records
    idx = _local_slots(meta, off3)
    k = np.argsort(lnbr[idx], axis=0, kind="stable")
    order[idx] = np.take_along_axis(idx, k, axis=0)
    return order


def _one_boundary_slot(meta: np.ndarray, lnbr: np.ndarray) -> bool:
    """True when no tile cell has more than one wall or empty face slot, so
    in the fast layout (records sorted by neighbour, negatives first) slots
    1 and 2 of every cell are interior faces."""
    if lnbr.shape[0] == 0:
        return True
    idx = _local_slots(meta, None)
    return bool(((lnbr[idx] < 0).sum(0) <= 1).all())


def tile_layout(nbr: np.ndarray, part: np.ndarray) -> dict:
    """Tiled face-slot layout (see ``esr_swe_tiles`` in include/esr_gb300.h).

    nbr [3, nc]: face slots in a tile-major cell numbering (neighbour cell,
    -1 wall, -2 empty); part [nc]: non-decreasing tile of every cell.  Per
    tile, the local list is the tile's cells followed by the rings of
    in-neighbours at distance 1..4, each ring sorted by cell; cells of
    levels <= 3 get local face slots.  Returns numpy arrays: meta [ntiles, 8]
    (cell_off, n0, n1, n2, n3, nL), off3, offh, halo, lnbr, slot_src (index
    into the flattened [3, nc] slot arrays), area_src, and stats."""
    if isinstance(nbr, torch.Tensor) and nbr.is_cuda:
        return _tile_layout_device(nbr, part)
    nc = nbr.shape[1]
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    part = np.ascontiguousarray(part, dtype=np.int64)
    ntiles = int(part.max()) + 1
    meta = np.zeros((ntiles, 8), np.int32)
    th, t3 = ctypes.c_int64(), ctypes.c_int64()
    _lib.call("esr_swe_tile_layout", nc, _lib.ptr(nbr), _lib.ptr(part), ntiles, _lib.ptr(meta), ctypes.byref(th),
              ctypes.byref(t3), None, None, None, None, None, None)
    off3 = np.empty(ntiles, np.int64)
    offh = np.empty(ntiles, np.int64)
    halo = np.empty(max(th.value, 1), np.int32)
    lnbr = np.empty(3 * t3.value, np.int32)
    slot_src = np.empty(3 * t3.value, np.int64)
    area_src = np.empty(t3.value, np.int64)
    _lib.call("esr_swe_tile_layout", nc, _lib.ptr(nbr), _lib.ptr(part), ntiles, _lib.ptr(meta), ctypes.byref(th),
              ctypes.byref(t3), _lib.ptr(off3), _lib.ptr(offh), _lib.ptr(halo), _lib.ptr(lnbr), _lib.ptr(slot_src),
              _lib.ptr(area_src))
    cum = meta[:, 1:6].astype(np.int64)
    max_own, max_l3, max_local = int(cum[:, 0].max()), int(cum[:, 3].max()), int(cum[:, 4].max())
    stats = dict(ntiles=ntiles, max_own=max_own, max_l3=max_l3, max_local=max_local,
                 max_halo3=int((cum[:, 3] - cum[:, 0]).max()), slot_info=int(_one_boundary_slot(meta, lnbr)),
                 mean_own=float(cum[:, 0].mean()), l3_over_own=float(t3.value / nc),
                 local_over_own=float(cum[:, 4].sum() / nc), smem=(3 * max_local + 6 * max_l3) * 4)
    return dict(meta=meta, off3=off3, offh=offh, halo=halo[:th.value], lnbr=lnbr, slot_src=slot_src,
                area_src=area_src, stats=stats)

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
    g = torch.Generator(device=dev).manual_seed(1234)  # seeded, drawn where the state lives
    h0 = (1.0 + 0.05 * torch.rand(nc, generator=g, dtype=torch.float64, device=dev)).to(dtype)
    u0 = (0.01 * torch.randn(nc, generator=g, dtype=torch.float64, device=dev)).to(dtype)
    v0 = (0.01 * torch.randn(nc, generator=g, dtype=torch.float64, device=dev)).to(dtype)
    saved = {k: (t[k].data, t[k].elempart) for k in ("h", "uh", "vh", "area")}
    state_saved = eng.state.clone()
    cur_saved = eng.cur
    order = eng.order
    try:
        # per-op path, original order
        area_orig = torch.empty_like(t["area"].data)
        area_orig[order] = t["area"].data
        t["area"].data, t["area"].elempart = area_orig, None
        for k, v in zip(STATE, (h0, u0, v0)):
            t[k].data, t[k].elempart = v.clone(), None
        type(m).forward(m)
        ref = [t[k].data.clone() for k in STATE]
    finally:
        for k, (d, e) in saved.items():
            t[k].data, t[k].elempart = d, e
    # fused path, engine order
    eng.state[:, 0] = h0[order]
    eng.state[:, 1] = u0[order]
    eng.state[:, 2] = v0[order]
    eng._fill_geometry()
    eng.step(1)
    out = eng.state[:, :3].clone()
    eng.cur = cur_saved
    eng.state.copy_(state_saved)
    eng._bind_views()
    torch.cuda.synchronize(dev)
    ok = True
    for j, k in enumerate(STATE):
        fused = torch.empty_like(ref[j])
        fused[order] = out[:, j]
        if eng.precision == "exact":
            good = torch.equal(fused, ref[j])
        else:
            # rounding differences scale with the flux terms (~h^2), so the
            # tolerance is relative to the depth, for every component
            scale = ref[0].abs().max().item() or 1.0
            good = (fused - ref[j]).abs().max().item() <= FAST_STEP_RTOL[dtype] * scale
        if not good:
            diff = (fused - ref[j]).abs().max().item()
            logger.warning(f"fused shallow-water step ({eng.precision}) differs from the module's forward on {k}"
                           f" (max |diff| {diff:.3e}); keeping the per-op path")
            ok = False
    return ok


def try_install(m, modules: List, mode: Optional[str] = None, precision: Optional[str] = None) -> Optional[SweEngine]:
    mode = mode or DEFAULT_MODE
    precision = precision or DEFAULT_PRECISION
    binding = bind(m)
    if binding is None:
        binding = find_roles(m)
        if binding is None:
            return None
        logger.info(f"{type(m).__name__}: shallow-water roles found from its structure")
    reorder = "none" if _shared_with_others(m, modules) else "rcm"  # "none": no renumbering allowed
    if reorder == "none" and mode == "auto":
        mode = "staged"
    try:
        eng = SweEngine(m, binding, reorder=reorder, mode=mode, precision=precision)
    except NotImplementedError as e:
        logger.info(f"{type(m).__name__}: not fused ({e})")
        return None
    ok = _verify(m, eng, binding)
    eng.setup_phases.mark("compile_time_check")
    if not ok:
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
