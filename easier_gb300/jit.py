"""``init`` and ``compile``: the install point of the GB300 path.

Mirrors easier/core/jit.py (init :242-291, compile :294-419).  At world
size 1 the reference's partition / halo / allgather passes reduce to the
identity, so ``compile`` here

1. loads every ``esr.Tensor`` onto the CUDA device,
2. validates every Selector / Reducer index (the range checks of
   passes/collective_initialization.py:76-106) and builds their device
   form: an int32 index for a Selector; for a Reducer the stable CSR that the
   reference's reorder pass gives it (sparse_encoding.py:244-338),
3. installs a fused engine on modules it recognises (the shallow-water step,
   see ``swe.py``; the solvers build theirs at ``solve()``), which is where
   the reference's own JitEngine is installed (jit.py:413-415).

Every other module keeps its Python ``forward``: its Selector / Reducer /
aggregator calls run in the GB300 kernels, elementwise glue in torch.
"""
from __future__ import annotations

import os
from typing import List, Literal, Optional

import numpy as np
import torch

from . import module as _m
from .utils import EasierJitException, init_logger, logger

_initialized_backend: Optional[str] = None


def init(comm_backend: str, **kwargs) -> None:
    """Initialise torch.distributed (jit.py:242-291).  Accepts 'gloo',
    'nccl', 'mpi' or 'cpu:gloo,cuda:nccl'.  The GB300 path runs one process
    per GPU; with CUDA available the process's device is LOCAL_RANK."""
    global _initialized_backend
    if not isinstance(comm_backend, str):
        raise EasierJitException("`comm_backend` must be str")
    import torch.distributed as dist
    if "WORLD_SIZE" not in os.environ:
        os.environ.setdefault("WORLD_SIZE", "1")
        os.environ.setdefault("RANK", "0")
        os.environ.setdefault("LOCAL_RANK", "0")
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29511")
    if torch.cuda.is_available():
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if not dist.is_initialized():
        dist.init_process_group(comm_backend, **kwargs)
    init_logger(dist.get_rank())
    _initialized_backend = comm_backend
    logger.info(f"torch.distributed backend={comm_backend} rank={dist.get_rank()}")


def _world_size() -> int:
    import torch.distributed as dist
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def _device_type_of(objs) -> str:
    types = {o.device.type for o in objs if isinstance(o, _m.DataLoaderBase)}
    if len(types) > 1:
        raise EasierJitException(f"Must involve only one torch device type (cpu/cuda), got {sorted(types)}")
    return types.pop() if types else "cpu"


def _load_selector(sel: _m.Selector, device) -> None:
    idx = sel.easier_data_loader.fully_load("cpu")
    if idx.dtype not in (torch.int64, torch.int32, torch.int16, torch.int8, torch.uint8):
        raise EasierJitException(f"{sel.easier_hint_name}: Selector idx must be an integer tensor")
    idx = idx.to(torch.int64).reshape(-1)
    if idx.numel():
        lo, hi = int(idx.min()), int(idx.max())
        if lo < 0:
            raise EasierJitException(f"{sel.easier_hint_name}: Selector idx has negative values")
        if hi >= 2 ** 31 - 1:
            raise EasierJitException(f"{sel.easier_hint_name}: Selector idx exceeds int32")
        sel._idx_max = hi
    else:
        sel._idx_max = -1
    sel.idx = idx.to(device)
    sel._idx32 = idx.to(torch.int32).to(device)
    sel.easier_index_status = "rewritten"


def _load_reducer(red: _m.Reducer, device) -> None:
    from . import mesh
    idx = red.easier_data_loader.fully_load(device if torch.device(device).type == "cuda" else "cpu")
    if idx.dtype not in (torch.int64, torch.int32, torch.int16, torch.int8, torch.uint8):
        raise EasierJitException(f"{red.easier_hint_name}: Reducer idx must be an integer tensor")
    if red.reduce not in ("sum", "prod", "mean", "amax", "amin"):
        raise EasierJitException(f"{red.easier_hint_name}: unknown reduce op {red.reduce!r}")
    if not isinstance(red.n, int) or red.n < 0:
        raise EasierJitException(f"{red.easier_hint_name}: Reducer.n must be a non-negative int")
    idx = idx.to(torch.int64).reshape(-1)
    if idx.shape[0] >= 2 ** 31 - 1 or red.n >= 2 ** 31 - 1:
        raise EasierJitException(f"{red.easier_hint_name}: Reducer larger than int32 indexing")
    if torch.device(device).type == "cuda":
        # the stable CSR on the GPU: one stable sort, the same arrays as
        # esr_csr_from_index
        idx = idx.to(device)
        if idx.numel() and (int(idx.min()) < 0 or int(idx.max()) >= red.n):
            raise EasierJitException(f"{red.easier_hint_name}: Reducer index out of range [0, {red.n})")
        red.idx = idx
        red._rowptr32, red._perm32 = mesh._stable_csr_device(idx, red.n)
    else:
        idx_np = idx.numpy()
        try:
            rowptr, perm = mesh.csr_from_index(idx_np, red.n)
        except ValueError as e:
            raise EasierJitException(f"{red.easier_hint_name}: {e}") from e
        red.idx = torch.from_numpy(idx_np).to(device)
        red._rowptr32 = torch.from_numpy(rowptr.astype(np.int32)).to(device)
        red._perm32 = torch.from_numpy(perm.astype(np.int32)).to(device)
    red.easier_index_status = "rewritten"
    red.set_is_full()


def _load_tensor(t: _m.Tensor, device) -> None:
    if t.easier_data_ready:
        return
    t.data = t.easier_data_loader.fully_load(device)
    t.elempart = None
    t.easier_data_ready = True


def compile(modules: List[_m.Module], backend: Literal["torch", "cpu", "cuda", "none"], *,
            load_dir: Optional[str] = None, partition_mode: Literal["metis", "evenly"] = "metis",
            fuse: bool = True, precision: Optional[str] = None) -> List[_m.Module]:
    """Compile modules for the GB300 path (see module docstring).

    ``backend`` must be 'cuda' (or 'torch' with CUDA-placed modules).
    ``load_dir`` (the reference's compile cache) is accepted and ignored: the
    world-size-1 layout is recomputed in milliseconds.  ``fuse=False`` keeps
    every module on the per-op path (used to cross-check the fused engines).
    ``precision`` ('exact' default, or 'fast') picks the fused shallow-water
    arithmetic: 'exact' is bitwise the reference; 'fast' contracts to FMA and
    replaces the divisions by one reciprocal per face (FP32 within 1e-5 of
    the reference after 1,000 steps).
    """
    if not isinstance(modules, (list, tuple)) or not all(isinstance(m, _m.Module) for m in modules):
        raise EasierJitException("compile() expects a list of easier.Module")
    if backend not in ("torch", "cpu", "cuda", "none"):
        raise EasierJitException(f"Argument `jit_backend` cannot be {backend}")
    if partition_mode not in ("metis", "evenly"):
        raise EasierJitException(f"Argument `partition_mode` cannot be {partition_mode}")
    objs = _m.get_easier_objects(list(modules))
    orig_type = _device_type_of(objs)
    if backend in ("cpu", "none") or (backend == "torch" and orig_type != "cuda"):
        raise EasierJitException(
            "easier_gb300 implements the CUDA backend only (backend='cuda'); the CPU backends are the"
            " reference package's")
    if _world_size() > 1:
        raise EasierJitException(
            "easier_gb300 runs at world size 1 (one GPU per process, independent replicas)")
    if not torch.cuda.is_available():
        raise EasierJitException("backend='cuda' needs a CUDA device")
    device = torch.device("cuda", torch.cuda.current_device())
    from . import _lib
    _lib.lib()  # fail now, loudly, if the native library is unusable

    for obj, names in objs.items():
        if hasattr(obj, "easier_hint_name"):
            try:
                obj.easier_hint_name = names[0]
            except AttributeError:
                pass
    for obj in objs:
        if isinstance(obj, _m.Selector) and obj.easier_index_status == "placeholder":
            _load_selector(obj, device)
        elif isinstance(obj, _m.Reducer) and obj.easier_index_status == "placeholder":
            _load_reducer(obj, device)
        elif isinstance(obj, _m.Tensor):
            _load_tensor(obj, device)
    for m in objs:
        if isinstance(m, _m.Module):
            m.easier_jit_backend = backend
            m.partition_mode = partition_mode

    if fuse:
        from . import swe
        for m in modules:
            eng = swe.try_install(m, modules, precision=precision)
            if eng is not None:
                logger.info(f"{type(m).__name__}: fused shallow-water engine installed ({eng.describe()})")
    logger.info("EASIER just-in-time compilation has completed")
    return list(modules)
