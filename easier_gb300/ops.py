"""Device ops behind Selector / Reducer / aggregators.

Each op checks its inputs on the host (device, dtype, shape, index range
known since compile) and launches the matching C-ABI kernel on torch's
current stream.  Non-CUDA tensors raise: there is no CPU path.
"""
from __future__ import annotations

import torch

from . import _lib
from .utils import EasierJitException


def _require_cuda(t: torch.Tensor, what: str) -> None:
    if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
        raise EasierJitException(f"{what}: easier_gb300 runs on CUDA tensors only (got {getattr(t, 'device', type(t))})")


def select(sel, tensor: torch.Tensor) -> torch.Tensor:
    """Selector.forward: tensor[idx] (easier/core/module.py:364-371)."""
    _require_cuda(tensor, "Selector")
    idx = sel._idx32
    if idx.device != tensor.device:
        raise EasierJitException("Selector input is on a different device than its index")
    if sel._idx_max >= tensor.shape[0]:
        raise IndexError(f"index {sel._idx_max} is out of bounds for dimension 0 with size {tensor.shape[0]}")
    src = tensor.contiguous()
    m = idx.shape[0]
    out = torch.empty((m,) + tuple(src.shape[1:]), dtype=src.dtype, device=src.device)
    row_bytes = src.element_size() * int(torch.Size(src.shape[1:]).numel())
    _lib.call("esr_gather", _lib.ptr(src), src.shape[0], row_bytes, _lib.ptr(idx), m, _lib.ptr(out),
              _lib.stream_handle(src.device))
    return out


def reduce(red, tensor: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
    """Reducer.forward: out.scatter_reduce_(0, idx, t, op, include_self=False)
    (easier/core/module.py:441-461), as a deterministic in-order segment
    reduction over the CSR of idx."""
    _require_cuda(tensor, "Reducer")
    _require_cuda(out, "Reducer out")
    if tensor.dtype != out.dtype:
        raise RuntimeError(f"scatter_reduce(): Expected self.dtype to be equal to src.dtype ({out.dtype} vs {tensor.dtype})")
    m = red._perm32.shape[0]
    if tensor.shape[0] < m or tuple(tensor.shape[1:]) != tuple(out.shape[1:]):
        raise RuntimeError(
            f"Reducer: input of shape {tuple(tensor.shape)} does not match idx length {m} and"
            f" out shape {tuple(out.shape)}")
    src = tensor.contiguous()
    dst = out if out.is_contiguous() else out.contiguous()
    cols = int(torch.Size(src.shape[1:]).numel())
    _lib.call("esr_segreduce", _lib.dtype_code(src.dtype), _lib.REDUCE_OPS[red.reduce], _lib.ptr(src), cols,
              _lib.ptr(red._rowptr32), _lib.ptr(red._perm32), red.n, _lib.ptr(dst), _lib.stream_handle(src.device))
    if dst is not out:
        out.copy_(dst)
    return out


_AGG = {"sum": _lib.AGG_SUM, "prod": _lib.AGG_PROD, "norm": _lib.AGG_NORM, "max": _lib.AGG_MAX, "min": _lib.AGG_MIN}


def aggregate(tensor: torch.Tensor, kind: str) -> torch.Tensor:
    """esr.sum/prod/norm/max/min: op over dim 0 with keepdim
    (easier/core/module.py:825-884); FP64 accumulation, fixed order."""
    _require_cuda(tensor, f"esr.{kind}")
    if kind == "norm" and not tensor.dtype.is_floating_point:
        raise RuntimeError("norm(): input dtype should be floating point")
    if kind in ("max", "min") and tensor.shape[0] == 0:
        raise IndexError(f"{kind}(): Expected reduction dim 0 to have non-zero size.")
    src = tensor.contiguous()
    n = src.shape[0]
    cols = int(torch.Size(src.shape[1:]).numel())
    out = torch.empty((1,) + tuple(src.shape[1:]), dtype=src.dtype, device=src.device)
    nbytes = _lib.lib().esr_aggregate_workspace_bytes(n, cols)
    ws = torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=src.device)
    _lib.call("esr_aggregate", _lib.dtype_code(src.dtype), _AGG[kind], _lib.ptr(src), n, cols, _lib.ptr(out),
              _lib.ptr(ws), _lib.stream_handle(src.device))
    return out


def dot(a: torch.Tensor, b: torch.Tensor, out: torch.Tensor = None, workspace: torch.Tensor = None) -> torch.Tensor:
    """FP64-accumulated dot product of two equal-length vectors; returns a
    1-element FP64 device tensor."""
    _require_cuda(a, "dot")
    if a.shape != b.shape or a.dtype != b.dtype:
        raise ValueError("dot: operands must have equal shape and dtype")
    n = a.numel()
    if out is None:
        out = torch.empty(1, dtype=torch.float64, device=a.device)
    if workspace is None:
        workspace = torch.zeros(int(_lib.lib().esr_dot_workspace_bytes(n)), dtype=torch.uint8, device=a.device)
    _lib.call("esr_dot", _lib.dtype_code(a.dtype), _lib.ptr(a.contiguous()), _lib.ptr(b.contiguous()), n,
              _lib.ptr(out), _lib.ptr(workspace), _lib.stream_handle(a.device))
    return out


def device_status(clear: bool = True, device=None) -> int:
    """OR of the device-side error bits raised since the last clear."""
    import ctypes
    v = ctypes.c_int(0)
    _lib.call("esr_device_status", ctypes.byref(v), 1 if clear else 0, _lib.stream_handle(device))
    return v.value
