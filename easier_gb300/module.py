"""Public module API: ``Tensor``, ``Module``, ``Selector``, ``Reducer``,
aggregators and data factories.

Same names, arguments, semantics and error messages as
easier/core/module.py; after ``compile(backend='cuda')`` the device work of
``Selector.forward``, ``Reducer.forward`` and the aggregators runs in the
GB300 kernels of ``libesr_gb300.so`` (see ``ops.py``).  There is no CPU
execution path: calling them on CPU tensors raises.
"""
from __future__ import annotations

import builtins
import os
from typing import Dict, List, Literal, Optional, Sequence, Tuple, Union

import torch
from torch import nn

from .data_loader import (ATTRIBUTE_PLACEHOLDER, ArangeTensorLoader, DataLoaderBase, FulledTensorLoader,
                          H5DataLoader, InMemoryTensorLoader)
from .utils import EasierJitException


# ---------------------------------------------------------------- factories
def hdf5(file: str, dataset: str, dtype: Optional[torch.dtype] = None,
         device: Union[torch.device, str, None] = None, **h5_file_kwargs):
    """Handle to an HDF5 dataset (module.py:35-52).  Needs h5py."""
    return H5DataLoader(file, dataset, dtype=dtype, device=device or "cpu", **h5_file_kwargs)


def full(size: Sequence[int], fill_value, *, dtype: Optional[torch.dtype] = None,
         device: Optional[Union[torch.device, str]] = None):
    if isinstance(fill_value, bool) or not isinstance(fill_value, (int, float)):
        raise TypeError("fill_value must be integer or floating-point")
    default_dtype = torch.int64 if isinstance(fill_value, int) else torch.float64
    return FulledTensorLoader(fill_value, size, dtype or default_dtype, device or "cpu")


def zeros(size: Sequence[int], dtype: Optional[torch.dtype] = None,
          device: Optional[Union[torch.device, str]] = None):
    return full(size, 0, dtype=dtype or torch.float64, device=device or "cpu")


def ones(size: Sequence[int], dtype: Optional[torch.dtype] = None,
         device: Optional[Union[torch.device, str]] = None):
    return full(size, 1, dtype=dtype or torch.float64, device=device or "cpu")


def _dtype_device_like(input, dtype=None, device=None):
    return (dtype or input.dtype), torch.device(device if device is not None else input.device)


def full_like(input, fill_value, *, dtype=None, device=None):
    dtype, device = _dtype_device_like(input, dtype, device)
    return full(input.shape, fill_value, dtype=dtype, device=device)


def zeros_like(input, dtype=None, device=None):
    dtype, device = _dtype_device_like(input, dtype, device)
    return zeros(input.shape, dtype=dtype, device=device)


def ones_like(input, dtype=None, device=None):
    dtype, device = _dtype_device_like(input, dtype, device)
    return ones(input.shape, dtype=dtype, device=device)


def arange(*args, **kwargs):
    def _end(end, dtype=None, device=None):
        return 0, end, 1, dtype, device

    def _start_end(start, end, step=1, dtype=None, device=None):
        return start, end, step, dtype, device

    for matcher in (_end, _start_end):
        try:
            start, end, step, dtype, device = matcher(*args, **kwargs)
            break
        except TypeError:
            continue
    else:
        raise TypeError(f"Unexpected arguments {args} to easier.arange")
    for a in (start, end, step):
        if not isinstance(a, (int, float)):
            raise TypeError("argument to easier.arange must be integer or floating-point")
    default = torch.int64 if isinstance(start + end + step, int) else torch.float64
    return ArangeTensorLoader(start, end, step, dtype or default, device or "cpu")


def _resolve_data_loader(arg) -> DataLoaderBase:
    if isinstance(arg, DataLoaderBase):
        return arg
    if isinstance(arg, Tensor) or hasattr(arg, ATTRIBUTE_PLACEHOLDER):
        raise TypeError("Cannot use another easier.Tensor (or its .data property) to initialize easier.Tensor")
    if isinstance(arg, torch.Tensor):
        return InMemoryTensorLoader(arg)
    raise TypeError(f"Unknown data type {type(arg)}")


def _resolve_to_args(cls_name, args, kwargs):
    vals = list(args) + list(kwargs.values())
    if len(vals) != 1:
        raise NotImplementedError(
            f"Currently easier.{cls_name}.to() only supports one argument,"
            " consider using method chaining `.to(dtype).to(device)`")
    arg = vals[0]
    if isinstance(arg, torch.dtype):
        return None, arg
    if isinstance(arg, (str, torch.device)):
        return torch.device(arg), None
    raise TypeError(f"easier.{cls_name}.to() does not accept the argument of type {type(arg)}")


IdxStatus = Literal["placeholder", "partially_loaded", "rewritten"]


# ------------------------------------------------------------ Selector
class Selector(nn.Module):
    """``forward(t) = t[idx]`` along dim 0 (module.py:339-383)."""

    def __init__(self, idx: Union[torch.Tensor, DataLoaderBase]):
        super().__init__()
        self.easier_data_loader = _resolve_data_loader(idx)
        self.easier_index_status: IdxStatus = "placeholder"
        self.idx: torch.Tensor = self.easier_data_loader.get_placeholder()
        self.easier_hint_name: str = ""
        # filled by compile(): int32 device copy and the largest index
        self._idx32: Optional[torch.Tensor] = None
        self._idx_max: int = -1

    def forward(self, tensor: torch.Tensor) -> torch.Tensor:
        if self.easier_index_status != "rewritten":
            raise RuntimeError("Selector.idx not ready, run compile() first")
        from . import ops
        return ops.select(self, tensor)

    def to(self, device: Union[str, torch.device]):
        if self.easier_index_status != "placeholder":
            raise RuntimeError("The properties of easier.Selector can only be modified before easier.compile()")
        self.easier_data_loader = self.easier_data_loader.to(device=device)
        self.idx = self.easier_data_loader.get_placeholder()
        return self


ReduceOp = Literal["sum", "prod", "mean", "amax", "amin"]


# ------------------------------------------------------------- Reducer
class Reducer(nn.Module):
    """``forward(t, out=None)``: ``out.scatter_reduce_(0, idx, t, reduce,
    include_self=False)`` with ``out`` zero-filled when not given
    (module.py:389-477)."""

    def __init__(self, idx: Union[torch.Tensor, DataLoaderBase], n: int, reduce: ReduceOp = "sum") -> None:
        super().__init__()
        self.n = n
        self.reduce = reduce
        self.easier_data_loader = _resolve_data_loader(idx)
        self.easier_index_status: IdxStatus = "placeholder"
        self.idx: torch.Tensor = self.easier_data_loader.get_placeholder()
        self.easier_hint_name: str = ""
        # filled by compile(): CSR of idx (rows = output rows, in-row order =
        # original element order) as int32 device tensors
        self._rowptr32: Optional[torch.Tensor] = None
        self._perm32: Optional[torch.Tensor] = None
        self.easier_is_full: bool = False

    def set_is_full(self):
        assert self.easier_index_status == "rewritten", "Reducer.idx must have been rewritten or loaded"
        counts = self._rowptr32[1:] - self._rowptr32[:-1]
        self.easier_is_full = bool((counts > 0).all().item()) if self.n > 0 else True

    def forward(self, tensor: torch.Tensor, *, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        if self.easier_index_status != "rewritten":
            raise RuntimeError("Reducer.idx not ready, run compile() first")
        shape = tensor.shape
        if out is None:
            out = torch.zeros((self.n,) + tuple(shape[1:]), dtype=tensor.dtype, device=tensor.device)
        if out.shape[0] != self.n:
            raise ValueError(
                f"{out.shape[0]} the length of the first dimension of `out`"
                f" and {self.n} the specified `Reducer.n` do not match")
        from . import ops
        return ops.reduce(self, tensor, out)

    def to(self, device: Union[str, torch.device]):
        if self.easier_index_status != "placeholder":
            raise RuntimeError("The properties of easier.Reducer can only be modified before easier.compile()")
        self.easier_data_loader = self.easier_data_loader.to(device=device)
        self.idx = self.easier_data_loader.get_placeholder()
        return self


# -------------------------------------------------------------- Tensor
class Tensor(nn.Parameter):
    """Partitioned or replicated tensor descriptor (module.py:480-644)."""

    def __new__(cls, data: Union[torch.Tensor, DataLoaderBase], mode: Literal["partition", "replicate"],
                requires_grad: bool = False) -> "Tensor":
        dl = _resolve_data_loader(data)
        tensor = super().__new__(cls, dl.get_placeholder(), requires_grad)
        tensor.easier_data_loader = dl
        return tensor

    def __init__(self, data, mode: Literal["partition", "replicate"], requires_grad: bool = False) -> None:
        self.easier_data_ready: Literal[False, True, "rank0_only"] = False
        self.is_partition = mode == "partition"
        self.is_replica = mode == "replicate"
        self.easier_hint_name: str = ""
        # original index of every local row (None = identity order)
        self.elempart: Optional[torch.Tensor] = None

    def __repr__(self) -> str:
        if self.is_replica:
            body = " " + repr(self.easier_data_loader) if not self.easier_data_ready else "\n" + repr(self.data)
            return "Replicated easier.Tensor" + body
        body = " " + repr(self.easier_data_loader) if not self.easier_data_ready else ""
        return "Managed partitioned easier.Tensor" + body

    def __setitem__(self, indices, val):
        if not self.easier_data_ready:
            raise RuntimeError("Tensor data is not ready, run compile() first")
        self.data.__setitem__(indices, val)
        return self

    def to(self, *args, **kwargs):
        if self.easier_data_ready is not False:
            raise RuntimeError("The properties of easier.Tensor can only be modified before easier.compile()")
        device, dtype = _resolve_to_args("Tensor", args, kwargs)
        self.easier_data_loader = self.easier_data_loader.to(device=device, dtype=dtype)
        self.data = self.easier_data_loader.get_placeholder()
        return self

    def collect(self) -> torch.Tensor:
        """The full tensor in the original element order, on the device the
        user program specified (module.py:588-612)."""
        if not self.easier_data_ready:
            raise RuntimeError("Tensor data is not ready, run compile() first")
        if self.elempart is None:
            out = self.data.clone()
        else:
            out = torch.empty_like(self.data)
            out[self.elempart] = self.data
        return out.to(self.easier_data_loader.device)

    def save(self, h5_file_path, h5_dataset_path, **h5_file_kwargs) -> None:
        if not self.easier_data_ready:
            raise RuntimeError("Tensor data is not ready, run compile() first")
        try:
            import h5py
        except ImportError as e:
            raise EasierJitException("easier.Tensor.save() needs h5py, which is not installed") from e
        path = os.path.expanduser(h5_file_path)
        d = os.path.dirname(path)
        if d:
            os.makedirs(d, exist_ok=True)
        with h5py.File(path, mode="a", **h5_file_kwargs) as f:
            f.create_dataset(h5_dataset_path, data=self.collect().cpu().numpy())


# -------------------------------------------------------------- Module
def get_easier_objects(top_modules) -> Dict[object, List[str]]:
    """Every Module/Selector/Reducer/Tensor/DataLoader reachable from the
    top modules, with the attribute paths that reach it (first one used as
    its hint name)."""
    objs: Dict[int, Tuple[object, List[str]]] = {}

    def add(obj, name):
        if id(obj) in objs:
            objs[id(obj)][1].append(name)
            return False
        objs[id(obj)] = (obj, [name])
        return True

    def visit(mod: nn.Module, prefix: str):
        if not add(mod, prefix):
            return
        for pname, p in mod.named_parameters(recurse=False):
            if isinstance(p, Tensor):
                if add(p, f"{prefix}.{pname}"):
                    add(p.easier_data_loader, f"{prefix}.{pname}:loader")
        if isinstance(mod, (Selector, Reducer)):
            add(mod.easier_data_loader, f"{prefix}.idx:loader")
        for k, v in list(vars(mod).items()):
            if isinstance(v, DataLoaderBase):
                add(v, f"{prefix}.{k}")
        for cname, child in mod.named_children():
            visit(child, f"{prefix}.{cname}")

    for i, m in enumerate(top_modules):
        visit(m, f"({type(m).__name__}#{i})")
    return {o: names for o, names in objs.values()}


class Module(nn.Module):
    """User modules; ``forward()`` mutates ``esr.Tensor``s (module.py:710-822)."""

    def __init__(self):
        super().__init__()
        self.easier_raw_graph = None
        self.easier_hint_name: str = ""
        self.easier_jit_backend: Literal["torch", "cpu", "cuda", "none", None] = None
        self.partition_mode: Literal["metis", "evenly"] = "metis"

    def forward(self):
        pass

    def to(self, *args, **kwargs):
        if self.easier_jit_backend is not None:
            raise RuntimeError("The properties of easier.Module can only be modified before easier.compile()")
        device, fp_dtype = _resolve_to_args("Module", args, kwargs)
        if fp_dtype is not None and not fp_dtype.is_floating_point:
            raise ValueError(f"easier.Module.to() does not accept the dtype {fp_dtype}, floating point dtypes are required")
        for obj in get_easier_objects([self]):
            if isinstance(obj, (Selector, Reducer)) and device is not None:
                obj.to(device)
            if isinstance(obj, Tensor):
                if device is not None:
                    obj.to(device)
                if fp_dtype is not None and obj.easier_data_loader.dtype.is_floating_point:
                    obj.to(fp_dtype)
            if isinstance(obj, Module):
                for k, v in list(obj.__dict__.items()):
                    if isinstance(v, DataLoaderBase):
                        dt = fp_dtype if v.dtype.is_floating_point else None
                        setattr(obj, k, v.to(dtype=dt, device=device))
        return self


# ---------------------------------------------------------- aggregators
def sum(tensor: torch.Tensor) -> torch.Tensor:
    """``torch.sum(t, dim=0, keepdim=True)`` (module.py:829-837)."""
    from . import ops
    return ops.aggregate(tensor, "sum")


def prod(tensor: torch.Tensor) -> torch.Tensor:
    from . import ops
    return ops.aggregate(tensor, "prod")


def norm(tensor: torch.Tensor, p: Union[int, str] = 2) -> torch.Tensor:
    """``torch.norm(t, p, dim=0, keepdim=True)``; p = 2 only."""
    if p not in (2, "fro"):
        raise NotImplementedError("easier_gb300 implements the 2-norm aggregator only")
    from . import ops
    return ops.aggregate(tensor, "norm")


def max(tensor: torch.Tensor) -> torch.Tensor:
    from . import ops
    return ops.aggregate(tensor, "max")


def min(tensor: torch.Tensor) -> torch.Tensor:
    from . import ops
    return ops.aggregate(tensor, "min")


easier_aggregators = (sum, prod, norm, max, min)
