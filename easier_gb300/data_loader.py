"""Data loaders behind ``esr.Tensor`` / ``Selector`` / ``Reducer`` inputs.

A loader describes data (shape, dtype, device) without materialising it
until ``compile`` loads it onto the runtime device, as in
easier/core/runtime/data_loader.py (DataLoaderBase :61-313,
InMemoryTensorLoader :316-403, FulledTensorLoader :754-830,
ArangeTensorLoader :833-900).  At world size 1 a load is always a full
load, so the partial-load machinery of the reference is not needed.
"""
from __future__ import annotations

import copy
from typing import Optional, Tuple, Union

import numpy as np
import torch

from .utils import EasierJitException

ATTRIBUTE_PLACEHOLDER = "easier_placeholder"


class DataLoaderBase:
    shape: Tuple[int, ...]
    dtype: torch.dtype
    device: torch.device

    def to(self, *, dtype: Optional[torch.dtype] = None,
           device: Optional[Union[torch.device, str]] = None) -> "DataLoaderBase":
        clone = copy.copy(self)
        if dtype is not None:
            clone.dtype = dtype
        if device is not None:
            clone.device = torch.device(device)
        return clone

    def _materialise(self) -> torch.Tensor:
        raise NotImplementedError

    def fully_load(self, device: Union[torch.device, str, None] = None) -> torch.Tensor:
        """The full data, converted to this loader's dtype, on `device`."""
        t = self._materialise()
        dev = torch.device(device) if device is not None else self.device
        return t.to(dtype=self.dtype).to(dev).contiguous()

    def get_placeholder(self, device=None) -> torch.Tensor:
        """A zero-memory tensor carrying shape/dtype/device, like the
        reference's placeholder (data_loader.py:249-300)."""
        if device is None:
            device = self.device
        if len(self.shape) == 0:
            ph = torch.zeros((), dtype=self.dtype, device=device)
        else:
            ph = torch.zeros((1,), dtype=self.dtype, device=device).expand(self.shape)

        def _to_forbidden(self, *args, **kwargs):
            raise EasierJitException("Cannot call .to() on placeholders!")
        ph.to = _to_forbidden.__get__(ph)
        setattr(ph, ATTRIBUTE_PLACEHOLDER, True)
        return ph

    def minmax(self):
        t = self._materialise()
        if t.numel() == 0:
            return None, None
        return t.min().item(), t.max().item()


class InMemoryTensorLoader(DataLoaderBase):
    def __init__(self, tensor: torch.Tensor) -> None:
        self.dtype = tensor.dtype
        self.shape = tuple(tensor.shape)
        self.device = tensor.device
        self.tensor = tensor.detach().cpu()

    def _materialise(self) -> torch.Tensor:
        return self.tensor

    def __repr__(self) -> str:
        return f"{self.__class__.__name__}(shape={self.shape}, dtype={self.dtype})"


class FulledTensorLoader(DataLoaderBase):
    def __init__(self, value, shape, dtype, device) -> None:
        self.value = value
        self.shape = tuple(shape)
        self.dtype = dtype
        self.device = torch.device(device)

    def _materialise(self) -> torch.Tensor:
        return torch.full(self.shape, self.value, dtype=self.dtype)

    def fully_load(self, device=None) -> torch.Tensor:
        dev = torch.device(device) if device is not None else self.device
        return torch.full(self.shape, self.value, dtype=self.dtype, device=dev)

    def __repr__(self) -> str:
        return f"FulledTensorLoader(value={self.value}, shape={self.shape}, dtype={self.dtype})"


class ArangeTensorLoader(DataLoaderBase):
    def __init__(self, start, end, step, dtype, device) -> None:
        if step == 0:
            raise ValueError("step must not be 0")
        self._start, self._end, self._step = start, end, step
        self.shape = (len(range(start, end, step)) if isinstance(start + end + step, int)
                      else int(torch.arange(start, end, step).shape[0]),)
        self.dtype = dtype
        self.device = torch.device(device)

    def _materialise(self) -> torch.Tensor:
        return torch.arange(self._start, self._end, self._step, dtype=self.dtype)

    def __repr__(self) -> str:
        return f"ArangeTensorLoader(start={self._start}, end={self._end}, step={self._step}, dtype={self.dtype})"


class H5DataLoader(DataLoaderBase):
    """HDF5 dataset handle; needs h5py (not part of the GB300 image)."""

    def __init__(self, file: str, dataset: str, *, dtype=None, device="cpu", **h5_file_kwargs) -> None:
        try:
            import h5py  # noqa: F401
        except ImportError as e:
            raise EasierJitException(
                "esr.hdf5() needs h5py, which is not installed; build the data in memory and pass a"
                " torch.Tensor instead") from e
        import h5py
        self._file, self._dataset, self._kw = file, dataset, h5_file_kwargs
        with h5py.File(file, "r", **h5_file_kwargs) as f:
            d = f[dataset]
            self.shape = tuple(d.shape)
            # (h5py gives a NumPy scalar, not an array, for a scalar dataset)
            raw = torch.from_numpy(np.asarray(d[:0] if d.shape else d[()])).dtype
        self.dtype = dtype if dtype is not None else raw
        self.device = torch.device(device)

    def _materialise(self) -> torch.Tensor:
        import h5py
        with h5py.File(self._file, "r", **self._kw) as f:
            d = f[self._dataset]
            return torch.from_numpy(np.array(d[...] if d.shape else d[()]))
