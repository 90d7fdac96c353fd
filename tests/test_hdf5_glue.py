"""esr.hdf5 / Tensor.save go through h5py where it is installed (it is not
part of this image): their calls are checked here against an in-memory
stand-in with h5py's File / dataset interface (File(path, mode), f[name],
.shape, d[...], d[()], d[:0], f.create_dataset(name, data=...)), and
without h5py both raise the framework's error."""
import sys
import types

import numpy as np
import pytest
import torch

import easier_gb300 as esr
from easier_gb300.utils import EasierJitException

_STORE = {}


class _Dataset:
    def __init__(self, arr):
        self._a = np.asarray(arr)
        self.shape = self._a.shape

    def __getitem__(self, key):
        return self._a[key]


class _File:
    def __init__(self, path, mode="r", **kw):
        if mode == "r" and path not in _STORE:
            raise OSError(f"no such file {path}")
        self._d = _STORE.setdefault(path, {})
        self.mode = mode

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def __getitem__(self, name):
        return self._d[name]

    def create_dataset(self, name, data=None):
        if self.mode == "r":
            raise OSError("read-only")
        if name in self._d:
            raise ValueError(f"dataset {name} exists")
        self._d[name] = _Dataset(np.array(data))
        return self._d[name]


@pytest.fixture
def fake_h5py(monkeypatch):
    mod = types.ModuleType("h5py")
    mod.File = _File
    monkeypatch.setitem(sys.modules, "h5py", mod)
    _STORE.clear()
    yield mod
    _STORE.clear()


def test_hdf5_loader_reads_shape_dtype_and_data(fake_h5py):
    arr = np.arange(12, dtype=np.float64).reshape(6, 2)
    with fake_h5py.File("mesh.h5", "a") as f:
        f.create_dataset("geometry/sx", data=arr)
        f.create_dataset("scalar", data=np.float32(2.5))
    ld = esr.hdf5("mesh.h5", "geometry/sx")
    assert ld.shape == (6, 2) and ld.dtype == torch.float64
    assert torch.equal(ld.fully_load("cpu"), torch.from_numpy(arr))
    ld32 = esr.hdf5("mesh.h5", "geometry/sx", dtype=torch.float32)
    assert ld32.fully_load("cpu").dtype == torch.float32
    sc = esr.hdf5("mesh.h5", "scalar")
    assert sc.shape == () and sc.dtype == torch.float32
    assert float(sc.fully_load("cpu")) == 2.5


def test_tensor_save_writes_the_collected_data(fake_h5py, tmp_path):
    from easier_gb300 import jit
    t = esr.Tensor(torch.arange(5, dtype=torch.float64), mode="partition")
    jit._load_tensor(t, "cpu")  # what compile() does to a Tensor
    path = str(tmp_path / "out" / "snap.h5")
    t.save(path, "h")
    got = _STORE[path]["h"][...]
    assert np.array_equal(got, np.arange(5, dtype=np.float64))
    with pytest.raises(ValueError):
        t.save(path, "h")  # h5py refuses to overwrite a dataset; the error reaches the caller


def test_without_h5py_both_raise_the_framework_error(monkeypatch):
    monkeypatch.setitem(sys.modules, "h5py", None)  # import h5py -> ImportError
    with pytest.raises(EasierJitException, match="h5py"):
        esr.hdf5("x.h5", "d")
    t = esr.Tensor(torch.zeros(3, dtype=torch.float64), mode="partition")
    t.easier_data_ready = True
    with pytest.raises(EasierJitException, match="h5py"):
        t.save("x.h5", "d")
