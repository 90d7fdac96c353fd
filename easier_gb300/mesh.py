"""Host-side mesh generation, geometry, assembly and ordering.

numpy in, numpy out; the work runs in the native library's host code
(``csrc/host_mesh.cpp``, ``csrc/host_order.cpp``).  The index arrays are
bit-identical to the reference's generator (csrc/triangular_mesh.cpp) and
the geometry is computed in the reference's operation order, so its values
are bitwise those of the reference's CPU run.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import _lib


def _i64(x):
    return np.ascontiguousarray(x, dtype=np.int64)


def _f64(x):
    return np.ascontiguousarray(x, dtype=np.float64)


@dataclass
class TriangularMesh:
    """Unit-square mesh with 4 triangles per square (csrc/triangular_mesh.cpp)."""
    n: int
    src: np.ndarray      # [ne] int64
    dst: np.ndarray      # [ne] int64
    cells: np.ndarray    # [nc, 3] int64
    bcells: np.ndarray   # [nbc] int64
    bpoints: np.ndarray  # [nbc, 2] int64
    points: np.ndarray   # [np, 2] float64

    @property
    def nc(self):
        return self.cells.shape[0]

    @property
    def ne(self):
        return self.src.shape[0]

    @property
    def nbc(self):
        return self.bcells.shape[0]


def mesh_sizes(n: int):
    out = [ctypes.c_int64() for _ in range(4)]
    _lib.call("esr_mesh_sizes", n, *[ctypes.byref(o) for o in out])
    return tuple(o.value for o in out)


def _on_cuda(mesh) -> bool:
    return isinstance(mesh.src, torch.Tensor) and mesh.src.is_cuda


def triangular_mesh(n: int, device=None) -> TriangularMesh:
    """Same arrays as the reference's ``generate_triangular_mesh(n)``.  With
    a CUDA ``device`` the mesh is generated there (esr_mesh_triangular_device,
    bitwise the host generator's) and the fields are device tensors."""
    nc, ne, nbc, npts = mesh_sizes(n)
    if device is not None and torch.device(device).type == "cuda":
        dev = torch.device(device)
        i64 = dict(dtype=torch.int64, device=dev)
        m = TriangularMesh(n, torch.empty(ne, **i64), torch.empty(ne, **i64), torch.empty((nc, 3), **i64),
                           torch.empty(nbc, **i64), torch.empty((nbc, 2), **i64),
                           torch.empty((npts, 2), dtype=torch.float64, device=dev))
        _lib.call("esr_mesh_triangular_device", n, _lib.ptr(m.src), _lib.ptr(m.dst), _lib.ptr(m.cells),
                  _lib.ptr(m.bcells), _lib.ptr(m.bpoints), _lib.ptr(m.points), _lib.stream_handle(dev))
        return m
    src = np.empty(ne, np.int64)
    dst = np.empty(ne, np.int64)
    cells = np.empty((nc, 3), np.int64)
    bcells = np.empty(nbc, np.int64)
    bpoints = np.empty((nbc, 2), np.int64)
    points = np.empty((npts, 2), np.float64)
    _lib.call("esr_mesh_triangular", n, _lib.ptr(src), _lib.ptr(dst), _lib.ptr(cells), _lib.ptr(bcells),
              _lib.ptr(bpoints), _lib.ptr(points))
    return TriangularMesh(n, src, dst, cells, bcells, bpoints, points)


@dataclass
class SweGeometry:
    """Inputs of the shallow-water module (assemble_shallow_water.py:185-253)."""
    sx: np.ndarray
    sy: np.ndarray
    alpha: np.ndarray
    area: np.ndarray
    x: np.ndarray
    y: np.ndarray
    bsx: np.ndarray
    bsy: np.ndarray


def swe_geometry(mesh: TriangularMesh) -> SweGeometry:
    """assemble_shallow_water.py:154-253; a mesh of CUDA tensors is
    assembled on its device (esr_swe_geometry_device, bitwise the host's)."""
    nc, ne, nbc = mesh.nc, mesh.ne, mesh.nbc
    if _on_cuda(mesh):
        dev = mesh.src.device
        g = SweGeometry(*(torch.empty(k, dtype=torch.float64, device=dev) for k in (ne, ne, ne, nc, nc, nc, nbc, nbc)))
        _lib.call("esr_swe_geometry_device", nc, ne, nbc, mesh.points.shape[0], _lib.ptr(mesh.src),
                  _lib.ptr(mesh.dst), _lib.ptr(mesh.cells), _lib.ptr(mesh.bcells), _lib.ptr(mesh.bpoints),
                  _lib.ptr(mesh.points), _lib.ptr(g.sx), _lib.ptr(g.sy), _lib.ptr(g.alpha), _lib.ptr(g.area),
                  _lib.ptr(g.x), _lib.ptr(g.y), _lib.ptr(g.bsx), _lib.ptr(g.bsy), _lib.stream_handle(dev))
        return g
    g = SweGeometry(*(np.empty(k, np.float64) for k in (ne, ne, ne, nc, nc, nc, nbc, nbc)))
    _lib.call("esr_swe_geometry", nc, ne, nbc, _lib.ptr(_i64(mesh.src)), _lib.ptr(_i64(mesh.dst)),
              _lib.ptr(_i64(mesh.cells)), _lib.ptr(_i64(mesh.bcells)), _lib.ptr(_i64(mesh.bpoints)),
              _lib.ptr(_f64(mesh.points)), _lib.ptr(g.sx), _lib.ptr(g.sy), _lib.ptr(g.alpha), _lib.ptr(g.area),
              _lib.ptr(g.x), _lib.ptr(g.y), _lib.ptr(g.bsx), _lib.ptr(g.bsy))
    return g


def gaussian_bump(x: np.ndarray, y: np.ndarray, x0: float = 0.5, y0: float = 0.5, width2: float = 0.01,
                  amp: float = 0.1) -> np.ndarray:
    """Initial depth h = 1 + amp*exp(-((x-x0)^2 + (y-y0)^2)/width2).  With
    x0 = y0 = 0, width2 = 0.01 this is the tutorial's corner bump
    (assemble_shallow_water.py:242-244); the benchmark centres it."""
    return 1 + amp * np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / width2)


@dataclass
class PoissonFV:
    """Cell-centred FV Poisson (assemble_poisson.py:160-230)."""
    Af: np.ndarray
    Ac: np.ndarray
    b: np.ndarray
    rho: np.ndarray
    centroid: np.ndarray


def _stable_csr_device(idx: torch.Tensor, n: int):
    """rowptr [n+1], perm [m] (int32) of a device index: the stable sort
    the reference's Reducer order follows."""
    perm = torch.sort(idx, stable=True).indices.to(torch.int32)
    rowptr = torch.zeros(n + 1, dtype=torch.int64, device=idx.device)
    rowptr[1:] = torch.cumsum(torch.bincount(idx, minlength=n), 0)
    return rowptr.to(torch.int32), perm


def poisson_fv(mesh: TriangularMesh) -> PoissonFV:
    """assemble_poisson.py:160-230; a mesh of CUDA tensors is assembled on
    its device (esr_poisson_fv_assemble_device: Af, Ac, centroid bitwise the
    host's; rho and b through CUDA's exp, within a few ulp)."""
    nc, ne, nbc = mesh.nc, mesh.ne, mesh.nbc
    if _on_cuda(mesh):
        dev = mesh.src.device
        f = dict(dtype=torch.float64, device=dev)
        out = PoissonFV(torch.empty(ne, **f), torch.empty(nc, **f), torch.empty(nc, **f), torch.empty(nc, **f),
                        torch.empty((nc, 2), **f))
        rowptr, perm = _stable_csr_device(mesh.src, nc)
        brow, bperm = _stable_csr_device(mesh.bcells, nc)
        _lib.call("esr_poisson_fv_assemble_device", nc, ne, nbc, mesh.points.shape[0], _lib.ptr(mesh.src),
                  _lib.ptr(mesh.dst), _lib.ptr(mesh.cells), _lib.ptr(mesh.bcells), _lib.ptr(mesh.bpoints),
                  _lib.ptr(mesh.points), _lib.ptr(rowptr), _lib.ptr(perm), _lib.ptr(brow), _lib.ptr(bperm),
                  _lib.ptr(out.Af), _lib.ptr(out.Ac), _lib.ptr(out.b), _lib.ptr(out.rho), _lib.ptr(out.centroid),
                  _lib.stream_handle(dev))
        return out
    out = PoissonFV(np.empty(ne), np.empty(nc), np.empty(nc), np.empty(nc), np.empty((nc, 2)))
    _lib.call("esr_poisson_fv_assemble", nc, ne, nbc, _lib.ptr(_i64(mesh.src)), _lib.ptr(_i64(mesh.dst)),
              _lib.ptr(_i64(mesh.cells)), _lib.ptr(_i64(mesh.bcells)), _lib.ptr(_i64(mesh.bpoints)),
              _lib.ptr(_f64(mesh.points)), _lib.ptr(out.Af), _lib.ptr(out.Ac), _lib.ptr(out.b),
              _lib.ptr(out.rho), _lib.ptr(out.centroid))
    return out


@dataclass
class P1System:
    """P1 stiffness on an n x n grid in Linsys form: y = reducer(x[col]*Ae) + x*Av."""
    n: int
    row: np.ndarray   # Reducer idx [nnz]
    col: np.ndarray   # Selector idx [nnz]
    Ae: np.ndarray    # [nnz]
    Av: np.ndarray    # [nunk]

    @property
    def nunk(self):
        return self.Av.shape[0]


def p1_system(n: int, kappa: Optional[np.ndarray] = None) -> P1System:
    nunk, nnz = ctypes.c_int64(), ctypes.c_int64()
    _lib.call("esr_p1_sizes", n, ctypes.byref(nunk), ctypes.byref(nnz))
    row = np.empty(nnz.value, np.int64)
    col = np.empty(nnz.value, np.int64)
    Ae = np.empty(nnz.value, np.float64)
    Av = np.empty(nunk.value, np.float64)
    k = None if kappa is None else _f64(kappa)
    if k is not None and k.shape != (2 * n * n,):
        raise ValueError(f"kappa must have 2*n*n = {2 * n * n} entries")
    _lib.call("esr_p1_assemble", n, _lib.ptr(k), _lib.ptr(row), _lib.ptr(col), _lib.ptr(Ae), _lib.ptr(Av))
    return P1System(n, row, col, Ae, Av)


def p1_nodes(n: int):
    """Coordinates (x, y) of the (n-1)^2 interior nodes in unknown order."""
    m = n - 1
    j, i = np.meshgrid(np.arange(1, n), np.arange(1, n), indexing="ij")
    return (i.reshape(-1) / n, j.reshape(-1) / n) if m > 0 else (np.empty(0), np.empty(0))


def random_mode_rhs(n: int, seed: int, modes: int = 16, kmax: int = 8) -> np.ndarray:
    """Lumped P1 load vector b_i = h^2 f(x_i) of
    f = sum_m c_m sin(k_m pi x) sin(l_m pi y), c ~ N(0,1), k, l ~ U{1..kmax}."""
    rng = np.random.default_rng(seed)
    c = rng.standard_normal(modes)
    k = rng.integers(1, kmax + 1, modes)
    l = rng.integers(1, kmax + 1, modes)
    x, y = p1_nodes(n)
    f = np.zeros_like(x)
    for m in range(modes):
        f += c[m] * np.sin(k[m] * np.pi * x) * np.sin(l[m] * np.pi * y)
    return f / (n * n)


def gaussian_random_field(n: int, seed: int, corr_len: float = 0.1, variance: float = 1.0) -> np.ndarray:
    """Stationary Gaussian field on the (n+1) x (n+1) grid nodes of the unit
    square with covariance variance*exp(-r^2 / (2 corr_len^2)), sampled by
    spectral (FFT) synthesis on a periodic box twice the domain size and
    rescaled to the exact target variance of the samples."""
    rng = np.random.default_rng(seed)
    m = 2 * (n + 1)
    h = 1.0 / n
    kx = np.fft.fftfreq(m, d=h) * 2 * np.pi
    K2 = kx[:, None] ** 2 + kx[None, :] ** 2
    spec = np.exp(-0.5 * K2 * corr_len ** 2)  # Gaussian covariance spectrum (up to scale)
    noise = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    field = np.fft.ifft2(np.sqrt(spec) * noise).real[: n + 1, : n + 1]
    field = field - field.mean()
    sd = field.std()
    return field * (np.sqrt(variance) / sd) if sd > 0 else field


def kappa_from_field(g: np.ndarray) -> np.ndarray:
    """Per-triangle coefficient kappa = exp(mean of g over the triangle's
    vertices), lower then upper triangle of each square (i, j)."""
    n = g.shape[0] - 1
    G = g.T  # G[i, j] = g at node (i, j): g was indexed [j, i]
    lo = (G[:-1, :-1] + G[1:, :-1] + G[1:, 1:]) / 3.0    # (i,j),(i+1,j),(i+1,j+1)
    up = (G[:-1, :-1] + G[1:, 1:] + G[:-1, 1:]) / 3.0    # (i,j),(i+1,j+1),(i,j+1)
    out = np.empty((n, n, 2))
    out[:, :, 0] = np.exp(lo.T)   # index [j, i]
    out[:, :, 1] = np.exp(up.T)
    return out.reshape(-1)


def csr_from_index(idx: np.ndarray, n: int):
    """Stable CSR (rowptr [n+1], perm [m]) of a Reducer index."""
    idx = _i64(idx)
    rowptr = np.empty(n + 1, np.int64)
    perm = np.empty(idx.shape[0], np.int64)
    _lib.call("esr_csr_from_index", _lib.ptr(idx), idx.shape[0], n, _lib.ptr(rowptr), _lib.ptr(perm))
    return rowptr, perm


def rcm_order(n: int, src: np.ndarray, dst: np.ndarray) -> np.ndarray:
    """Reverse Cuthill-McKee order (order[new] = old)."""
    src, dst = _i64(src), _i64(dst)
    order = np.empty(n, np.int64)
    _lib.call("esr_rcm_order", n, src.shape[0], _lib.ptr(src), _lib.ptr(dst), _lib.ptr(order))
    return order


def sell_layout(n: int, rowptr: np.ndarray, perm: np.ndarray, colidx: np.ndarray, ncols: int):
    """SELL-32 layout: slice_ptr, col (int32, -1 padding), src_pos."""
    rowptr, perm, colidx = _i64(rowptr), _i64(perm), _i64(colidx)
    nsl = (n + 31) // 32
    slice_ptr = np.empty(nsl + 1, np.int64)
    _lib.call("esr_sell_build", n, _lib.ptr(rowptr), _lib.ptr(perm), _lib.ptr(colidx), ncols,
              _lib.ptr(slice_ptr), None, None)
    total = int(slice_ptr[-1])
    col = np.empty(total, np.int32)
    src_pos = np.empty(total, np.int64)
    _lib.call("esr_sell_build", n, _lib.ptr(rowptr), _lib.ptr(perm), _lib.ptr(colidx), ncols,
              _lib.ptr(slice_ptr), _lib.ptr(col), _lib.ptr(src_pos))
    return slice_ptr, col, src_pos


def bisect_partition(n: int, src, dst, max_part: int):
    """Recursive-BFS-bisection parts of at most max_part vertices.  CUDA
    tensors: on the GPU (esr_bisect_partition_device), returning a CUDA
    int64 tensor; else on the host, returning a numpy array."""
    if isinstance(src, torch.Tensor) and src.is_cuda:
        return _bisect_partition_device(n, src, dst, max_part)
    src, dst = _i64(src), _i64(dst)
    part = np.empty(n, np.int64)
    nparts = ctypes.c_int64()
    _lib.call("esr_bisect_partition", n, src.shape[0], _lib.ptr(src), _lib.ptr(dst), int(max_part), _lib.ptr(part),
              ctypes.byref(nparts))
    return part, int(nparts.value)


def _bisect_partition_device(n: int, src: torch.Tensor, dst: torch.Tensor, max_part: int):
    dev = src.device
    src = src.to(torch.int64).contiguous()
    dst = dst.to(dev, torch.int64).contiguous()
    m = src.shape[0]
    nbytes = int(_lib.lib().esr_bisect_device_workspace_bytes(n, m, int(max_part)))
    if nbytes < 0:
        raise ValueError("graph sizes out of range for the device partition")
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    part = torch.empty(n, dtype=torch.int32, device=dev)
    nparts = ctypes.c_int64()
    _lib.call("esr_bisect_partition_device", n, m, _lib.ptr(src), _lib.ptr(dst), int(max_part), _lib.ptr(part),
              ctypes.byref(nparts), _lib.ptr(ws), nbytes, _lib.stream_handle(dev))
    return part.to(torch.int64), int(nparts.value)
