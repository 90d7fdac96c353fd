"""Native library: loads, exports every declared symbol, and its host-side
work (mesh, geometry, assembly, orderings) matches the reference fixtures
and the oracle exactly.  No device calls."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse
import scipy.sparse.csgraph

from easier_gb300 import _lib, mesh
from oracle import mesh as omesh
from oracle import sparse as osp

HEADER = Path(__file__).resolve().parent.parent / "include" / "esr_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(esr_[a-z0-9_]+)\s*\(", text)))


def test_library_loads_and_exports_every_declared_symbol():
    lib = _lib.lib()
    names = declared_functions()
    assert len(names) >= 25
    handle = ctypes.CDLL(str(_lib.library_path()))
    for name in names:
        assert hasattr(handle, name), name
    assert lib.esr_abi_version() == _lib.ABI_VERSION
    # the Python binding covers the whole C ABI
    assert set(names) <= set(_lib.exported_symbols())


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8])
def test_mesh_generator_matches_reference(golden, n):
    g = golden("mesh_small.npz")
    m = mesh.triangular_mesh(n)
    assert np.array_equal(m.src, g[f"n{n}_src"])
    assert np.array_equal(m.dst, g[f"n{n}_dst"])
    assert np.array_equal(m.cells.reshape(-1), g[f"n{n}_cells"])
    assert np.array_equal(m.bcells, g[f"n{n}_bcells"])
    assert np.array_equal(m.bpoints.reshape(-1), g[f"n{n}_bpoints"])
    assert np.array_equal(m.points.reshape(-1), g[f"n{n}_points"])


@pytest.mark.parametrize("n", [13, 64, 200])
def test_mesh_generator_matches_oracle_large(n):
    m = mesh.triangular_mesh(n)
    o = omesh.triangular_mesh(n)
    for k in ("src", "dst", "cells", "bcells", "bpoints", "points"):
        assert np.array_equal(getattr(m, k), o[k]), k
    nc, ne, nbc, npt = mesh.mesh_sizes(n)
    assert (nc, ne, nbc, npt) == (4 * n * n, 12 * n * n - 4 * n, 4 * n, (n + 1) ** 2 + n * n)


def test_swe_geometry_matches_reference(golden):
    g = golden("swe_geometry_n10.npz")
    geo = mesh.swe_geometry(mesh.triangular_mesh(10))
    for k in ("sx", "sy", "alpha", "area", "x", "y", "bsx", "bsy"):
        assert np.array_equal(getattr(geo, k), g[k]), k


@pytest.mark.parametrize("n", [7, 50])
def test_swe_geometry_matches_oracle(n):
    m = mesh.triangular_mesh(n)
    geo = mesh.swe_geometry(m)
    o = omesh.swe_geometry(omesh.triangular_mesh(n))
    for k in ("sx", "sy", "alpha", "area", "x", "y", "bsx", "bsy"):
        assert np.array_equal(getattr(geo, k), o[k]), k


def test_poisson_fv_matches_reference(golden):
    g = golden("poisson_fv_n10.npz")
    a = mesh.poisson_fv(mesh.triangular_mesh(10))
    for k in ("Af", "Ac", "centroid"):
        assert np.array_equal(getattr(a, k), g[k]), k
    # rho/b go through exp(): libm and torch may differ in the last bit
    for k in ("rho", "b"):
        assert np.allclose(getattr(a, k), g[k], rtol=4e-16, atol=0), k


@pytest.mark.parametrize("n,seed", [(4, None), (9, 3), (16, 5)])
def test_p1_assembly_matches_oracle(n, seed):
    kappa = None
    if seed is not None:
        kappa = mesh.kappa_from_field(mesh.gaussian_random_field(n, seed))
    s = mesh.p1_system(n, kappa)
    Av, A = omesh.p1_system(n, kappa)
    assert np.allclose(s.Av, Av, rtol=1e-14, atol=0)
    for r, c, v in zip(s.row, s.col, s.Ae):
        assert np.isclose(v, A.get((int(r), int(c)), 0.0), rtol=1e-14, atol=1e-300)
    assert np.all(np.diff(s.row) >= 0)
    # symmetric, and every nonzero coupling of the oracle is present
    M = scipy.sparse.coo_matrix((s.Ae, (s.row, s.col)), shape=(s.nunk, s.nunk)).tocsr()
    assert abs(M - M.T).max() == 0
    assert sum(1 for (a, b), v in A.items() if a != b and v != 0.0) == int((s.Ae != 0).sum())


def test_csr_from_index_is_the_stable_sort():
    rng = np.random.default_rng(0)
    idx = rng.integers(0, 97, 5000)
    rowptr, perm = mesh.csr_from_index(idx, 100)
    r2, p2 = osp.stable_csr(idx, 100)
    assert np.array_equal(rowptr, r2) and np.array_equal(perm, p2)
    with pytest.raises(ValueError):
        mesh.csr_from_index(np.array([0, 5, 100]), 100)
    with pytest.raises(ValueError):
        mesh.csr_from_index(np.array([-1]), 4)


@pytest.mark.parametrize("n", [1, 2, 4, 9])
def test_rcm_matches_oracle(n):
    m = mesh.triangular_mesh(n)
    order = mesh.rcm_order(m.nc, m.src, m.dst)
    assert np.array_equal(order, osp.rcm(m.nc, m.src, m.dst))


def test_rcm_bandwidth_close_to_scipy():
    m = mesh.triangular_mesh(40)
    order = mesh.rcm_order(m.nc, m.src, m.dst)
    assert np.array_equal(np.sort(order), np.arange(m.nc))
    G = scipy.sparse.coo_matrix((np.ones(m.ne), (m.src, m.dst)), shape=(m.nc, m.nc)).tocsr()
    sp_order = scipy.sparse.csgraph.reverse_cuthill_mckee(G, symmetric_mode=True)
    ours = osp.bandwidth(order, m.src, m.dst)
    theirs = osp.bandwidth(sp_order, m.src, m.dst)
    assert ours <= 1.25 * theirs, (ours, theirs)


def test_rcm_handles_disconnected_graph():
    src = np.array([0, 1, 3, 4])
    dst = np.array([1, 0, 4, 5])
    order = mesh.rcm_order(7, src, dst)
    assert np.array_equal(np.sort(order), np.arange(7))
    assert np.array_equal(order, osp.rcm(7, src, dst))


def test_sell_layout_keeps_row_order():
    rng = np.random.default_rng(2)
    n = 77
    row = np.sort(rng.integers(0, n, 400))
    col = rng.integers(0, n, 400)
    rowptr, perm = mesh.csr_from_index(row, n)
    slice_ptr, c, pos = mesh.sell_layout(n, rowptr, perm, col, n)
    assert slice_ptr[0] == 0 and np.all(np.diff(slice_ptr) % 32 == 0)
    for r in range(n):
        s, lane = divmod(r, 32)
        w = (slice_ptr[s + 1] - slice_ptr[s]) // 32
        got = [pos[slice_ptr[s] + 32 * k + lane] for k in range(w)]
        got = [g for g in got if g >= 0]
        assert got == list(perm[rowptr[r]:rowptr[r + 1]])
        assert all(c[slice_ptr[s] + 32 * k + lane] == col[perm[rowptr[r] + k]] for k in range(len(got)))
    with pytest.raises(ValueError):
        mesh.sell_layout(n, rowptr, perm, np.full(400, n), n)


def test_device_entry_points_check_their_arguments_first():
    """The host-stepping plan and the device partition refuse bad arguments
    before any CUDA call (dummy device pointers: run only where no GPU could
    be reached)."""
    import ctypes
    import pytest
    import torch
    if torch.cuda.is_available():
        pytest.skip("dummy device pointers: host-only check")
    lib = _lib.lib()
    d = 0x1000
    tiles = _lib.SweTiles(1000, 1, _lib.F32, 900, 800, 700, 100, d, d, d, d, d, d, d, 0, 1)
    plan = ctypes.c_void_p()
    e = d + 0x100
    for args, msg in (((d, e, None, d, 8), b"staging"), ((d, e, d, d, 0), b"chunks"), ((d, e, d, d, 65), b"chunks"),
                      ((d, d + 8, d, d, 8), b"aligned"), ((d, d, d, d, 8), b"distinct")):
        a, b_, stage, tl, ch = args
        rc = lib.esr_swe_host_plan_create(ctypes.byref(tiles), a, b_, stage, tl, ch, ctypes.byref(plan))
        assert rc == 1, (args, rc)
        assert msg in lib.esr_last_error(), (args, lib.esr_last_error())
    assert lib.esr_swe_host_step(None, 1e-3, d, 1, None) == 1
    assert lib.esr_bisect_device_workspace_bytes(0, 10, 5) == -1
    assert lib.esr_bisect_device_workspace_bytes(10, 10, 0) == -1
    assert lib.esr_bisect_device_workspace_bytes(1 << 31, 10, 5) == -1
    np_ = ctypes.c_int64()
    assert lib.esr_bisect_partition_device(0, 0, d, d, 5, d, ctypes.byref(np_), d, 1 << 20, None) == 1
    assert lib.esr_bisect_partition_device(10, 5, None, d, 5, d, ctypes.byref(np_), d, 1 << 20, None) == 1
    assert lib.esr_bisect_partition_device(10, 5, d, d, 5, d, ctypes.byref(np_), d, 16, None) == 1
    assert b"workspace too small" in lib.esr_last_error()
