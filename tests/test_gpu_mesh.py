"""Mesh generation, shallow-water geometry and FV Poisson assembly on the
GPU against the host generator and assembly (which are bitwise the
reference's: tests/test_oracle_golden.py, tests/test_native_host.py)."""
import time

import numpy as np
import pytest
import torch

import easier_gb300 as esr
from easier_gb300 import mesh, ops, workloads

pytestmark = pytest.mark.gpu


def _np(t):
    return t.cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


@pytest.mark.parametrize("n", [1, 2, 7, 100, 333])
def test_device_mesh_geometry_fv_equal_host(n):
    h = mesh.triangular_mesh(n)
    d = mesh.triangular_mesh(n, device="cuda")
    for k in ("src", "dst", "cells", "bcells", "bpoints", "points"):
        assert np.array_equal(_np(getattr(d, k)), getattr(h, k)), k
    gh, gd = mesh.swe_geometry(h), mesh.swe_geometry(d)
    for k in ("sx", "sy", "alpha", "area", "x", "y", "bsx", "bsy"):
        assert np.array_equal(_np(getattr(gd, k)), getattr(gh, k)), k
    fh, fd = mesh.poisson_fv(h), mesh.poisson_fv(d)
    for k in ("Af", "Ac", "centroid"):
        assert np.array_equal(_np(getattr(fd, k)), getattr(fh, k)), k
    for k in ("rho", "b"):  # CUDA's exp: within a few ulp
        a, b = _np(getattr(fd, k)), getattr(fh, k)
        assert np.all(np.abs(a - b) <= 8 * np.spacing(np.abs(b))), k
    assert ops.device_status() == 0


def test_device_mesh_and_geometry_full_size():
    """The bench's mesh (N=2000: 16,000,000 cells, 47,992,000 edges): bitwise
    the host's; prints both times."""
    n = 2000
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d = mesh.triangular_mesh(n, device="cuda")
    gd = mesh.swe_geometry(d)
    torch.cuda.synchronize()
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    h = mesh.triangular_mesh(n)
    gh = mesh.swe_geometry(h)
    t_host = time.perf_counter() - t0
    print(f"\nN=2000 mesh + geometry: GPU {t_dev:.3f} s, host {t_host:.3f} s")
    for k in ("src", "dst", "cells", "bcells", "points"):
        assert np.array_equal(_np(getattr(d, k)), getattr(h, k)), k
    for k in ("sx", "sy", "alpha", "area", "bsx", "bsy"):
        assert np.array_equal(_np(getattr(gd, k)), getattr(gh, k)), k


def test_swe_module_from_device_mesh_steps_like_host_built_one():
    """make_swe(..., device='cuda') builds mesh and geometry on the GPU; the
    compiled module then steps bit for bit like the host-built one."""
    outs = []
    for device in ("cpu", "cuda"):
        eqn = workloads.make_swe(40, dt=5e-4, dtype=torch.float32, device=device)
        [eqn] = esr.compile([eqn], "cuda")
        for _ in range(5):
            eqn()
        outs.append([getattr(eqn, k).collect().cpu() for k in ("h", "uh", "vh")])
    for a, b in zip(*outs):
        assert torch.equal(a, b)
