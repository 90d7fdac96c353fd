"""The C ABI from a C99 program: include/esr_gb300.h compiles as C, the
library links and its host-side entry points (mesh, stable CSR, RCM, tile
partition) give the same arrays as through the Python binding and the
oracle.  No device calls."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from easier_gb300 import _lib, mesh
from oracle import sparse as osp

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def c_program(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = _lib.library_path()
    _lib.lib()  # builds the library if it is missing
    out = tmp_path_factory.mktemp("cabi") / "c_abi_host"
    cmd = [cc, "-std=c99", "-Wall", "-Werror", "-I", str(HERE.parent / "include"), str(HERE / "c_abi_host.c"),
           str(lib), f"-Wl,-rpath,{lib.parent}", "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


@pytest.mark.parametrize("n,max_part", [(6, 40), (23, 300)])
def test_host_entry_points_from_c(c_program, tmp_path, n, max_part):
    subprocess.run([str(c_program), str(n), str(max_part), str(tmp_path)], check=True, timeout=60)

    def load(name):
        return np.fromfile(tmp_path / f"{name}.bin", dtype="<i8")

    nc, ne, nbc, npt, nparts = (int(v) for v in load("sizes"))
    assert (nc, ne, nbc, npt) == mesh.mesh_sizes(n)
    m = mesh.triangular_mesh(n)
    assert np.array_equal(load("src"), m.src)
    rowptr, perm = osp.stable_csr(m.dst, nc)
    assert np.array_equal(load("rowptr"), rowptr) and np.array_equal(load("perm"), perm)
    order = load("order")
    assert np.array_equal(order, mesh.rcm_order(nc, m.src, m.dst))
    assert np.array_equal(order, np.asarray(osp.rcm(nc, m.src, m.dst)))
    part, k = mesh.bisect_partition(nc, m.src, m.dst, max_part)
    assert nparts == k and np.array_equal(load("part"), part)
    assert np.bincount(part).max() <= max_part


@pytest.mark.gpu
def test_device_entry_points_from_c(tmp_path):
    """Selector gather + Reducer segment sum called from C99 on the caller's
    stream: bitwise the host loops in the reference's edge order."""
    import os
    cc = shutil.which("gcc") or shutil.which("cc")
    cuda = os.environ.get("CUDA_HOME") or "/usr/local/cuda"
    if cc is None or not (Path(cuda) / "include" / "cuda_runtime_api.h").exists():
        pytest.skip("no C compiler or CUDA headers")
    lib = _lib.library_path()
    _lib.lib()
    exe = tmp_path / "c_abi_device"
    cmd = [cc, "-std=c99", "-Wall", "-Werror", "-I", str(HERE.parent / "include"), "-I", f"{cuda}/include",
           str(HERE / "c_abi_device.c"), str(lib), f"-L{cuda}/lib64", "-lcudart", "-lm",
           f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{cuda}/lib64", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    res = subprocess.run([str(exe), "37"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0 and res.stdout.strip() == "ok", res.stderr
