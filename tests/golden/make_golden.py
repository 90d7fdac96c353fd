"""Generate the golden fixtures in this directory by running the reference.

Runs the EASIER reference package itself (imported from its source tree:
``EASIER_REFERENCE_ROOT``, else the tree ``oracle/build_ref.py`` finds) on its
CPU backend at world size 1, with its C++ extension compiled by
``oracle/build_ref.py``.  ``h5py`` / ``more_itertools`` / ``matplotlib`` are
absent here, so ``_stubs/`` stands in for them and the tutorial's HDF5 files
are replaced by an in-memory store (``esr.hdf5`` -> in-memory loader,
``Tensor.save`` -> store).  The tutorial modules themselves run unmodified.

OpenMP is pinned to one thread: the reference mesh generator writes shared
corner points from several loop iterations, so with more threads their last
bit depends on timing.

Usage:  python tests/golden/make_golden.py [group ...]   (groups: mesh,
        selector_reducer, poisson, poisson_fv_n100, linsys_p1, swe; default all)
Writes: tests/golden/*.npz (small; committed).
"""
import os
import sys
import time
from pathlib import Path

os.environ["OMP_NUM_THREADS"] = "1"
os.environ.setdefault("WORLD_SIZE", "1")
os.environ.setdefault("RANK", "0")
os.environ.setdefault("LOCAL_RANK", "0")
os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
os.environ.setdefault("MASTER_PORT", "29533")
os.environ.setdefault("EASIER_LOG_LEVEL", "WARNING")

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent

import numpy as np  # noqa: E402
import torch  # noqa: E402

torch.set_num_threads(1)
sys.path.insert(0, str(HERE / "_stubs"))
sys.path.insert(0, str(ROOT / "oracle"))
import build_ref  # noqa: E402

REF = build_ref.reference_root()
if REF is None:
    sys.exit("make_golden: no reference tree (set EASIER_REFERENCE_ROOT)")
_ext = build_ref.build(REF)
sys.modules["easier.cpp_extension"] = _ext
sys.path.insert(0, str(REF))
sys.path.insert(0, str(REF / "tutorial" / "shallow_water_equation"))
sys.path.insert(0, str(REF / "tutorial" / "poisson"))

import easier as esr  # noqa: E402
from easier.core.runtime.data_loader import InMemoryTensorLoader  # noqa: E402

STORE = {}
# dtype every floating dataset is served in.  The reference's
# Module.to(torch.float32) retypes FulledTensorLoader data (uh, vh) but a
# loader built from a file or an in-memory tensor keeps the dtype it was
# constructed with, so an FP32 run needs the datasets themselves in FP32.
FORCE_FLOAT = None


def _hdf5(file, dataset, dtype=None, device=None, **kw):
    t = STORE[(file, dataset)]
    if dtype is not None:
        t = t.to(dtype)
    if FORCE_FLOAT is not None and t.dtype.is_floating_point:
        t = t.to(FORCE_FLOAT)
    return InMemoryTensorLoader(t)


def _save(self, path, name, **kw):
    STORE[(path, name)] = self.collect().cpu().clone()


esr.hdf5 = _hdf5
esr.Tensor.save = _save
esr.init("gloo")

from assemble_shallow_water import assemble_shallow_water  # noqa: E402
from swe_main import ShallowWaterEquation  # noqa: E402
from assemble_poisson import assemble_poisson  # noqa: E402
from poisson_main import Poisson  # noqa: E402
from easier.numeric.solver import CG, GMRES  # noqa: E402


def put_mesh(n):
    src, dst, cells, bcells, bpoints, points = _ext.generate_triangular_mesh(n)
    path = f"mesh{n}"
    for k, v in dict(src=src, dst=dst, cells=cells.reshape(-1, 3), bcells=bcells, bpoints=bpoints.reshape(-1, 2),
                     points=points.reshape(-1, 2)).items():
        STORE[(path, k)] = v.clone()
    return path


def mesh_fixtures():
    out = {}
    for n in (1, 2, 3, 5, 8):
        r = _ext.generate_triangular_mesh(n)
        for k, v in zip(("src", "dst", "cells", "bcells", "bpoints", "points"), r):
            out[f"n{n}_{k}"] = v.numpy()
    np.savez_compressed(HERE / "mesh_small.npz", **out)


def swe_run(n, steps, dt, dtype, centre_bump):
    mp = put_mesh(n)
    sp = f"sw{n}"
    assemble_shallow_water(mp, sp)
    geom = {k: STORE[(sp, k)].numpy() for k in ("x", "y", "area", "sx", "sy", "bsx", "bsy", "h", "alpha")}
    if centre_bump:
        x, y = STORE[(sp, "x")], STORE[(sp, "y")]
        STORE[(sp, "h")] = 1 + 0.1 * torch.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.01)
    h0 = STORE[(sp, "h")].numpy().copy()
    global FORCE_FLOAT
    FORCE_FLOAT = dtype if dtype != torch.float64 else None
    try:
        eqn = ShallowWaterEquation(mp, sp, dt=dt)
        if dtype != torch.float64:
            eqn.to(dtype)
        [eqn] = esr.compile([eqn], "cpu", partition_mode="evenly")
    finally:
        FORCE_FLOAT = None
    assert all(t.dtype == dtype for t in (eqn.h, eqn.uh, eqn.vh, eqn.sx, eqn.area))
    t0 = time.perf_counter()
    for _ in range(steps):
        eqn()
    wall = time.perf_counter() - t0
    res = dict(h0=h0, h=eqn.h.collect().numpy(), uh=eqn.uh.collect().numpy(), vh=eqn.vh.collect().numpy(),
               steps=steps, dt=dt, wall_s=wall)
    return geom, res


def swe_fixtures():
    geom, res = swe_run(10, 100, 0.005, torch.float64, centre_bump=False)
    np.savez_compressed(HERE / "swe_geometry_n10.npz", **geom)
    np.savez_compressed(HERE / "swe_n10_f64_tutorial.npz", **res)
    _, res = swe_run(10, 100, 0.005, torch.float32, centre_bump=False)
    np.savez_compressed(HERE / "swe_n10_f32_tutorial.npz", **res)
    # the reference's CPU-runnable benchmark case: N=100, centred bump,
    # dt=5e-4, 1000 steps
    for dtype, tag in ((torch.float64, "f64"), (torch.float32, "f32")):
        _, res = swe_run(100, 1000, 5e-4, dtype, centre_bump=True)
        np.savez_compressed(HERE / f"swe_n100_{tag}_1000steps.npz", **res)
        print(f"swe n100 {tag}: {res['wall_s']:.1f} s for 1000 steps")


def poisson_fixtures():
    n = 10
    mp = put_mesh(n)
    pp = f"poisson{n}"
    assemble_poisson(mp, pp)
    asm = {k: STORE[(pp, k)].numpy() for k in ("Af", "Ac", "b", "rho", "centroid")}
    np.savez_compressed(HERE / "poisson_fv_n10.npz", **asm)
    out = {}
    for solver, tag in ((CG, "cg"), (GMRES, "gmres")):
        eqn = Poisson(mp, pp)
        sol = solver(eqn.A, eqn.b, eqn.x)
        [eqn, sol] = esr.compile([eqn, sol], "cpu", partition_mode="evenly")
        info = sol.solve(rtol=1e-8, maxiter=2000)
        out[f"{tag}_x"] = eqn.x.collect().numpy()
        out[f"{tag}_iters"] = np.array(info["iters"])
        out[f"{tag}_residual"] = np.array(info["residual"])
    np.savez_compressed(HERE / "poisson_fv_n10_solve.npz", **out)


def poisson_fv_n100_fixture():
    """The tutorial's FV Poisson at N=100 (40,000 cells, 119,600 directed
    edges) solved by the reference's CG (no preconditioner, as the tutorial
    does) to relative residual 1e-8."""
    n = 100
    mp = put_mesh(n)
    pp = f"poisson{n}"
    assemble_poisson(mp, pp)
    eqn = Poisson(mp, pp)
    sol = CG(eqn.A, eqn.b, eqn.x)
    [eqn, sol] = esr.compile([eqn, sol], "cpu", partition_mode="evenly")
    t0 = time.time()
    info = sol.solve(rtol=1e-8, maxiter=5000)
    out = {"cg_x": eqn.x.collect().numpy(), "cg_iters": np.array(info["iters"]),
           "cg_residual": np.array(info["residual"])}
    np.savez_compressed(HERE / "poisson_fv_n100_cg.npz", **out)
    print(f"poisson fv n100: {info['iters']} CG iterations in {time.time() - t0:.1f} s")


def linsys_p1_fixture():
    """The reference's Linsys + CG on a P1 system given as arrays (no
    reference assembly exists for P1; the arrays come from a plain numpy
    stencil written here)."""
    n = 12
    m = n - 1
    rows, cols, vals = [], [], []
    diag = np.full(m * m, 4.0)
    for j in range(m):
        for i in range(m):
            u = j * m + i
            for di, dj, v in ((-1, -1, 0.0), (0, -1, -1.0), (-1, 0, -1.0), (1, 0, -1.0), (0, 1, -1.0), (1, 1, 0.0)):
                ii, jj = i + di, j + dj
                if 0 <= ii < m and 0 <= jj < m:
                    rows.append(u)
                    cols.append(jj * m + ii)
                    vals.append(v)
    rng = np.random.default_rng(7)
    b = rng.standard_normal(m * m)

    class P1(esr.Module):
        def __init__(self):
            super().__init__()
            self.reducer = esr.Reducer(torch.tensor(rows), m * m)
            self.selector = esr.Selector(torch.tensor(cols))
            self.x = esr.Tensor(torch.zeros(m * m, dtype=torch.float64), mode="partition")
            self.b = esr.Tensor(torch.tensor(b), mode="partition")
            self.Av = esr.Tensor(torch.tensor(diag), mode="partition")
            self.Ae = esr.Tensor(torch.tensor(vals, dtype=torch.float64), mode="partition")
            from easier.numeric import Linsys
            self.A = Linsys(self.Av, self.Ae, self.selector, self.reducer)

    eqn = P1()
    sol = CG(eqn.A, eqn.b, eqn.x)
    [eqn, sol] = esr.compile([eqn, sol], "cpu", partition_mode="evenly")
    info = sol.solve(rtol=1e-10, maxiter=1000)
    np.savez_compressed(HERE / "linsys_p1_n12_cg.npz", row=np.array(rows), col=np.array(cols), Ae=np.array(vals),
                        Av=diag, b=b, x=eqn.x.collect().numpy(), iters=np.array(info["iters"]),
                        residual=np.array(info["residual"]))


def selector_reducer_fixture():
    """Selector / Reducer outputs of the reference on random data, every
    reduce op, 1-D and 3-D rows, with and without ``out=``."""
    g = torch.Generator().manual_seed(11)
    out = {}
    m, n_in, n = 200, 37, 23
    idx_sel = torch.randint(0, n_in, (m,), generator=g)
    idx_red = torch.randint(0, n, (m,), generator=g)
    idx_red[idx_red == 5] = 6  # leave row 5 unreferenced
    out["sel_idx"] = idx_sel.numpy()
    out["red_idx"] = idx_red.numpy()
    for dt, tag in ((torch.float64, "f64"), (torch.float32, "f32")):
        x1 = torch.randn(n_in, generator=g).to(dt)
        x3 = torch.randn(n_in, 3, 2, generator=g).to(dt)
        e1 = torch.randn(m, generator=g).to(dt)
        e3 = torch.randn(m, 3, 2, generator=g).to(dt)
        o3 = torch.randn(n, 3, 2, generator=g).to(dt)
        out[f"{tag}_x1"], out[f"{tag}_x3"] = x1.numpy(), x3.numpy()
        out[f"{tag}_e1"], out[f"{tag}_e3"], out[f"{tag}_o3"] = e1.numpy(), e3.numpy(), o3.numpy()
        sel = esr.Selector(idx_sel)
        sel.idx = idx_sel.clone()
        sel.easier_index_status = "rewritten"
        out[f"{tag}_sel1"] = sel(x1).numpy()
        out[f"{tag}_sel3"] = sel(x3).numpy()
        for op in ("sum", "prod", "mean", "amax", "amin"):
            red = esr.Reducer(idx_red, n, reduce=op)
            red.idx = idx_red.clone()
            red.easier_index_status = "rewritten"
            out[f"{tag}_{op}_1"] = red(e1).numpy()
            out[f"{tag}_{op}_3"] = red(e3).numpy()
            out[f"{tag}_{op}_3out"] = red(e3, out=o3.clone()).numpy()
    np.savez_compressed(HERE / "selector_reducer.npz", **out)


GROUPS = {"mesh": mesh_fixtures, "selector_reducer": selector_reducer_fixture, "poisson": poisson_fixtures,
          "poisson_fv_n100": poisson_fv_n100_fixture, "linsys_p1": linsys_p1_fixture, "swe": swe_fixtures}

if __name__ == "__main__":
    # python tests/golden/make_golden.py [group ...]  (default: all groups)
    t0 = time.time()
    for name in (sys.argv[1:] or list(GROUPS)):
        GROUPS[name]()
    print(f"golden fixtures written in {time.time() - t0:.0f} s")
