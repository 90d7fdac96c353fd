"""Fused shallow-water step on the GPU, through esr.compile(backend='cuda'),
against the reference's own runs (golden fixtures) and the oracle."""
import numpy as np
import pytest
import torch

import easier_gb300 as esr
from easier_gb300 import workloads
from oracle import mesh as omesh
from oracle import swe as oswe

pytestmark = pytest.mark.gpu


def _run(n, steps, dt, dtype, h0, fuse=True):
    eqn = workloads.make_swe(n, dt=dt, dtype=dtype, h=h0)
    [eqn] = esr.compile([eqn], "cuda", fuse=fuse)
    for _ in range(steps):
        eqn()
    torch.cuda.synchronize()
    return eqn, [getattr(eqn, k).collect().cpu().numpy() for k in ("h", "uh", "vh")]


@pytest.mark.parametrize("tag,dtype", [("f64", torch.float64), ("f32", torch.float32)])
def test_tutorial_n10_bitwise_vs_reference(golden, tag, dtype):
    g = golden(f"swe_n10_{tag}_tutorial.npz")
    eqn, out = _run(10, int(g["steps"]), float(g["dt"]), dtype, g["h0"])
    assert getattr(eqn, "easier_fused_engine", None) is not None
    for k, v in zip(("h", "uh", "vh"), out):
        assert np.array_equal(v, g[k]), k


@pytest.mark.parametrize("tag,dtype", [("f64", torch.float64), ("f32", torch.float32)])
def test_n100_1000_steps_bitwise_vs_reference(golden, tag, dtype):
    """The reference's CPU-runnable case at full length (40,000 cells,
    1,000 steps): bitwise equal to the reference's CPU backend."""
    g = golden(f"swe_n100_{tag}_1000steps.npz")
    eqn = workloads.make_swe(100, dt=float(g["dt"]), dtype=dtype, h=g["h0"])
    [eqn] = esr.compile([eqn], "cuda")
    eng = eqn.easier_fused_engine
    eng.step(int(g["steps"]))
    torch.cuda.synchronize()
    for k in ("h", "uh", "vh"):
        v = getattr(eqn, k).collect().cpu().numpy()
        assert np.array_equal(v, g[k]), k
    if dtype == torch.float32:
        # FP32 against the FP64 reference run: the stated 1e-5 relative bar
        g64 = golden("swe_n100_f64_1000steps.npz")
        h = eqn.h.collect().cpu().double().numpy()
        assert np.abs(h - g64["h"]).max() <= 1e-5 * np.abs(g64["h"]).max()


def test_per_op_path_equals_fused_path():
    n, steps = 24, 20
    m = omesh.triangular_mesh(n)
    geo = omesh.swe_geometry(m)
    h0 = 1 + 0.1 * np.exp(-((geo["x"] - 0.3) ** 2 + (geo["y"] - 0.6) ** 2) / 0.02)
    _, fused = _run(n, steps, 1e-3, torch.float64, h0, fuse=True)
    eqn, perop = _run(n, steps, 1e-3, torch.float64, h0, fuse=False)
    assert getattr(eqn, "easier_fused_engine", None) is None
    for a, b in zip(fused, perop):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_larger_mesh_bitwise_vs_oracle(dtype):
    n, steps, dt = 150, 5, 5e-4
    m = omesh.triangular_mesh(n)
    geo = omesh.swe_geometry(m)
    h0 = 1 + 0.1 * np.exp(-((geo["x"] - 0.5) ** 2 + (geo["y"] - 0.5) ** 2) / 0.01)
    p = oswe.SweProblem(m["src"], m["dst"], m["bcells"], geo["sx"], geo["sy"], geo["alpha"], geo["bsx"],
                        geo["bsy"], geo["area"], dt, dtype)
    ref = p.run(torch.from_numpy(h0).to(dtype), torch.zeros(m["cells"].shape[0], dtype=dtype),
                torch.zeros(m["cells"].shape[0], dtype=dtype), steps)
    _, out = _run(n, steps, dt, dtype, h0)
    for a, b in zip(out, ref):
        assert np.array_equal(a, b.numpy())


def test_collect_order_and_rcm_layout():
    eqn = workloads.make_swe(12, dt=1e-3)
    h_orig = eqn.h.easier_data_loader.fully_load("cpu").numpy()
    [eqn] = esr.compile([eqn], "cuda")
    eng = eqn.easier_fused_engine
    assert eng.reorder == "rcm"
    assert eqn.h.elempart is not None
    assert np.array_equal(eqn.h.collect().cpu().numpy(), h_orig)
    assert np.array_equal(eqn.x.collect().cpu().numpy(), eqn.x.easier_data_loader.fully_load("cpu").numpy())
    # the state views share the engine's packed buffer
    assert eqn.h.data.data_ptr() == eng.state.data_ptr()


def test_deterministic_and_in_place_writes_respected():
    eqn = workloads.make_swe(30, dt=5e-4)
    [eqn] = esr.compile([eqn], "cuda")
    a0 = eqn.h.collect().clone()
    for _ in range(10):
        eqn()
    a = eqn.h.collect()
    eqn2 = workloads.make_swe(30, dt=5e-4)
    [eqn2] = esr.compile([eqn2], "cuda")
    for _ in range(10):
        eqn2()
    assert torch.equal(a, eqn2.h.collect())
    # an in-place write through the esr.Tensor reaches the fused state
    eqn.h[:] = 1.0
    eqn()
    assert not torch.equal(eqn.h.collect(), a0)


def test_delta_matches_oracle():
    n = 16
    m = omesh.triangular_mesh(n)
    geo = omesh.swe_geometry(m)
    rng = np.random.default_rng(0)
    h = 1 + 0.1 * rng.random(4 * n * n)
    uh = 0.01 * rng.standard_normal(4 * n * n)
    vh = 0.01 * rng.standard_normal(4 * n * n)
    p = oswe.SweProblem(m["src"], m["dst"], m["bcells"], geo["sx"], geo["sy"], geo["alpha"], geo["bsx"],
                        geo["bsy"], geo["area"], 1e-3)
    ref = p.delta(*(torch.from_numpy(a) for a in (h, uh, vh)))
    eqn = workloads.make_swe(n, dt=1e-3, h=h)
    [eqn] = esr.compile([eqn], "cuda")
    eng = eqn.easier_fused_engine
    st = eng.state.clone()
    order = eng.order
    st[:, 1] = torch.from_numpy(uh).cuda()[order]
    st[:, 2] = torch.from_numpy(vh).cuda()[order]
    d = eng.delta(st)
    for j in range(3):
        got = torch.empty(4 * n * n, dtype=torch.float64)
        got[order.cpu()] = d[:, j].cpu()
        assert torch.equal(got, ref[j])


@pytest.mark.parametrize("n,tile,cta", [(37, 4096, 1024), (150, 4096, 1024), (150, 2048, 512), (150, 900, 256)])
def test_tiled_equals_staged_fp32(n, tile, cta, monkeypatch):
    """The tiled step (each CTA size: 1, 2 or 4 CTAs per SM) is bitwise the
    staged step."""
    from easier_gb300 import swe
    monkeypatch.setattr(swe, "DEFAULT_TILE_CELLS", tile)
    outs = []
    for mode in ("tiled", "staged"):
        monkeypatch.setattr(swe, "DEFAULT_MODE", mode)
        eqn = workloads.make_swe(n, dt=5e-4, dtype=torch.float32)
        [eqn] = esr.compile([eqn], "cuda")
        eng = eqn.easier_fused_engine
        assert eng.tiled == (mode == "tiled")
        if eng.tiled:
            assert eng.tile_threads() == cta
        eng.step(7)
        eqn()
        outs.append([getattr(eqn, k).collect().cpu() for k in ("h", "uh", "vh")])
    for a, b in zip(*outs):
        assert torch.equal(a, b)


@pytest.mark.parametrize("tag,dtype,tol", [("f32", torch.float32, 1e-5), ("f64", torch.float64, 1e-10)])
@pytest.mark.parametrize("mode", ["tiled", "staged"])
def test_fast_precision_within_stated_tolerance(golden, tag, dtype, tol, mode, monkeypatch):
    """precision='fast' after 1,000 steps at N=100 against the reference's
    FP64 run: relative max-norm error within 1e-5 (FP32) / 1e-10 (FP64)."""
    from easier_gb300 import swe
    monkeypatch.setattr(swe, "DEFAULT_MODE", mode)
    g = golden(f"swe_n100_{tag}_1000steps.npz")
    g64 = golden("swe_n100_f64_1000steps.npz")
    eqn = workloads.make_swe(100, dt=float(g["dt"]), dtype=dtype, h=g["h0"])
    [eqn] = esr.compile([eqn], "cuda", precision="fast")
    eng = eqn.easier_fused_engine
    assert eng.precision == "fast" and eng.tiled == (mode == "tiled" and dtype == torch.float32)
    eng.step(int(g["steps"]))
    got = np.concatenate([getattr(eqn, k).collect().cpu().double().numpy() for k in ("h", "uh", "vh")])
    ref = np.concatenate([g64[k] for k in ("h", "uh", "vh")])
    # relative max-norm error of the state vector (h, uh, vh)
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


def test_full_size_tiled_equals_staged_and_conserves_mass(monkeypatch):
    """The bench's mesh (N=2000: 16,000,000 cells, 4,572 tiles): the tiled
    step is bitwise the staged step in exact arithmetic (every tile, halo
    ring and face slot at the largest layout), and the fast tiled step keeps
    the total mass sum(h * area) (the central flux cancels across each
    interior face; walls carry no mass flux) to FP32 rounding."""
    from easier_gb300 import swe
    n, steps, dt = 2000, 2, 2.5e-4
    outs = []
    for mode in ("tiled", "staged"):
        monkeypatch.setattr(swe, "DEFAULT_MODE", mode)
        eqn = workloads.make_swe(n, dt=dt, dtype=torch.float32)
        [eqn] = esr.compile([eqn], "cuda", precision="exact")
        eng = eqn.easier_fused_engine
        assert eng.tiled == (mode == "tiled")
        eng.step(steps)
        outs.append([getattr(eqn, k).collect() for k in ("h", "uh", "vh")])
        if mode == "tiled":
            area = eqn.area.collect().double()
            mass0 = float((outs[0][0].double() * area).sum())
            eng.set_precision("fast")
            eng.step(20)
            mass1 = float((eqn.h.collect().double() * area).sum())
            assert abs(mass1 - mass0) <= 1e-6 * abs(mass0), (mass0, mass1)
            assert bool(torch.isfinite(eqn.h.collect()).all())
        del eqn, eng
        torch.cuda.empty_cache()
    for a, b in zip(*outs):
        assert torch.equal(a, b)


@pytest.mark.parametrize("n,target", [(37, None), (150, 300), (300, None), (400, 700), (400, 1450), (400, 1900)])
def test_pipelined_tile_kernel_equals_blocked_kernel_bitwise(n, target, monkeypatch):
    """Fast arithmetic: the persistent pipelined tile kernel (state of the
    next tile prefetched, geometry in registers, packed FP32x2 arithmetic)
    is bitwise the one-CTA-per-tile kernel on the same layout, with one tile
    per CTA (N=37, 150 without more tiles than SMs) and with CTAs walking
    several tiles (more tiles than SMs)."""
    from easier_gb300 import swe
    if target:
        monkeypatch.setattr(swe, "PIPE_TILE_TARGET", target)
    eqn = workloads.make_swe(n, dt=5e-4, dtype=torch.float32)
    [eqn] = esr.compile([eqn], "cuda", precision="fast")
    eng = eqn.easier_fused_engine
    assert eng.tiled and eng.tile_kernel_name().startswith("pipelined"), eng.describe()
    s0 = eng.state.clone()
    outs = []
    kernels = ["pipelined_512", "blocked"]
    if eng.tile_stats["max_own"] <= 1536:
        kernels.append("pipelined_768")
    for kern in kernels:
        eng.tile_kernel = kern
        eng.state.copy_(s0)
        eng.step(7)
        torch.cuda.synchronize()
        outs.append(eng.state.clone())
    from easier_gb300 import ops
    assert ops.device_status() == 0
    for o in outs[1:]:
        assert torch.equal(outs[0], o)


def _renamed_swe(n, dt, dtype):
    """The tutorial's shallow-water module with every attribute renamed and
    the geometry tensors declared in another order: the fused engine must
    find the roles from the module's structure."""
    from easier_gb300 import mesh

    class Renamed(esr.Module):
        def __init__(self):
            super().__init__()
            m = mesh.triangular_mesh(n)
            g = mesh.swe_geometry(m)
            t = lambda a: torch.as_tensor(a)  # noqa: E731
            self.step_size = dt
            self.label = 3.5   # another float attribute: not the step size
            self.to_cell = esr.Reducer(t(m.dst), m.nc)
            self.take_a = esr.Selector(t(m.src))
            self.take_b = esr.Selector(t(m.dst))
            self.to_cell_w = esr.Reducer(t(m.bcells), m.nc)
            self.take_w = esr.Selector(t(m.bcells))
            f = torch.float64
            self.cx = esr.Tensor(t(g.x).to(f), mode="partition")
            self.w_ny = esr.Tensor(t(g.bsy).to(f), mode="partition")
            self.vol = esr.Tensor(t(g.area).to(f), mode="partition")
            self.weight = esr.Tensor(t(g.alpha).to(f), mode="partition")
            self.ny = esr.Tensor(t(g.sy).to(f), mode="partition")
            self.w_nx = esr.Tensor(t(g.bsx).to(f), mode="partition")
            self.nx = esr.Tensor(t(g.sx).to(f), mode="partition")
            self.cy = esr.Tensor(t(g.y).to(f), mode="partition")
            self.q = esr.Tensor(esr.zeros((m.nc,), dtype=f), mode="partition")
            self.depth = esr.Tensor(t(mesh.gaussian_bump(g.x, g.y)).to(f), mode="partition")
            self.p = esr.Tensor(esr.zeros((m.nc,), dtype=f), mode="partition")

        def face(self, phi):
            return (1 - self.weight) * self.take_a(phi) + self.weight * self.take_b(phi)

        def rate(self, h, uh, vh):
            h_f, uh_f, vh_f = self.face(h), self.face(uh), self.face(vh)
            u_f = uh_f / h_f
            v_f = vh_f / h_f
            hsq = 0.5 * h_f * h_f
            a = uh_f * self.nx
            b = vh_f * self.ny
            wall = 0.5 * self.take_w(h) ** 2
            dh = -(self.to_cell(a + b)) / self.vol
            du = -(self.to_cell((u_f * uh_f + hsq) * self.nx + u_f * b) + self.to_cell_w(wall * self.w_nx)) / self.vol
            dv = -(self.to_cell(v_f * a + (v_f * vh_f + hsq) * self.ny) + self.to_cell_w(wall * self.w_ny)) / self.vol
            return dh, du, dv

        def forward(self):
            k, h, p, q = self.step_size, self.depth, self.p, self.q
            a1, b1, c1 = self.rate(h, p, q)
            a2, b2, c2 = self.rate(h + 0.5 * k * a1, p + 0.5 * k * b1, q + 0.5 * k * c1)
            a3, b3, c3 = self.rate(h + 0.5 * k * a2, p + 0.5 * k * b2, q + 0.5 * k * c2)
            a4, b4, c4 = self.rate(h + k * a3, p + k * b3, q + k * c3)
            self.depth[:] += k / 6 * (a1 + a2 + a3 + a4)
            self.p[:] += k / 6 * (b1 + b2 + b3 + b4)
            self.q[:] += k / 6 * (c1 + c2 + c3 + c4)

    mod = Renamed()
    if dtype != torch.float64:
        mod.to(dtype)
    return mod


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_engine_finds_roles_of_a_renamed_module(dtype):
    """A module with the tutorial's step under other attribute names gets the
    fused engine (roles found from its structure, checked on its own
    forward) and steps bit for bit like the tutorial module."""
    n, dt, steps = 30, 5e-4, 6
    ren = _renamed_swe(n, dt, dtype)
    [ren] = esr.compile([ren], "cuda")
    assert getattr(ren, "easier_fused_engine", None) is not None
    for _ in range(steps):
        ren()
    tut = workloads.make_swe(n, dt=dt, dtype=dtype)
    [tut] = esr.compile([tut], "cuda")
    for _ in range(steps):
        tut()
    for a, b in (("depth", "h"), ("p", "uh"), ("q", "vh")):
        assert torch.equal(getattr(ren, a).collect().cpu(), getattr(tut, b).collect().cpu()), a


@pytest.mark.parametrize("precision", ["fast", "exact"])
def test_host_resident_stepping_equals_device_stepping(precision):
    """SweEngine.step_host (esr_swe_host_step: chunked uploads and downloads
    of a state in pinned host memory, overlapped both ways) gives bitwise
    the device-resident steps, for any chunk count, and leaves the module's
    views on the result."""
    eqn = workloads.make_swe(150, dt=5e-4, dtype=torch.float32)
    [eqn] = esr.compile([eqn], "cuda", precision=precision)
    eng = eqn.easier_fused_engine
    assert eng.tiled
    s0 = eng.state.clone()
    eng.step(5)
    torch.cuda.synchronize()
    want = eng.state[:, :3].cpu()
    for chunks in (1, 3, 8):
        eng.state.copy_(s0)
        host = torch.empty((eng.nc, 3), dtype=torch.float32, pin_memory=True)
        host.copy_(s0[:, :3].cpu())
        eng.step_host(host, 5, chunks=chunks)
        assert torch.equal(host, want), chunks
        assert torch.equal(eng.state[:, :3].cpu(), want)
        h = torch.empty_like(want[:, 0])
        h[eng.order.cpu()] = want[:, 0]
        assert torch.equal(eqn.h.collect().cpu(), h)
    with pytest.raises(ValueError):
        eng.step_host(torch.zeros((eng.nc, 4)), 1)
