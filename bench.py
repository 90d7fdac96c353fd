"""Benchmark of the GB300 sparse-mesh path; prints one JSON line.

Workloads (``--workload``):
  swe      shallow water on the tutorial mesh, N=2000 (16,000,000 cells,
           47,992,000 directed edges), centred Gaussian bump, dt=2.5e-4 (5e-4
           is unstable at this resolution); one bench step = one time step
           (one temporally blocked kernel for FP32); metric cell-steps/s.
           Default dtype f32, ``--precision fast`` (FMA, reciprocal per face;
           within 1e-5 of the reference) or ``exact`` (bitwise the reference);
           the other arithmetic and FP64 are reported under ``secondary``.
  poisson  P1 Poisson, 1000x1000 grid (998,001 unknowns, 5,980,016 directed
           couplings), random-mode RHS, Jacobi-PCG to relative residual 1e-8;
           one bench step = one solve; metric solves/s
           (``--precision native|mixed|df64``).
  poisson-fv  the tutorial's cell-centred FV Poisson (tutorial/poisson) on
           the tutorial mesh, N=500 (1,000,000 cells, 2,998,000 directed
           edges), CG without a preconditioner as the tutorial runs it, to
           relative residual 1e-8; metric solves/s.
  batched  256 P1 Poisson instances, side N ~ U{32..512} (seeded), GRF
           kappa, random-mode RHS, packed block-diagonal, lockstep
           Jacobi-PCG per instance to FP64-verified relative residual 1e-8;
           one bench step = one batch solve; metric solves/s
           (``--precision df64|fp64``).

``--impl reference`` times the oracle (the reference's CPU algorithm, the
same aten ops its CPU backend runs) on this machine's host cores, on a
bounded sample of the same workload.  Under torchrun (N>1) every rank runs
an independent replica (the path does not shard at world size 1); the
printed value is all ranks' work over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402
import torch  # noqa: E402


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _barrier(world):
    if world > 1:
        torch.distributed.barrier()


def _max_over_ranks(world, v: float) -> float:
    if world == 1:
        return v
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------- workload configuration --
# Both arms (ours and --impl reference) print the same config dict for the
# same arguments: it names the workload only, never a result.
def swe_sizes(n):
    """Cells, directed interior edges and wall faces of the tutorial mesh
    (4 triangles per grid square)."""
    return 4 * n * n, 12 * n * n - 4 * n, 4 * n


def swe_config(args, world):
    nc, ne, nbc = swe_sizes(args.n)
    s = 4 if args.dtype == "f32" else 8
    resident = nc * (16 + 3 * 16 + 4) + ne * 4
    return {"workload": f"shallow water, tutorial mesh N={args.n} ({nc} cells, {ne} directed edges), dt={args.dt}",
            "cells": nc, "edges": ne, "dt": args.dt, "dtype": args.dtype, "precision": args.precision,
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (state + geometry ~%.2f GB resident)" % (resident * s / 4 / 1e9)}


def poisson_config(args, world):
    if args.workload == "poisson-fv":
        nc, ne, _ = swe_sizes(args.n)
        return {"workload": f"FV Poisson (the tutorial's), tutorial mesh N={args.n} ({nc} cells, {ne} directed "
                            f"edges), CG without preconditioner to FP64 true rel. residual 1e-8",
                "unknowns": nc, "precision": args.precision, "parallelism": f"replicas x{world}",
                "l2": "working set larger than L2 (matrix + 6 vectors)" if nc >= 1_000_000 else
                      "working set smaller than L2"}
    return {"workload": f"P1 Poisson {args.n}x{args.n} grid, 16 random sine modes (seed 0), Jacobi-PCG to FP64 "
                        f"true rel. residual 1e-8",
            "unknowns": (args.n - 1) ** 2, "precision": args.precision, "parallelism": f"replicas x{world}",
            "l2": "working set larger than L2 (matrix + 6 vectors)"}


def batched_config(args, world):
    from easier_gb300.numeric.batched import p1_sides
    sides = p1_sides(args.count, args.nmin, args.nmax, seed=args.seed)
    what = "GNN-preconditioned flexible CG vs Jacobi-PCG" if args.workload == "gnn" else "Jacobi-PCG"
    return {"workload": f"batched P1 Poisson, {args.count} instances (seed {args.seed}), N ~ U{{{args.nmin}.."
                        f"{args.nmax}}}, GRF kappa (corr. 0.1, var 1), {what} per instance to FP64 true rel. "
                        f"residual 1e-8",
            "instances": args.count, "unknowns": int(((sides - 1) ** 2).sum()), "seed": args.seed,
            "precision": "fp64" if args.workload != "gnn" and args.precision == "fp64" else "df64",
            "parallelism": f"replicas x{world}", "l2": "working set larger than L2 (vectors alone > 1 GB)"}


# ------------------------------------------------------------------ SWE --
def swe_algorithmic_bytes(nc, ne, nbc, s):
    """Bytes of one time step under the per-delta byte model: per delta
    ne*(4+3s) [src idx, sx, sy, alpha] + nc*(3s+s+4+3s) [state, area,
    rowptr, delta] + nbc*(4+2s) [wall idx, bsx, bsy]; per step 4 deltas +
    nc*3s*6 for the stage combination (state, 4 deltas, state out)."""
    b_delta = ne * (4 + 3 * s) + nc * (3 * s + s + 4 + 3 * s) + nbc * (4 + 2 * s)
    return 4 * b_delta + nc * 3 * s * 6


def _time_steps(eng, steps, dev, stream):
    eng.step(2)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    eng.step(steps)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    return e0.elapsed_time(e1)


def swe_secondary(args, eng32, dev, stream):
    """The other arithmetic of the FP32 engine, and the FP64 step (the
    reference's precision) in both arithmetics, on fewer steps."""
    import easier_gb300 as esr
    from easier_gb300 import workloads
    out = {}
    other = "exact" if args.precision == "fast" else "fast"
    keep, keep_kernel = eng32.precision, eng32.tile_kernel
    eng32.set_precision(other)
    eng32.tile_kernel = "auto"  # a kernel chosen for the headline may not take the other arithmetic
    steps = max(20, args.steps // 5)
    ms = _time_steps(eng32, steps, dev, stream)
    b = swe_algorithmic_bytes(eng32.nc, eng32.b["ne"], eng32.b["nbc"], 4)
    out[f"f32_{other}"] = {"value": eng32.nc * steps / (ms / 1e3), "unit": "cell-steps/s", "steps": steps,
                           "ms_per_step": ms / steps, "kernel": "tiled" if eng32.tiled else "staged",
                           "hbm_frac_of_measured": b / (ms / steps / 1e3) / 1e9 / _peaks()[0]}
    eng32.set_precision(keep)
    eng32.tile_kernel = keep_kernel
    if args.no_f64:
        return out
    eqn = workloads.make_swe(args.n, dt=args.dt, dtype=torch.float64)
    [eqn] = esr.compile([eqn], "cuda", precision="exact")
    eng = eqn.easier_fused_engine
    b = swe_algorithmic_bytes(eng.nc, eng.b["ne"], eng.b["nbc"], 8)
    for prec in ("exact", "fast"):
        eng.set_precision(prec)
        steps = max(10, args.steps // 50)
        ms = _time_steps(eng, steps, dev, stream)
        out[f"f64_{prec}"] = {"value": eng.nc * steps / (ms / 1e3), "unit": "cell-steps/s", "steps": steps,
                              "ms_per_step": ms / steps, "finite": bool(torch.isfinite(eng.state).all()),
                              "hbm_frac_of_measured": b / (ms / steps / 1e3) / 1e9 / _peaks()[0],
                              "bound": "fp64 pipe (GB300 FP64 rate is 1/59 of FP32)"}
    del eqn, eng
    torch.cuda.empty_cache()
    # the module's own forward on the per-op path (compile(fuse=False)): the
    # reference's op sequence with its Selector/Reducer calls on the gather /
    # segmented-reduce kernels and the elementwise glue in torch
    eqn = workloads.make_swe(args.n, dt=args.dt, dtype=torch.float64)
    [eqn] = esr.compile([eqn], "cuda", fuse=False)
    steps = 3
    eqn()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        eqn()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    out["f64_per_op"] = {"value": eqn.nc * steps / (ms / 1e3), "unit": "cell-steps/s", "steps": steps,
                         "ms_per_step": ms / steps, "path": "module forward, one kernel per op"}
    del eqn
    torch.cuda.empty_cache()
    return out


def swe_cpu_baseline(n, dtype, dt, steps):
    """Oracle SWE step on the host cores; returns (cell-steps/s, threads)."""
    from easier_gb300 import mesh
    from oracle import swe as oswe
    m = mesh.triangular_mesh(n)
    g = mesh.swe_geometry(m)
    p = oswe.SweProblem(m.src, m.dst, m.bcells, g.sx, g.sy, g.alpha, g.bsx, g.bsy, g.area, dt, dtype)
    h = torch.from_numpy(mesh.gaussian_bump(g.x, g.y)).to(dtype)
    uh = torch.zeros_like(h)
    vh = torch.zeros_like(h)
    t0 = time.perf_counter()
    for _ in range(steps):
        h, uh, vh = p.step(h, uh, vh)
    wall = time.perf_counter() - t0
    return m.nc * steps / wall, torch.get_num_threads(), wall


def bench_swe(args, world, rank, local):
    import ctypes

    import easier_gb300 as esr
    from easier_gb300 import _lib, workloads
    dtype = torch.float32 if args.dtype == "f32" else torch.float64
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    # one small compile first, untimed in the N=2000 figures: the first use
    # of each torch kernel on a fresh machine is compiled for this GPU by
    # the CUDA driver and cached for later processes (measured: the N=2000
    # compile takes ~25 s in a fresh machine's first process, 1.7 s after)
    t0 = time.perf_counter()
    small = workloads.make_swe(256, dt=args.dt, dtype=dtype, device=dev)  # 262,144 cells: large-array paths
    [small] = esr.compile([small], "cuda", precision=args.precision)
    torch.cuda.synchronize(dev)
    t_first = time.perf_counter() - t0
    del small
    t_setup = time.perf_counter()
    # mesh and geometry generated on the GPU (bitwise the host generator's)
    eqn = workloads.make_swe(args.n, dt=args.dt, dtype=dtype, device=dev)
    torch.cuda.synchronize(dev)
    t_mesh = time.perf_counter() - t_setup
    if args.tile_cells:
        from easier_gb300 import swe
        swe.DEFAULT_TILE_CELLS = args.tile_cells
    t0 = time.perf_counter()
    [eqn] = esr.compile([eqn], "cuda", precision=args.precision)
    t_compile = time.perf_counter() - t0
    eng = eqn.easier_fused_engine
    if eng is None:
        raise RuntimeError("the fused shallow-water engine was not installed")
    if args.tile_kernel:  # this engine only (the exact-arithmetic figures keep theirs)
        eng.tile_kernel = args.tile_kernel
    nc = eng.nc
    stream = torch.cuda.current_stream(dev)
    eng.step(args.warmup)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        _barrier(world)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        eng.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        _barrier(world)
    ms = e0.elapsed_time(e1)
    ms_max = _max_over_ranks(world, ms)
    h = eqn.h.collect()
    if not bool(torch.isfinite(h).all()):
        raise RuntimeError("non-finite shallow-water state after the timed steps")
    value = world * nc * args.steps / (ms_max / 1e3)
    bytes_step = swe_algorithmic_bytes(nc, eng.b["ne"], eng.b["nbc"], 4 if dtype == torch.float32 else 8)
    touched = eng.touched_bytes_per_step()
    lps = eng.launches_per_step()
    peak, peak_kind = _peaks()
    achieved = bytes_step / (ms / args.steps / 1e3) / 1e9
    secondary = swe_secondary(args, eng, dev, stream) if args.dtype == "f32" else {}

    # end to end with the state in host memory: every step uploads the state
    # (h, uh, vh per cell: 12 bytes, the 4th lane of the device layout is
    # padding) from pinned host memory, runs one step and reads it back --
    # through esr_swe_host_step (the tiled layout: chunked copies, the link
    # used both ways), else the plain C-ABI step between two copies
    host = torch.empty((nc, 3), dtype=dtype, pin_memory=True)
    host.copy_(eng.state[:, :3])
    ke = max(1, min(args.steps, args.e2e_steps))
    if eng.tiled:
        eng.step_host(host, 1, chunks=args.host_chunks)  # plan set up outside the timed region
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    e0.record(stream)
    if eng.tiled:
        eng.step_host(host, ke, chunks=args.host_chunks)
        path = (f"SweEngine.step_host -> esr_swe_host_step ({args.host_chunks} chunks a step; uploads, downloads "
                "and the step's tile groups overlapped)")
    else:
        stage = torch.empty((nc, 3), dtype=dtype, device=dev)
        a = eng.bufs[0]
        for _ in range(ke):
            stage.copy_(host, non_blocking=True)
            a[:, :3].copy_(stage)
            _lib.call("esr_swe_step", ctypes.byref(eng._mesh), float(args.dt), _lib.ptr(a), 1,
                      _lib.ptr(eng.ws), stream.cuda_stream)
            stage.copy_(a[:, :3])
            host.copy_(stage, non_blocking=True)
        path = "esr_swe_step via ctypes between copies of the state from/to pinned host memory"
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = e0.elapsed_time(e1)
    e2e_wall = time.perf_counter() - t0
    e2e_ms = _max_over_ranks(world, max(e2e_ms, e2e_wall * 1e3))
    e2e = {"value": world * nc * ke / (e2e_ms / 1e3), "unit": "cell-steps/s",
           "h2d_bytes_per_step": host.numel() * host.element_size(),
           "d2h_bytes_per_step": host.numel() * host.element_size(), "steps": ke, "path": path}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, thr, wall = swe_cpu_baseline(args.n, dtype, args.dt, args.cpu_steps)
        cpu = {"value": v, "unit": "cell-steps/s", "cores": thr, "kind": "port",
               "sample": f"{args.cpu_steps} oracle steps (torch CPU ops, reference op order) at N={args.n}, "
                         f"{args.dtype}, {wall:.1f} s"}
    traffic = _ncu_traffic(eng.traffic_key() if eng.tiled else "swe", args)
    step_s = ms / args.steps / 1e3
    kernel_bytes = touched / lps  # what one launch of the fused kernel must move, each array once
    line = {
        "metric": "SWE cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
        "data": "synthetic (tutorial mesh generator, centred Gaussian bump, uh=vh=0)",
        "config": swe_config(args, world),
        "roofline": {"bound": "hbm", "achieved": kernel_bytes / (step_s / lps) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": kernel_bytes / (step_s / lps) / 1e9 / peak, "peak_kind": peak_kind,
                     "traffic": traffic,
                     "kernel": ((("swe_tile_pipe_kernel" if eng.tile_kernel_name().startswith("pipelined") else
                                  "swe_tile_step_kernel") + " (1 launch per step)") if eng.tiled else
                                "swe_stage_kernel (4 launches per step; bytes and time per step / 4)"),
                     "algorithmic_bytes_per_launch": kernel_bytes,
                     "bytes_model": eng.bytes_model(),
                     "dram_frac": (traffic / (step_s / lps) / 1e9 / peak) if traffic else None,
                     "contract_model_bytes_per_step": bytes_step,
                     "contract_model_frac": achieved / peak,
                     "contract_model": "the unfused step's bytes (four delta passes and the stage combination "
                                       "through HBM): not what the fused kernel moves, so not an HBM fraction"},
        "engine": eng.describe(),
        "setup_s": {"mesh_geometry_and_module": t_mesh,
                    "engine_phases": {k: round(v, 4) for k, v in getattr(eng, "setup_phases").times.items()},
                    "compile": t_compile,
                    "first_small_compile": t_first,
                    "compile_note": "N=2000: tiled layout built on the GPU (BFS-bisection partition kernels, "
                                    "device sorts for slots and halo rings) and the compile-time check of one "
                                    "fused step against the module's own forward; after one N=256 mesh and "
                                    "compile (first_small_compile), which pays the first use of every kernel in "
                                    "the process -- on a fresh machine the CUDA driver compiles torch's kernels "
                                    "for this GPU then, once per machine"},
        "parity": ("bitwise equal to the reference CPU backend" if args.precision == "exact" else
                   "state within 1e-5 (FP32) relative max-norm of the FP64 oracle (N=100 x 1,000 steps, N=2000 x 5 "
                   "steps)"),
        "secondary": secondary,
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": lps * args.steps, "clocks": clk.summary(),
    }
    if not args.no_solvers:
        eng._free_host_plan()
        del eqn, eng, host
        torch.cuda.empty_cache()
        line["secondary"]["solvers"] = solver_secondaries(args, world, rank, local)
    return line


def _ncu_traffic(kind, args):
    """DRAM bytes per launch of this kernel variant on this mesh (ncu
    dram__bytes_read.sum + dram__bytes_write.sum of one launch), from the
    committed profile summary, if there is one."""
    f = ROOT / "profiles" / "traffic.json"
    if not f.exists():
        return None
    d = json.loads(f.read_text())
    return d.get(f"{kind}_{args.dtype}_n{args.n}")


# -------------------------------------------------------------- Poisson --
def bench_poisson(args, world, rank, local):
    import easier_gb300 as esr
    from easier_gb300 import workloads
    from easier_gb300.numeric.preconditioner import Jacobi
    from easier_gb300.numeric.solver import CG
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    fv = args.workload == "poisson-fv"
    if fv:  # the tutorial's FV Poisson and its solver call: CG without a preconditioner
        eqn = workloads.make_poisson_fv(args.n)
        sol = CG(eqn.A, eqn.b, eqn.x)
    else:
        eqn = workloads.P1Poisson(args.n, rhs_seed=0)
        sol = CG(eqn.A, eqn.b, eqn.x, M=Jacobi(eqn.A))
    [eqn, sol] = esr.compile([eqn, sol], "cuda")
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        eqn.x.data.zero_()
        sol.solve(rtol=1e-8, precision=args.precision)
    torch.cuda.synchronize(dev)
    iters = []
    launches0 = getattr(sol._fused, "kernel_launches", 0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        _barrier(world)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for _ in range(args.steps):
            eqn.x.data.zero_()
            info = sol.solve(rtol=1e-8, precision=args.precision)
            iters.append(info["iters"])
        e1.record(stream)
        torch.cuda.synchronize(dev)
        _barrier(world)
    ms = _max_over_ranks(world, e0.elapsed_time(e1))
    bnorm = float(torch.linalg.vector_norm(eqn.b.data))
    rel = info["true_residual"] / bnorm
    if not rel <= 1e-8 * 1.0001:
        raise RuntimeError(f"true relative residual {rel:.3e} above 1e-8")
    nit = statistics.mean(iters)
    eng = sol._fused
    if hasattr(eng, "bytes_per_iteration"):
        bytes_it = eng.bytes_per_iteration()
    else:
        bytes_it = eng.bytes_per_row_iteration() * eng.pack.n
    achieved = bytes_it * nit / (ms / args.steps / 1e3) / 1e9
    dtype = {"native": "f64", "mixed": "f32-spmv/f64-dot", "df64": "df64 (f32 pairs)"}[args.precision]
    peak, peak_kind = _peaks()
    line = {
        "metric": "Poisson solves/s", "value": world * args.steps / (ms / 1e3), "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": dtype,
        "data": ("tutorial FV Poisson right hand side (Gaussian source)" if fv else
                 "synthetic (16 random sine modes, seed 0)"),
        "config": poisson_config(args, world),
        "solve": {"couplings": int(eqn.selector.idx.numel()), "iterations": nit, "bytes_per_iteration": bytes_it,
                  "replacements": info.get("restarts", info.get("replacements")), "true_rel_residual": rel},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None,
                     "bytes_model": "per iteration: SpMV col + value per stored slot and the diagonal, 14 vector "
                                    "touches of 8 bytes per row (x iterations of the solve)"},
        "gpu_launches": int(getattr(eng, "kernel_launches", 0) - launches0),
        "clocks": clk.summary(),
    }
    # end to end through the public API: b from pinned host memory into the
    # module's tensor, solve, x back to pinned host memory, every step
    b_host = eqn.b.data.cpu().pin_memory()
    x_host = torch.empty_like(b_host).pin_memory()
    k_e2e = max(1, min(args.steps, 3))
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(k_e2e):
        eqn.b.data.copy_(b_host, non_blocking=True)
        eqn.x.data.zero_()
        sol.solve(rtol=1e-8, precision=args.precision)
        x_host.copy_(eqn.x.data, non_blocking=True)
    torch.cuda.synchronize(dev)
    e2e_s = (time.perf_counter() - t0) / k_e2e
    nb = b_host.numel() * b_host.element_size()
    line["e2e"] = {"value": world / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb,
                   "path": "CG.solve on the compiled module, b in and x out through pinned host memory"}
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import cg as ocg
        row, col, Ae, Av, bb = _poisson_arrays(args, eqn)
        k = 40
        t0 = time.perf_counter()
        ocg.cg(row, col, Ae, Av, bb, rtol=0.0, maxiter=k - 1, jacobi=not fv)
        per_it = (time.perf_counter() - t0) / k
        what = f"FV Poisson N={args.n} CG" if fv else f"{args.n}x{args.n} P1 Jacobi-PCG"
        line["cpu_baseline"] = {"value": 1.0 / (per_it * (nit + 1)), "unit": "solves/s",
                                "cores": torch.get_num_threads(), "kind": "port",
                                "sample": f"{k} oracle iterations of the {what} system "
                                          f"({per_it * 1e3:.1f} ms each), scaled to the {nit:.0f} iterations of a "
                                          f"solve"}
    return line


def _poisson_arrays(args, eqn):
    """(row, col, Ae, Av, b) of the workload's system for the oracle (host
    numpy, the generators' order)."""
    from easier_gb300 import mesh
    if args.workload == "poisson-fv":
        m = mesh.triangular_mesh(args.n)
        a = mesh.poisson_fv(m)
        return m.src, m.dst, a.Af, a.Ac, a.b
    s = mesh.p1_system(args.n)
    return s.row, s.col, s.Ae, s.Av, mesh.random_mode_rhs(args.n, 0)


# -------------------------------------------------------- batched Poisson --
def batched_cpu_baseline(insts, iters, budget_s=20.0, count=16):
    """Oracle Jacobi-PCG on a seeded subset of the instances, each run for a
    bounded number of iterations; the per-(unknown x iteration) cost is
    scaled by every instance's iteration count from the GPU run."""
    from oracle import cg as ocg
    rng = np.random.default_rng(0)
    pick = rng.choice(len(insts), size=min(count, len(insts)), replace=False)
    work, wall = 0.0, 0.0
    per = max(1.0, budget_s / len(pick))
    for i in pick:
        s = insts[i]
        k = 10
        while True:
            t0 = time.perf_counter()
            ocg.cg(s.row, s.col, s.Ae, s.Av, s.b, rtol=0.0, maxiter=k - 1, jacobi=True)
            dt = time.perf_counter() - t0
            if dt >= 0.25 * per or k >= iters[i] + 1:
                break
            k *= 4
        work += k * s.n
        wall += dt
    cost = wall / work
    total = sum((it + 1) * s.n for it, s in zip(iters, insts)) * cost
    sizes = sorted(int(round(np.sqrt(insts[i].n))) + 1 for i in pick)
    return len(insts) / total, (f"oracle Jacobi-PCG on {len(pick)} seeded instances (N={sizes}), bounded iterations, "
                                f"{cost * 1e9:.2f} ns per unknown-iteration scaled by the {len(insts)} instances' "
                                f"iteration counts")


def bench_batched(args, world, rank, local):
    from easier_gb300.numeric.batched import BatchedPCG, p1_instances
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    prec = "fp64" if args.precision == "fp64" else "df64"
    t0 = time.perf_counter()
    insts = p1_instances(args.count, args.nmin, args.nmax, seed=args.seed)
    eng = BatchedPCG(insts, jacobi=True, precision=prec, device=dev, graph_iters=args.chunk)
    prep = time.perf_counter() - t0
    t0 = time.perf_counter()
    if args.shape:  # a fixed work shape (tiles per chunk, CTAs), e.g. the one autotune picks
        tpc, grid = (int(v) for v in args.shape.split(","))
        eng.set_shape(tpc, grid)
        tuning = None
    else:
        tuning = eng.autotune() if not args.no_autotune else None
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    x_start = torch.zeros_like(eng.b64)
    maxiter = 100000  # bounds the device-side loop of the one-launch graph

    def one_solve():
        # the whole batch solve is ONE CUDA graph launch (init, device-side
        # loop of iteration bodies with FP64 verification)
        if args.polled:
            eng.run(1e-8)
        else:
            eng.solve_graph(1e-8, maxiter=maxiter)

    for _ in range(args.warmup):
        eng.load_packed(x0=x_start)
        one_solve()
    torch.cuda.synchronize(dev)
    launches0 = eng.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        _barrier(world)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for _ in range(args.steps):
            eng.load_packed(x0=x_start)
            one_solve()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        _barrier(world)
    ms = _max_over_ranks(world, e0.elapsed_time(e1))
    res = [eng._info(s) for s in eng.instances()]
    if args.polled:
        launches = eng.kernel_launches - launches0
    else:  # kernels the device-side loop ran: init, then per body compaction, k iterations, verification
        kk = eng.graph_iters
        bodies = -(-(max(r["iters"] for r in res) + 1) // kk)
        per_it = 2 if eng.precision == "df64" else 3
        launches = args.steps * (1 + bodies * (1 + per_it * kk + 4 + 1))
    bad = [i for i, r in enumerate(res) if r["status"] != "converged" or not r["true_residual"] <= 1e-8 * r["bnorm"]
           * 1.0001]
    if bad:
        raise RuntimeError(f"{len(bad)} instances not FP64-verified at rel. residual 1e-8, e.g. {res[bad[0]]}")
    iters = [r["iters"] for r in res]
    pk = eng.pack
    npad = np.diff(pk.inst_block0.astype(np.int64)) * 256
    row_its = float(sum((it + 1 + r["restarts"]) * n for it, r, n in zip(iters, res, npad)))
    bytes_solve = row_its * eng.bytes_per_row_iteration()
    sec = ms / args.steps / 1e3
    achieved = bytes_solve / sec / 1e9
    peak, peak_kind = _peaks()
    # end to end: packed right hand sides from pinned host memory in, FP64
    # solutions back to pinned host memory, every step
    b_host = eng.b64.cpu().pin_memory()
    x_host = torch.empty(pk.n, dtype=torch.float64).pin_memory()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        eng.load_packed(b64=b_host.to(dev, non_blocking=True), x0=x_start)
        one_solve()
        x_host.copy_(eng.solution(), non_blocking=True)
    torch.cuda.synchronize(dev)
    e2e_sec = (time.perf_counter() - t0) / e2e_steps
    line = {
        "metric": "Poisson solves/s (batched)", "value": world * pk.ninst / sec, "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == "fp64" else "df64 (f32 pairs)",
        "data": f"synthetic (seed {args.seed}: GRF kappa corr. 0.1 var 1, 16 random sine modes)",
        "config": batched_config(args, world),
        "solve": {"packed_rows": pk.n, "stored_slots": int(pk.slice_ptr[-1]),
                  "iterations_max": max(iters), "iterations_mean": float(np.mean(iters)),
                  "restarts": int(sum(r["restarts"] for r in res)),
                  "graph_iters": eng.graph_iters, "tiles_per_chunk": eng.tiles_per_chunk, "grid": eng.grid,
                  "launch": ("host-polled CUDA graphs of graph_iters iterations" if args.polled else
                             "one CUDA graph launch per batch solve (device-side while loop)"),
                  "autotune": None if tuning is None else
                  {"s": tune_s, "ms_per_iter_all_running": tuning["ms_per_iter"],
                   "candidates": len(tuning["table"])},
                  "setup_s": prep},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None,
                     "bytes_per_row_iteration": eng.bytes_per_row_iteration()},
        "e2e": {"value": world * pk.ninst / e2e_sec, "unit": "solves/s", "h2d_bytes_per_step": pk.n * 8,
                "d2h_bytes_per_step": pk.n * 8},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        v, sample = batched_cpu_baseline(insts, iters)
        line["cpu_baseline"] = {"value": v, "unit": "solves/s", "cores": torch.get_num_threads(), "kind": "port",
                                "sample": sample}
    return line


# ---------------------------------------------------- GNN-preconditioned --
def gnn_row_bytes(slots_per_row: float) -> float:
    """Algorithmic bytes of one GNN application per packed row: 4 layers
    each reading and writing the row's 32 BF16 features (64 + 64 bytes) and
    each stored slot's column index and edge inputs (4 + 8 bytes), plus the
    residual, kappa input and output (20 bytes)."""
    return 4 * (128 + 12 * slots_per_row) + 20


POLY_DEGREE = 4  # the polynomial-Jacobi control of the GNN line


def bench_gnn(args, world, rank, local):
    """Flexible CG with the GNN preconditioner against Jacobi-PCG and
    against a degree-4 polynomial-Jacobi PCG (five damped Jacobi sweeps per
    application, four of them SpMVs), all batched and df64, on held-out
    seeded instances."""
    from easier_gb300.numeric.batched import BatchedPCG, POLY_OMEGA, p1_instances
    from easier_gb300.numeric.preconditioner.gnn import GnnWeights, WEIGHTS_FILE
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    insts = p1_instances(args.count, args.nmin, args.nmax, seed=args.seed)
    stream = torch.cuda.current_stream(dev)
    out = {}
    for name, kw in (("jacobi", {}), ("poly_jacobi", {"poly_degree": POLY_DEGREE}),
                     ("gnn", {"gnn": GnnWeights.load()})):
        eng = BatchedPCG(insts, jacobi=True, precision="df64", device=dev, graph_iters=args.chunk, **kw)
        eng.autotune()
        x0 = torch.zeros_like(eng.b64)
        for _ in range(args.warmup):
            eng.load_packed(x0=x0)
            eng.run(1e-8)
        torch.cuda.synchronize(dev)
        l0 = eng.kernel_launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            _barrier(world)
            torch.cuda.synchronize(dev)
            e0.record(stream)
            for _ in range(args.steps):
                eng.load_packed(x0=x0)
                eng.run(1e-8)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            _barrier(world)
        ms = _max_over_ranks(world, e0.elapsed_time(e1))
        res = [eng._info(s) for s in eng.instances()]
        bad = [r for r in res if r["status"] != "converged" or not r["true_residual"] <= 1e-8 * r["bnorm"] * 1.0001]
        if bad:
            raise RuntimeError(f"{name}: {len(bad)} instances not FP64-verified at 1e-8, e.g. {bad[0]}")
        its = np.array([r["iters"] for r in res])
        # algorithmic bytes: the CG iterations (engine byte model per packed
        # row) plus, per GNN application, GNN_ROW_BYTES per packed row
        npad = np.diff(eng.pack.inst_block0.astype(np.int64)) * 256
        slots = eng.pack.slice_ptr[-1] / eng.pack.n
        cg_bytes = float(sum((r["iters"] + 1 + r["restarts"]) * n for r, n in zip(res, npad)))
        cg_bytes *= eng.bytes_per_row_iteration()
        gnn_apps = float(sum(r["fallback_iter"] * n for r, n in zip(res, npad))) if name == "gnn" else 0.0
        gnn_bytes = gnn_apps * gnn_row_bytes(slots)
        sec = ms / args.steps / 1e3
        out[name] = {"solves_per_s": world * len(insts) / sec, "ms_per_batch": ms / args.steps,
                     "bytes_per_solve_batch": cg_bytes + gnn_bytes,
                     "achieved_gbs": (cg_bytes + gnn_bytes) / sec / 1e9,
                     "iters_mean": float(its.mean()), "iters_max": int(its.max()),
                     "fallbacks": int(sum(r["fallbacks"] for r in res)),
                     "theta_clips": int(sum(r["clips"] for r in res)),
                     "launches": eng.kernel_launches - l0, "clocks": clk.summary()}
        del eng
        torch.cuda.empty_cache()
    g, j, pj = out["gnn"], out["jacobi"], out["poly_jacobi"]
    pj["degree"], pj["omega"] = POLY_DEGREE, POLY_OMEGA
    peak, peak_kind = _peaks()
    return {
        "metric": "Poisson solves/s (batched, GNN-preconditioned flexible CG)", "value": g["solves_per_s"],
        "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": g["ms_per_batch"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "df64 (f32 pairs) CG, bf16 GNN with f32 accumulation",
        "data": f"synthetic held-out instances (seed {args.seed}); weights {WEIGHTS_FILE.name}",
        "config": batched_config(args, world),
        "solve": {"gnn": {k: v for k, v in g.items() if k != "clocks"},
                  "jacobi": {k: v for k, v in j.items() if k != "clocks"},
                  "poly_jacobi": {k: v for k, v in pj.items() if k != "clocks"},
                  "gnn_over_jacobi_solves_per_s": g["solves_per_s"] / j["solves_per_s"],
                  "gnn_over_poly_jacobi_solves_per_s": g["solves_per_s"] / pj["solves_per_s"]},
        "roofline": {"bound": "hbm", "achieved": g["achieved_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": g["achieved_gbs"] / peak, "peak_kind": peak_kind, "traffic": None,
                     "bytes_model": "df64 CG bytes per packed row-iteration (engine model) plus, per GNN "
                                    "application, 4 layers x (BF16 features in and out, 64 + 64 bytes, and 12 "
                                    "bytes per stored slot) + 20 bytes of inputs and output per packed row"},
        "gpu_launches": g["launches"],
        "clocks": g["clocks"],
    }


# ------------------------------------------- solver figures beside SWE --
def solver_secondaries(args, world, rank, local):
    """The solver workloads, each bounded, on the default SWE line:
    P1-1000 Jacobi-PCG in FP64 and double-float (3 timed solves each), the
    tutorial's FV Poisson at N=500 with its CG (3 timed solves), the
    256-instance batch in double-float (one timed one-launch batch solve)
    and GNN flexible CG against Jacobi-PCG and polynomial-Jacobi PCG on the
    held-out batch (one timed batch each).  Each keeps its own CUDA-event
    timing, FP64-verified residuals, roofline and clock record."""
    import copy
    out = {}
    runs = (("poisson_p1_1000_fp64", bench_poisson, dict(workload="poisson", n=1000, precision="native", steps=3,
                                                          warmup=1, seed=0)),
            ("poisson_p1_1000_df64", bench_poisson, dict(workload="poisson", n=1000, precision="df64", steps=3,
                                                          warmup=1, seed=0)),
            ("poisson_fv_500_fp64", bench_poisson, dict(workload="poisson-fv", n=500, precision="native", steps=3,
                                                         warmup=1, seed=0)),
            ("batched_256_df64", bench_batched, dict(workload="batched", precision="df64", steps=1, warmup=1,
                                                      seed=0)),
            ("gnn_vs_jacobi_256_heldout", bench_gnn, dict(workload="gnn", precision="df64", steps=1, warmup=1,
                                                          seed=1)))
    for name, fn, over in runs:
        a = copy.copy(args)
        for k, v in over.items():
            setattr(a, k, v)
        # CPU baselines only where a bounded sample costs seconds (the
        # single-system solves: 40 oracle iterations)
        a.no_cpu_baseline = args.no_cpu_baseline or fn is not bench_poisson
        t0 = time.perf_counter()
        line = fn(a, world, rank, local)
        keep = {k: line[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "dtype", "config", "solve",
                                     "roofline", "e2e", "gpu_launches", "clocks", "cpu_baseline") if k in line}
        keep["wall_s"] = time.perf_counter() - t0
        out[name] = keep
        torch.cuda.empty_cache()
    return out


# ------------------------------------------------------------ reference --
REF_BUDGET_S = 120.0  # timed work of the reference arm: it ends within a few minutes at any --steps


def _bounded(step, steps, budget_s=REF_BUDGET_S):
    """Runs step(k) for k < steps, stopping once budget_s has passed (after
    at least one); returns (steps run, wall seconds)."""
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        step(done)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return done, time.perf_counter() - t0


def bench_reference(args, world):
    """The reference's CPU algorithm (oracle: the aten ops its CPU backend
    runs, in its order) on the host cores, with inputs built by the oracle's
    own mesh, geometry and assembly restatements (nothing of this package's
    native library runs here): each step one full step / solve of the
    workload, as many of the requested steps as fit REF_BUDGET_S (at most
    one warm-up step).  The config dict is the one our arm prints."""
    from oracle import cg as ocg
    from oracle import mesh as omesh
    torch.set_num_threads(os.cpu_count() or 1)
    requested = args.steps
    args.warmup = min(args.warmup, 1)
    t_setup = time.perf_counter()
    if args.workload == "swe":
        from oracle import swe as oswe
        dtype = torch.float32 if args.dtype == "f32" else torch.float64
        m = omesh.triangular_mesh(args.n)
        g = omesh.swe_geometry(m)
        p = oswe.SweProblem(m["src"], m["dst"], m["bcells"], g["sx"], g["sy"], g["alpha"], g["bsx"], g["bsy"],
                            g["area"], args.dt, dtype)
        x, y = np.asarray(g["x"]), np.asarray(g["y"])
        h = torch.from_numpy(1 + 0.1 * np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.01)).to(dtype)
        st = [h, torch.zeros_like(h), torch.zeros_like(h)]
        nc = int(h.shape[0])

        def one(_):
            st[:] = p.step(*st)
        setup = time.perf_counter() - t_setup
        for _ in range(args.warmup):
            one(0)
        args.steps, wall = _bounded(one, requested)
        v = nc * args.steps / wall
        unit, metric = "cell-steps/s", "SWE cell-steps/s"
        sample = f"{args.steps} full oracle steps at N={args.n} ({nc} cells), {args.dtype}"
        cfg = swe_config(args, world)
        eager = _swe_eager_gpu(m, g, h, args, dtype) if torch.cuda.is_available() else None
    elif args.workload in ("batched", "gnn"):
        from easier_gb300 import mesh as gen  # numpy generators of the seeded fields and right hand sides
        from easier_gb300.numeric.batched import p1_sides
        sides = p1_sides(args.count, args.nmin, args.nmax, seed=args.seed)
        order = np.random.default_rng(0).permutation(len(sides))
        cache = {}

        def instance(i):
            if i not in cache:
                n = int(sides[i])
                kappa = gen.kappa_from_field(gen.gaussian_random_field(n, args.seed * 100_003 + 2 * i))
                row, col, Ae, Av = omesh.p1_arrays(n, kappa)
                b = gen.random_mode_rhs(n, args.seed * 100_003 + 2 * i + 1)
                cache[i] = (row, col, Ae, Av, b, n)
            return cache[i]
        setup = time.perf_counter() - t_setup
        for i in order[:args.warmup]:
            row, col, Ae, Av, b, _ = instance(i)
            ocg.cg(row, col, Ae, Av, b, rtol=1e-8, jacobi=True)
        sizes = []
        timed = order[args.warmup:]
        build_s = [0.0]

        def one(k):
            t0 = time.perf_counter()
            row, col, Ae, Av, b, n = instance(timed[k % len(timed)])
            build_s[0] += time.perf_counter() - t0
            ocg.cg(row, col, Ae, Av, b, rtol=1e-8, jacobi=True)
            sizes.append(n)
        args.steps, wall = _bounded(one, requested)
        wall -= build_s[0]
        v = args.steps / wall
        unit, metric = "solves/s", "Poisson solves/s (batched)"
        sample = (f"{args.steps} full Jacobi-PCG solves of seeded instances drawn from the batch "
                  f"(N={sizes}), one per step (instance assembly not timed)")
        cfg = batched_config(args, world)
    else:
        fv = args.workload == "poisson-fv"
        if fv:  # the tutorial's FV Poisson, CG without a preconditioner as the tutorial runs it
            m = omesh.triangular_mesh(args.n)
            a = omesh.poisson_fv(m)
            row, col, Ae, Av, b = m["src"], m["dst"], a["Af"], a["Ac"], a["b"]
        else:
            from easier_gb300 import mesh as gen
            row, col, Ae, Av = omesh.p1_arrays(args.n)
            b = gen.random_mode_rhs(args.n, 0)
        setup = time.perf_counter() - t_setup
        for _ in range(args.warmup):
            ocg.cg(row, col, Ae, Av, b, rtol=1e-8, jacobi=not fv)
        its = []

        def one(_):
            its.append(ocg.cg(row, col, Ae, Av, b, rtol=1e-8, jacobi=not fv)[1])
        args.steps, wall = _bounded(one, requested)
        v = args.steps / wall
        unit, metric = "solves/s", "Poisson solves/s"
        sample = (f"{args.steps} full CG solves ({its[-1]} iterations each) of the FV Poisson at N={args.n}" if fv else
                  f"{args.steps} full Jacobi-PCG solves ({its[-1]} iterations each) on the {args.n}x{args.n} P1 grid")
        cfg = poisson_config(args, world)
    cores = torch.get_num_threads()
    if args.steps < requested:
        sample += f"; {args.steps} of the {requested} requested steps fit the {REF_BUDGET_S:.0f} s budget"
    sample += f"; oracle input set-up {setup:.1f} s (not timed)"
    line = {"impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.dtype if args.workload == "swe" else "f64",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": v, "unit": unit, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.workload == "swe" and eager is not None:
        line["reference_eager_gpu"] = eager
    return line


def _swe_eager_gpu(m, g, h, args, dtype, steps=10):
    """The second baseline: the reference's SWE op sequence (aten index
    gathers, scatter_reduce_ with atomics, elementwise ops) as eager torch
    kernels on this GPU -- what its backend='cuda' runs, without its
    JitEngine interpreter -- timed with CUDA events."""
    from oracle import swe as oswe
    dev = torch.device("cuda", 0)
    p = oswe.SweProblem(m["src"], m["dst"], m["bcells"], g["sx"], g["sy"], g["alpha"], g["bsx"], g["bsy"],
                        g["area"], args.dt, dtype, device=dev)
    st = [h.to(dev), torch.zeros_like(h, device=dev), torch.zeros_like(h, device=dev)]
    st[:] = p.step(*st)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        st[:] = p.step(*st)
    e1.record()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    nc = int(h.shape[0])
    out = {"value": nc / (ms / 1e3), "unit": "cell-steps/s", "ms_per_step": ms, "steps": steps,
           "path": "reference op sequence as eager torch on the GPU (aten index + scatter_reduce_ with atomics; "
                   "the reference's backend='cuda' without its interpreter)"}
    del p, st
    torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=None)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["swe", "poisson", "poisson-fv", "batched", "gnn"], default="swe")
    ap.add_argument("--count", type=int, default=256, help="batched: instances")
    ap.add_argument("--nmin", type=int, default=32, help="batched: smallest mesh side")
    ap.add_argument("--nmax", type=int, default=512, help="batched: largest mesh side")
    ap.add_argument("--seed", type=int, default=None, help="batched: instance seed (gnn: held-out seed 1)")
    ap.add_argument("--chunk", type=int, default=32, help="batched: iterations per CUDA graph")
    ap.add_argument("--no-autotune", action="store_true", help="batched: keep the default work shape")
    ap.add_argument("--polled", action="store_true", help="batched: host-polled graphs instead of one launch")
    ap.add_argument("--shape", default=None, help="batched: fixed work shape TILES_PER_CHUNK,CTAS (no autotune)")
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--dtype", choices=["f32", "f64"], default="f32")
    ap.add_argument("--dt", type=float, default=None)
    ap.add_argument("--precision", choices=["native", "mixed", "df64", "fp64", "exact", "fast"], default=None)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-f64", action="store_true")
    ap.add_argument("--no-solvers", action="store_true", help="swe: leave out the solver figures")
    ap.add_argument("--tile-cells", type=int, default=None, help="swe: target cells per tile (FP32 tiled step)")
    ap.add_argument("--host-chunks", type=int, default=None, help="swe: pieces of the end-to-end state copies")
    ap.add_argument("--tile-kernel", default=None,
                    choices=["auto", "blocked", "pipelined", "pipelined_512", "pipelined_768"],
                    help="swe: tile kernel of the FP32 tiled step")
    args = ap.parse_args()
    if args.n is None:
        args.n = {"swe": 2000, "poisson-fv": 500}.get(args.workload, 1000)
    if args.host_chunks is None:
        from easier_gb300 import swe as _swe
        args.host_chunks = _swe.HOST_CHUNKS
    if args.dt is None:
        # dt = 5e-4 at N=2000 exceeds the scheme's stability limit (the state
        # turns non-finite within ~200 steps); 2.5e-4 is stable for 1000+
        # steps.  The per-step cost does not depend on dt.
        args.dt = 5e-4 if args.n <= 1000 else 2.5e-4
    if args.precision is None:
        args.precision = "fast" if args.workload == "swe" else "native"
    if args.seed is None:
        args.seed = 1 if args.workload == "gnn" else 0
    world, rank, local = _dist()
    if args.impl == "reference":
        if args.steps is None:
            args.steps = {"swe": 3, "poisson": 1, "poisson-fv": 2, "batched": 4, "gnn": 4}[args.workload]
        if args.warmup is None:
            args.warmup = {"swe": 1, "poisson": 0, "poisson-fv": 0, "batched": 1, "gnn": 1}[args.workload]
        if rank != 0:
            return
        print(json.dumps(bench_reference(args, world)), flush=True)
        return
    if args.steps is None:
        args.steps = {"swe": 1000, "poisson": 10, "poisson-fv": 10, "batched": 5, "gnn": 3}[args.workload]
    if args.warmup is None:
        args.warmup = 10 if args.workload == "swe" else 3
    if args.warmup < 3:
        args.warmup = 3
    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    run = {"swe": bench_swe, "poisson": bench_poisson, "poisson-fv": bench_poisson, "batched": bench_batched,
           "gnn": bench_gnn}[args.workload]
    line = run(args, world, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
