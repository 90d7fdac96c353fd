"""The oracle against fixtures produced by running the reference itself
(tests/golden/make_golden.py).  Bitwise wherever the reference's CPU run is
deterministic."""
import numpy as np
import pytest
import torch

from oracle import cg as ocg
from oracle import mesh as omesh
from oracle import sparse as osp
from oracle import swe as oswe


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8])
def test_mesh_matches_reference(golden, n):
    g = golden("mesh_small.npz")
    m = omesh.triangular_mesh(n)
    for k in ("src", "dst", "bcells"):
        assert np.array_equal(m[k], g[f"n{n}_{k}"]), k
    assert np.array_equal(m["cells"].reshape(-1), g[f"n{n}_cells"])
    assert np.array_equal(m["bpoints"].reshape(-1), g[f"n{n}_bpoints"])
    assert np.array_equal(m["points"].reshape(-1), g[f"n{n}_points"])


def test_swe_geometry_matches_reference(golden):
    g = golden("swe_geometry_n10.npz")
    geo = omesh.swe_geometry(omesh.triangular_mesh(10))
    for k in ("sx", "sy", "alpha", "area", "x", "y", "bsx", "bsy"):
        assert np.array_equal(geo[k], g[k]), k


def test_poisson_fv_matches_reference(golden):
    g = golden("poisson_fv_n10.npz")
    a = omesh.poisson_fv(omesh.triangular_mesh(10))
    for k in ("Af", "Ac", "b", "rho", "centroid"):
        assert np.array_equal(a[k], g[k]), k


def test_selector_reducer_match_reference(golden):
    g = golden("selector_reducer.npz")
    n = g["f64_o3"].shape[0]
    for tag in ("f64", "f32"):
        assert np.array_equal(osp.select(torch.from_numpy(g[f"{tag}_x1"]), g["sel_idx"]).numpy(), g[f"{tag}_sel1"])
        assert np.array_equal(osp.select(torch.from_numpy(g[f"{tag}_x3"]), g["sel_idx"]).numpy(), g[f"{tag}_sel3"])
        for op in ("sum", "prod", "mean", "amax", "amin"):
            e1, e3, o3 = (torch.from_numpy(g[f"{tag}_{k}"]) for k in ("e1", "e3", "o3"))
            assert np.array_equal(osp.reduce(e1, g["red_idx"], n, op).numpy(), g[f"{tag}_{op}_1"]), op
            assert np.array_equal(osp.reduce(e3, g["red_idx"], n, op).numpy(), g[f"{tag}_{op}_3"]), op
            assert np.array_equal(osp.reduce(e3, g["red_idx"], n, op, out=o3).numpy(), g[f"{tag}_{op}_3out"]), op


def _swe_problem(n, dt, dtype):
    m = omesh.triangular_mesh(n)
    geo = omesh.swe_geometry(m)
    return oswe.SweProblem(m["src"], m["dst"], m["bcells"], geo["sx"], geo["sy"], geo["alpha"], geo["bsx"],
                           geo["bsy"], geo["area"], dt, dtype)


@pytest.mark.parametrize("dtype,tag", [(torch.float64, "f64"), (torch.float32, "f32")])
def test_swe_tutorial_n10_matches_reference(golden, dtype, tag):
    g = golden(f"swe_n10_{tag}_tutorial.npz")
    p = _swe_problem(10, float(g["dt"]), dtype)
    h0 = torch.from_numpy(g["h0"]).to(dtype)
    h, uh, vh = p.run(h0, torch.zeros_like(h0), torch.zeros_like(h0), int(g["steps"]))
    assert np.array_equal(h.numpy(), g["h"])
    assert np.array_equal(uh.numpy(), g["uh"])
    assert np.array_equal(vh.numpy(), g["vh"])


def test_swe_n100_1000_steps_matches_reference(golden):
    """The reference's CPU-runnable benchmark case, full length, FP64."""
    g = golden("swe_n100_f64_1000steps.npz")
    p = _swe_problem(100, float(g["dt"]), torch.float64)
    h0 = torch.from_numpy(g["h0"])
    h, uh, vh = p.run(h0, torch.zeros_like(h0), torch.zeros_like(h0), int(g["steps"]))
    assert np.array_equal(h.numpy(), g["h"])
    assert np.array_equal(uh.numpy(), g["uh"])
    assert np.array_equal(vh.numpy(), g["vh"])


def test_cg_matches_reference_fv(golden):
    g = golden("poisson_fv_n10_solve.npz")
    m = omesh.triangular_mesh(10)
    a = omesh.poisson_fv(m)
    x, iters, res = ocg.cg(m["src"], m["dst"], a["Af"], a["Ac"], a["b"], rtol=1e-8, maxiter=2000)
    assert abs(iters - int(g["cg_iters"])) <= 2
    ref = g["cg_x"]
    assert np.linalg.norm(x.numpy() - ref) <= 1e-7 * np.linalg.norm(ref)


def test_cg_matches_reference_fv_n100(golden):
    """The tutorial's FV Poisson at N=100 (40,000 cells), the reference's CG
    to relative residual 1e-8: same iterations, same solution."""
    g = golden("poisson_fv_n100_cg.npz")
    m = omesh.triangular_mesh(100)
    a = omesh.poisson_fv(m)
    x, iters, res = ocg.cg(m["src"], m["dst"], a["Af"], a["Ac"], a["b"], rtol=1e-8, maxiter=5000)
    assert abs(iters - int(g["cg_iters"])) <= 1
    ref = g["cg_x"]
    assert np.linalg.norm(x.numpy() - ref) <= 1e-9 * np.linalg.norm(ref)


def test_cg_matches_reference_p1(golden):
    g = golden("linsys_p1_n12_cg.npz")
    x, iters, res = ocg.cg(g["row"], g["col"], g["Ae"], g["Av"], g["b"], rtol=1e-10, maxiter=1000)
    assert abs(iters - int(g["iters"])) <= 1
    assert np.allclose(x.numpy(), g["x"], rtol=1e-9, atol=1e-12)


def test_rcm_oracle_is_a_permutation_with_small_bandwidth():
    m = omesh.triangular_mesh(6)
    order = osp.rcm(m["src"].shape[0] and 4 * 36, m["src"], m["dst"])
    assert np.array_equal(np.sort(order), np.arange(4 * 36))
    assert osp.bandwidth(order, m["src"], m["dst"]) < osp.bandwidth(np.arange(4 * 36), m["src"], m["dst"]) * 2
