"""The tile partition on the GPU (esr_bisect_partition_device) against the
host partition (esr_bisect_partition): the same parts, vertex for vertex;
and the whole tiled layout a CUDA engine builds on the GPU against the one
the host functions build, array for array."""
import numpy as np
import pytest
import torch

from easier_gb300 import mesh, swe

pytestmark = pytest.mark.gpu


def _graph(n):
    m = mesh.triangular_mesh(n)
    src, dst = np.asarray(m.src, np.int64), np.asarray(m.dst, np.int64)
    return int(max(src.max(), dst.max()) + 1), src, dst


@pytest.mark.parametrize("n,max_part", [(5, 7), (30, 100), (41, 333), (64, 1900), (20, 1), (12, 10**6),
                                        (200, 1900)])
def test_device_partition_equals_the_host_partition(n, max_part):
    nc, src, dst = _graph(n)
    hp, hn = mesh.bisect_partition(nc, src, dst, max_part)
    s, d = torch.from_numpy(src).cuda(), torch.from_numpy(dst).cuda()
    dp, dn = mesh.bisect_partition(nc, s, d, max_part)
    dp2, _ = mesh.bisect_partition(nc, s, d, max_part)
    assert dn == hn
    assert torch.equal(dp, dp2)
    assert np.array_equal(dp.cpu().numpy(), hp)


def test_device_partition_of_a_high_degree_graph():
    """Degrees above 8 take the CSR rows instead of the fixed-width ones: a
    mesh plus hub vertices joined to many cells, and duplicate edges."""
    nc, src, dst = _graph(40)
    rng = np.random.default_rng(5)
    hubs = rng.integers(0, nc, 6)
    extra_s = np.repeat(hubs, 25)
    extra_d = rng.integers(0, nc, extra_s.size)
    src2 = np.concatenate([src, extra_s, src[:50]])
    dst2 = np.concatenate([dst, extra_d, dst[:50]])
    for max_part in (97, 640):
        hp, hn = mesh.bisect_partition(nc, src2, dst2, max_part)
        dp, dn = mesh.bisect_partition(nc, torch.from_numpy(src2).cuda(), torch.from_numpy(dst2).cuda(), max_part)
        assert dn == hn
        assert np.array_equal(dp.cpu().numpy(), hp)


def test_device_partition_of_a_disconnected_graph():
    """Two copies of a mesh side by side (no edge between them)."""
    nc, src, dst = _graph(24)
    src2, dst2 = np.concatenate([src, src + nc]), np.concatenate([dst, dst + nc])
    hp, hn = mesh.bisect_partition(2 * nc, src2, dst2, 500)
    dp, dn = mesh.bisect_partition(2 * nc, torch.from_numpy(src2).cuda(), torch.from_numpy(dst2).cuda(), 500)
    assert dn == hn
    assert np.array_equal(dp.cpu().numpy(), hp)


@pytest.mark.parametrize("n,target", [(64, 700), (300, 1900)])
def test_engine_layout_built_on_the_gpu_equals_the_host_built_layout(n, target, monkeypatch):
    """Every array of the fused engine's tiled layout: cell order, face
    slots, tile meta, halo, local neighbours, geometry records."""
    import easier_gb300 as esr
    from easier_gb300 import workloads
    monkeypatch.setattr(swe, "PIPE_TILE_TARGET", target)
    got = {}
    for on_device in (False, True):
        monkeypatch.setattr(swe, "LAYOUT_ON_DEVICE", on_device)
        eqn = workloads.make_swe(n, dt=5e-4, dtype=torch.float32)
        [eqn] = esr.compile([eqn], "cuda", precision="fast")
        eng = eqn.easier_fused_engine
        assert eng.tiled
        got[on_device] = {k: getattr(eng, k).cpu() for k in ("order", "nbr", "slot_pos", "tile_meta", "tile_off3",
                                                                "tile_offh", "tile_halo", "tile_lnbr", "tile_gsrc",
                                                                "tile_area_src", "tile_fast_order", "t_slots")}
        got[on_device]["stats"] = dict(eng.tile_stats)
    for k, v in got[False].items():
        if k == "stats":
            assert v == got[True][k]
        else:  # bit patterns (the records carry int32 neighbour indices in a float lane: -1, -2 are NaNs)
            w = got[True][k]
            if v.dtype == torch.float32:
                v, w = v.view(torch.int32), w.view(torch.int32)
            assert torch.equal(v, w), k


def test_device_partition_rejects_a_bad_edge():
    nc, src, dst = _graph(6)
    dst = dst.copy()
    dst[3] = nc + 5
    with pytest.raises(ValueError, match="out of range"):
        mesh.bisect_partition(nc, torch.from_numpy(src).cuda(), torch.from_numpy(dst).cuda(), 10)
