"""The tile partition on the GPU (esr_bisect_partition_device) against the
host partition (esr_bisect_partition): the same part sizes in the same
order, deterministic, and parts as compact as the host's (the halo the
tile layout builds around them)."""
import numpy as np
import pytest
import torch

from easier_gb300 import mesh, swe

pytestmark = pytest.mark.gpu


def _graph(n):
    m = mesh.triangular_mesh(n)
    src, dst = np.asarray(m.src, np.int64), np.asarray(m.dst, np.int64)
    return int(max(src.max(), dst.max()) + 1), src, dst


@pytest.mark.parametrize("n,max_part", [(5, 7), (30, 100), (41, 333), (64, 1900), (20, 1), (12, 10**6)])
def test_device_partition_sizes_and_determinism(n, max_part):
    nc, src, dst = _graph(n)
    hp, hn = mesh.bisect_partition(nc, src, dst, max_part)
    s, d = torch.from_numpy(src).cuda(), torch.from_numpy(dst).cuda()
    dp, dn = mesh.bisect_partition(nc, s, d, max_part)
    dp2, _ = mesh.bisect_partition(nc, s, d, max_part)
    assert dn == hn
    assert torch.equal(dp, dp2)
    dp = dp.cpu().numpy()
    assert dp.min() == 0 and dp.max() == dn - 1
    assert np.array_equal(np.bincount(dp, minlength=dn), np.bincount(hp, minlength=hn))


def test_device_partition_of_a_disconnected_graph():
    """Two copies of a mesh side by side (no edge between them)."""
    nc, src, dst = _graph(24)
    src2, dst2 = np.concatenate([src, src + nc]), np.concatenate([dst, dst + nc])
    hp, hn = mesh.bisect_partition(2 * nc, src2, dst2, 500)
    dp, dn = mesh.bisect_partition(2 * nc, torch.from_numpy(src2).cuda(), torch.from_numpy(dst2).cuda(), 500)
    assert dn == hn
    assert np.array_equal(np.bincount(dp.cpu().numpy(), minlength=dn), np.bincount(hp, minlength=hn))


@pytest.mark.parametrize("n,target", [(200, 1900), (400, 1900)])
def test_device_partition_is_as_compact_as_the_host_partition(n, target):
    m = mesh.triangular_mesh(n)
    src, dst, b = (np.asarray(a, np.int64) for a in (m.src, m.dst, m.bcells))
    nc = int(max(src.max(), dst.max()) + 1)
    stats = {}
    for where in ("host", "device"):
        if where == "device":
            part, _ = mesh.bisect_partition(nc, torch.from_numpy(src).cuda(), torch.from_numpy(dst).cuda(), target)
            part = part.cpu().numpy()
        else:
            part, _ = mesh.bisect_partition(nc, src, dst, target)
        order = np.argsort(part, kind="stable")
        inv = np.empty(nc, np.int64)
        inv[order] = np.arange(nc)
        lay = swe.cell_layout(nc, inv[src], inv[dst], inv[b], reorder="tiles")
        stats[where] = swe.tile_layout(lay["nbr"], part[order])["stats"]
    h, d = stats["host"], stats["device"]
    assert d["ntiles"] == h["ntiles"] and d["max_own"] == h["max_own"]
    assert d["l3_over_own"] <= h["l3_over_own"] * 1.05, (d["l3_over_own"], h["l3_over_own"])
    assert d["max_local"] <= 4096


def test_device_partition_rejects_a_bad_edge():
    nc, src, dst = _graph(6)
    dst = dst.copy()
    dst[3] = nc + 5
    with pytest.raises(ValueError, match="out of range"):
        mesh.bisect_partition(nc, torch.from_numpy(src).cuda(), torch.from_numpy(dst).cuda(), 10)
