"""Host-side layouts of the fused shallow-water step (no GPU).

The tiled kernel runs, per tile, stage k on the local cells of level
<= 4-k, reading neighbours through the local face slots.  This simulates that
exact schedule on the CPU from the layout arrays and requires the result to
be bitwise the oracle's global step: it proves the tile lists, halo rings and
local slots are complete and correctly indexed."""
import numpy as np
import pytest
import torch

from easier_gb300 import mesh, swe
from oracle import mesh as omesh
from oracle import swe as oswe


def _tile_layout_numpy(nbr: np.ndarray, part: np.ndarray) -> dict:
    """Independent numpy construction of the tiled layout (checker of the
    native builder).  Same definition as esr_swe_tile_layout.

    nbr [3, nc]: face slots in a tile-major cell numbering (neighbour cell,
    -1 wall, -2 empty); part [nc]: non-decreasing tile of every cell.  Per
    tile, the local list is the tile's cells followed by the rings of
    in-neighbours at distance 1..4, each ring sorted by cell; cells of
    levels <= 3 get local face slots.  Returns numpy arrays: meta [ntiles, 8]
    (cell_off, n0, n1, n2, n3, nL), off3, offh, halo, lnbr, slot_src (index
    into the flattened [3, nc] slot arrays), area_src, and stats."""
    nc = nbr.shape[1]
    ntiles = int(part.max()) + 1
    counts = np.bincount(part, minlength=ntiles)
    cell_off = np.concatenate([[0], np.cumsum(counts)[:-1]])
    keys = [part * nc + np.arange(nc, dtype=np.int64)]         # level 0, sorted
    seen = keys[0]
    inner = nbr >= 0
    nbr_part = np.where(inner, part[np.where(inner, nbr, 0)], -1)
    border = np.nonzero(((nbr_part != part[None, :]) & inner).any(axis=0))[0]
    f_cells, f_tiles = border, part[border]
    for _level in range(1, 5):
        cand_c = nbr[:, f_cells]
        ok = cand_c >= 0
        cand = np.unique(np.broadcast_to(f_tiles, cand_c.shape)[ok] * nc + cand_c[ok].astype(np.int64))
        pos = np.minimum(np.searchsorted(seen, cand), seen.shape[0] - 1)
        new = cand[seen[pos] != cand]
        keys.append(new)
        seen = np.union1d(seen, new)
        f_cells, f_tiles = new % nc, new // nc
    all_keys = np.concatenate(keys)
    levels = np.concatenate([np.full(k.shape[0], lv, np.int64) for lv, k in enumerate(keys)])
    tiles = all_keys // nc
    cells = all_keys % nc
    o = np.lexsort((cells, levels, tiles))
    tiles, levels, cells, all_keys = tiles[o], levels[o], cells[o], all_keys[o]
    tile_start = np.searchsorted(tiles, np.arange(ntiles + 1))
    local = np.arange(tiles.shape[0], dtype=np.int64) - tile_start[tiles]
    cnt = np.bincount(tiles * 5 + levels, minlength=ntiles * 5).reshape(ntiles, 5)
    cum = np.cumsum(cnt, axis=1)                                 # n0, n1, n2, n3, nL
    if not np.array_equal(cnt[:, 0], counts):
        raise RuntimeError("tile layout: inconsistent tile sizes")
    korder = np.argsort(all_keys)
    sorted_keys = all_keys[korder]
    sel = levels <= 3
    t3, c3, l3 = tiles[sel], cells[sel], local[sel]
    off3 = np.concatenate([[0], np.cumsum(cum[:, 3])[:-1]]).astype(np.int64)
    base3 = off3[t3]
    n3_t = cum[t3, 3]
    total3 = int(cum[:, 3].sum())
    lnbr = np.empty(3 * total3, np.int32)
    slot_src = np.empty(3 * total3, np.int64)
    for k in range(3):
        g = nbr[k, c3].astype(np.int64)
        dst_i = 3 * base3 + k * n3_t + l3
        q = np.where(g >= 0, t3 * nc + np.maximum(g, 0), -1)
        p = np.minimum(np.searchsorted(sorted_keys, np.maximum(q, 0)), sorted_keys.shape[0] - 1)
        found = sorted_keys[p] == q
        if not np.all(found | (g < 0)):
            raise RuntimeError("tile layout: a neighbour is outside the halo")
        lnbr[dst_i] = np.where(g >= 0, local[korder[p]], g).astype(np.int32)
        slot_src[dst_i] = k * nc + c3
    area_src = np.empty(total3, np.int64)
    area_src[base3 + l3] = c3
    halo = cells[levels >= 1].astype(np.int32)
    offh = np.concatenate([[0], np.cumsum(cum[:, 4] - cum[:, 0])[:-1]]).astype(np.int64)
    meta = np.zeros((ntiles, 8), np.int32)
    meta[:, 0] = cell_off
    meta[:, 1:6] = cum
    max_own, max_l3, max_local = int(cum[:, 0].max()), int(cum[:, 3].max()), int(cum[:, 4].max())
    stats = dict(ntiles=ntiles, max_own=max_own, max_l3=max_l3, max_local=max_local,
                 max_halo3=int((cum[:, 3] - cum[:, 0]).max()), slot_info=int(all(int((lnbr[3 * off3[t] + np.arange(3) * cum[t, 3] + jj] < 0).sum()) <= 1
                                   for t in range(ntiles) for jj in range(cum[t, 3]))),
                 mean_own=float(counts.mean()), l3_over_own=float(total3 / nc),
                 local_over_own=float(cum[:, 4].sum() / nc), smem=(3 * max_local + 6 * max_l3) * 4)
    return dict(meta=meta, off3=off3, offh=offh, halo=halo, lnbr=lnbr, slot_src=slot_src, area_src=area_src,
                stats=stats)


@pytest.mark.parametrize("n,tile", [(3, 8), (12, 100), (40, 700), (64, 4096)])
def test_native_tile_layout_matches_numpy(n, tile):
    m = mesh.triangular_mesh(n)
    lay = swe.cell_layout(m.nc, m.src, m.dst, m.bcells, tile_cells=tile)
    a = swe.tile_layout(lay["nbr"], lay["part"])
    b = _tile_layout_numpy(lay["nbr"], lay["part"])
    for k in ("meta", "off3", "offh", "halo", "lnbr", "slot_src", "area_src"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    assert a["stats"] == b["stats"]


def _flux_sums(q, own, nbrs, fx, fy, al):
    """Per-slot contribution of swe_main.py:87-119 (one slot, vectorised)."""
    oh, ou, ov = own
    nh, nu, nv = nbrs
    om = 1 - al
    hf = om * nh + al * oh
    uhf = om * nu + al * ou
    vhf = om * nv + al * ov
    uf = uhf / hf
    vf = vhf / hf
    hfs = 0.5 * hf * hf
    uhsx = uhf * fx
    vhsy = vhf * fy
    return uhsx + vhsy, (uf * uhf + hfs) * fx + uf * vhsy, vf * uhsx + (vf * vhf + hfs) * fy


def _delta(count, n3, lnbr, sx, sy, al, area, S):
    hs, us, vs = S
    j = torch.arange(count)
    own = (hs[j], us[j], vs[j])
    z = torch.zeros(count, dtype=hs.dtype)
    Sh, Su, Sv, Bu, Bv = z.clone(), z.clone(), z.clone(), z.clone(), z.clone()
    for k in range(3):
        q = lnbr[k * n3 + j]
        inner = q >= 0
        qq = torch.where(inner, q, torch.zeros_like(q))
        fh, fu, fv = _flux_sums(q, own, (hs[qq], us[qq], vs[qq]), sx[k * n3 + j], sy[k * n3 + j], al[k * n3 + j])
        Sh = torch.where(inner, Sh + fh, Sh)
        Su = torch.where(inner, Su + fu, Su)
        Sv = torch.where(inner, Sv + fv, Sv)
        wall = q == -1
        gb = 0.5 * (own[0] * own[0])
        Bu = torch.where(wall, Bu + gb * sx[k * n3 + j], Bu)
        Bv = torch.where(wall, Bv + gb * sy[k * n3 + j], Bv)
    ar = area[j]
    return -Sh / ar, -(Su + Bu) / ar, -(Sv + Bv) / ar


def _simulate_tiled(lay, tl, state, geom_slots, area, dt, dtype):
    """The schedule of swe_tile_step_kernel, on the host."""
    meta, off3, offh = tl["meta"], tl["off3"], tl["offh"]
    halo = torch.from_numpy(tl["halo"].astype(np.int64))
    lnbr = torch.from_numpy(tl["lnbr"].astype(np.int64))
    sxf, syf, alf = (g.reshape(-1)[torch.from_numpy(tl["slot_src"])] for g in geom_slots)
    arf = area[torch.from_numpy(tl["area_src"])]
    c1, c3, c4 = (torch.tensor(v, dtype=dtype) for v in (0.5 * dt, dt, dt / 6))
    out = torch.empty_like(state)
    for t in range(meta.shape[0]):
        cell_off, n0, n1, n2, n3, nL = (int(v) for v in meta[t, :6])
        gid = torch.cat([torch.arange(cell_off, cell_off + n0), halo[int(offh[t]):int(offh[t]) + nL - n0]])
        s0 = [state[gid, c] for c in range(3)]
        o = int(off3[t])
        args = (lnbr[3 * o:3 * o + 3 * n3], sxf[3 * o:3 * o + 3 * n3], syf[3 * o:3 * o + 3 * n3],
                alf[3 * o:3 * o + 3 * n3], arf[o:o + n3])
        S = s0
        acc = None
        for stage, (count, c) in enumerate(((n3, c1), (n2, c1), (n1, c3), (n0, c4)), start=1):
            d = _delta(count, n3, *args, S)
            if stage < 4:
                S = [s0[i][:count] + c * d[i] for i in range(3)]
                S = [torch.cat([S[i], torch.zeros(nL - count, dtype=dtype)]) for i in range(3)]
                acc = [d[i][:n0] for i in range(3)] if stage == 1 else [acc[i] + d[i][:n0] for i in range(3)]
            else:
                for i in range(3):
                    out[cell_off:cell_off + n0, i] = s0[i][:n0] + c * (acc[i] + d[i])
    return out


@pytest.mark.parametrize("n,tile,dtype", [(6, 40, torch.float64), (16, 300, torch.float64), (16, 130, torch.float32)])
def test_tiled_schedule_matches_oracle_step(n, tile, dtype):
    m = omesh.triangular_mesh(n)
    geo = omesh.swe_geometry(m)
    nc, dt = m["cells"].shape[0], 2e-3
    lay = swe.cell_layout(nc, m["src"], m["dst"], m["bcells"], tile_cells=tile)
    assert lay["part"] is not None and lay["width"] == 3
    tl = swe.tile_layout(lay["nbr"], lay["part"])
    st = tl["stats"]
    assert st["ntiles"] > 2 and st["max_own"] <= tile
    order = torch.from_numpy(lay["order"])
    pos = torch.from_numpy(lay["pos"])
    fx = torch.cat([torch.from_numpy(geo["sx"]), torch.from_numpy(geo["bsx"])]).to(dtype)
    fy = torch.cat([torch.from_numpy(geo["sy"]), torch.from_numpy(geo["bsy"])]).to(dtype)
    fa = torch.cat([torch.from_numpy(geo["alpha"]), torch.zeros(len(geo["bsx"]), dtype=torch.float64)]).to(dtype)
    valid = pos >= 0
    safe = torch.where(valid, pos, torch.zeros_like(pos))
    slots = [torch.where(valid, f[safe], torch.zeros(1, dtype=dtype)) for f in (fx, fy, fa)]
    area = torch.from_numpy(geo["area"]).to(dtype)[order]
    rng = np.random.default_rng(n)
    h = torch.from_numpy(1 + 0.1 * rng.random(nc)).to(dtype)
    uh = torch.from_numpy(0.01 * rng.standard_normal(nc)).to(dtype)
    vh = torch.from_numpy(0.01 * rng.standard_normal(nc)).to(dtype)
    p = oswe.SweProblem(m["src"], m["dst"], m["bcells"], geo["sx"], geo["sy"], geo["alpha"], geo["bsx"], geo["bsy"],
                        geo["area"], dt, dtype)
    ref = p.step(h, uh, vh)
    state = torch.stack([h[order], uh[order], vh[order], torch.zeros(nc, dtype=dtype)], 1)
    got = _simulate_tiled(lay, tl, state, slots, area, dt, dtype)
    for i in range(3):
        back = torch.empty(nc, dtype=dtype)
        back[order] = got[:, i]
        assert torch.equal(back, ref[i]), i


def test_tile_layout_invariants():
    m = mesh.triangular_mesh(30)
    lay = swe.cell_layout(m.nc, m.src, m.dst, m.bcells, tile_cells=512)
    tl = swe.tile_layout(lay["nbr"], lay["part"])
    meta = tl["meta"]
    # tiles cover the cells contiguously and in order
    assert meta[0, 0] == 0 and np.all(meta[1:, 0] == meta[:-1, 0] + meta[:-1, 1])
    assert meta[-1, 0] + meta[-1, 1] == m.nc
    # level counts are cumulative and halo rings are non-empty but small
    assert np.all(np.diff(meta[:, 1:6], axis=1) >= 0)
    st = tl["stats"]
    assert 1.0 < st["l3_over_own"] < 1.5 and st["local_over_own"] < 1.6
    # every local neighbour index of a level<=3 cell points inside its tile's list
    for t in range(meta.shape[0]):
        n3, nL = meta[t, 4], meta[t, 5]
        o = tl["off3"][t]
        q = tl["lnbr"][3 * o:3 * o + 3 * n3]
        assert np.all((q < nL) & (q >= -2))
    # the tile-major numbering is a permutation; bisection parts are balanced
    assert np.array_equal(np.sort(lay["order"]), np.arange(m.nc))
    assert meta[:, 1].max() - meta[:, 1].min() <= 1


def test_staged_layout_without_tiles():
    m = mesh.triangular_mesh(5)
    lay = swe.cell_layout(m.nc, m.src, m.dst, m.bcells, tile_cells=None)
    assert lay["part"] is None and lay["width"] == 3
    nbr = lay["nbr"]
    # every cell: 3 interior faces, or 2 interior + 1 wall
    walls = (nbr == -1).sum(0)
    assert set(np.unique(walls)) <= {0, 1}
    assert (nbr == -2).sum() == 0
    assert walls.sum() == m.nbc


def test_bisect_partition_balanced_and_deterministic():
    m = mesh.triangular_mesh(40)
    p1, n1 = mesh.bisect_partition(m.nc, m.src, m.dst, 1000)
    p2, n2 = mesh.bisect_partition(m.nc, m.src, m.dst, 1000)
    assert n1 == n2 and np.array_equal(p1, p2)
    sizes = np.bincount(p1)
    assert sizes.max() <= 1000 and sizes.min() >= 500


def test_fast_record_order_sorts_each_cells_slots():
    """The fast-arithmetic record order permutes only within a cell's three
    slots and sorts them by local neighbour index."""
    m = mesh.triangular_mesh(30)
    lay = swe.cell_layout(m.nc, m.src, m.dst, m.bcells, tile_cells=500)
    tl = swe.tile_layout(lay["nbr"], lay["part"])
    order = swe._slots_by_neighbour(tl["meta"], tl["off3"], tl["lnbr"])
    assert np.array_equal(np.sort(order), np.arange(order.size))
    lnbr = tl["lnbr"]
    for t in range(tl["meta"].shape[0]):
        n3, base = int(tl["meta"][t, 4]), 3 * int(tl["off3"][t])
        idx = base + np.arange(3 * n3).reshape(3, n3)
        got = order[idx]
        # same cell (column), ascending neighbours
        assert np.array_equal(np.sort(got, axis=0), np.sort(idx, axis=0))
        assert np.all(np.diff(lnbr[got], axis=0) >= 0)


@pytest.mark.parametrize("n,tile", [(3, 8), (12, 100), (40, 700), (64, 1900), (3, 1000), (1, 5)])
def test_device_layout_functions_match_the_host_ones(n, tile):
    """The torch layout path a CUDA engine runs on the GPU (cell slots, tile
    rings, record order, slot_info), run here on CPU tensors with the host
    partition: every array equals the host functions' (numpy / C++)."""
    m = mesh.triangular_mesh(n)
    src, dst, b = (np.asarray(a, np.int64) for a in (m.src, m.dst, m.bcells))
    host = swe.cell_layout(m.nc, src, dst, b, reorder="tiles", tile_cells=tile)
    dev = swe._cell_layout_device(m.nc, *(torch.from_numpy(a) for a in (src, dst, b)), "tiles", tile)
    for k in ("order", "nbr", "pos", "part"):
        assert np.array_equal(np.asarray(host[k]), dev[k].numpy()), k
    assert host["width"] == dev["width"]
    th = swe.tile_layout(host["nbr"], host["part"])
    td = swe._tile_layout_device(dev["nbr"], dev["part"])
    for k in ("meta", "off3", "offh", "halo", "lnbr", "slot_src", "area_src"):
        assert np.array_equal(np.asarray(th[k]), td[k].numpy()), k
    assert th["stats"] == td["stats"]
    oh = swe._slots_by_neighbour(th["meta"], th["off3"], th["lnbr"])
    od = swe._slots_by_neighbour(td["meta"], td["off3"], td["lnbr"])
    assert np.array_equal(oh, od.numpy())


def test_device_tile_layout_rejects_bad_input():
    m = mesh.triangular_mesh(6)
    lay = swe.cell_layout(m.nc, m.src, m.dst, m.bcells, reorder="tiles", tile_cells=20)
    nbr, part = torch.from_numpy(lay["nbr"]), torch.from_numpy(lay["part"])
    with pytest.raises(ValueError, match="non-decreasing"):
        swe._tile_layout_device(nbr, part.flip(0))
    bad = nbr.clone()
    bad[0, 3] = m.nc
    with pytest.raises(ValueError, match="out of range"):
        swe._tile_layout_device(bad, part)
    skip = part.clone()
    skip[part >= 1] += 1
    with pytest.raises(ValueError, match="skip"):
        swe._tile_layout_device(nbr, skip)


@pytest.mark.parametrize("as_torch", [False, True])
def test_split_wide_tiles_cuts_the_tiles_over_the_limit(as_torch):
    """Tiles whose local list exceeds the limit are each cut in two (new
    tiles after the others); the rest keep their cells."""
    m = mesh.triangular_mesh(40)
    src, dst, b = (np.asarray(a, np.int64) for a in (m.src, m.dst, m.bcells))
    conv = (lambda a: torch.from_numpy(a)) if as_torch else (lambda a: a)
    lay = (swe._cell_layout_device(m.nc, conv(src), conv(dst), conv(b), "tiles", 600) if as_torch else
           swe.cell_layout(m.nc, src, dst, b, reorder="tiles", tile_cells=600))
    tiles = (swe._tile_layout_device if as_torch else swe.tile_layout)(lay["nbr"], lay["part"])
    meta = np.asarray(tiles["meta"])
    nl = meta[:, 5]
    limit = int(np.sort(nl)[-3])  # the two widest tiles exceed it
    wide = np.nonzero(nl > limit)[0]
    assert wide.size == 2
    assert swe.split_wide_tiles(lay, tiles, int(nl.max())) is None
    part = swe.split_wide_tiles(lay, tiles, limit)
    part = np.asarray(part)
    order = np.asarray(lay["order"])
    old = np.empty(m.nc, np.int64)
    old[order] = np.asarray(lay["part"])
    ntiles = meta.shape[0]
    assert part.max() == ntiles + 1
    for j, t in enumerate(wide):
        cells = old == t
        assert set(np.unique(part[cells])) == {t, ntiles + j}
        sizes = np.bincount(part[cells] == t)
        assert abs(int(sizes[0]) - int(sizes[1])) <= 1
    keep = ~np.isin(old, wide)
    assert np.array_equal(part[keep], old[keep])
    lay2 = (swe._cell_layout_device(m.nc, conv(src), conv(dst), conv(b), "tiles", None, conv(part)) if as_torch else
            swe.cell_layout(m.nc, src, dst, b, reorder="tiles", part=part))
    st2 = (swe._tile_layout_device if as_torch else swe.tile_layout)(lay2["nbr"], lay2["part"])["stats"]
    assert st2["ntiles"] == ntiles + 2 and st2["max_local"] < int(nl.max())
