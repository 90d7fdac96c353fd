"""Selector / Reducer / aggregators on the GPU through the public API,
against the reference's own outputs (golden) and the oracle: bitwise."""
import numpy as np
import pytest
import torch

import easier_gb300 as esr
from easier_gb300 import ops
from oracle import sparse as osp

pytestmark = pytest.mark.gpu


def _compiled(sel_idx=None, red_idx=None, n=None, op="sum"):
    class M(esr.Module):
        def __init__(self):
            super().__init__()
            if sel_idx is not None:
                self.sel = esr.Selector(torch.as_tensor(sel_idx))
            if red_idx is not None:
                self.red = esr.Reducer(torch.as_tensor(red_idx), n, reduce=op)
    m = M()
    esr.compile([m], "cuda")
    return m


def test_selector_reducer_match_reference_golden(golden):
    g = golden("selector_reducer.npz")
    n = g["f64_o3"].shape[0]
    ms = _compiled(sel_idx=g["sel_idx"])
    for tag in ("f64", "f32"):
        for k in ("1", "3"):
            x = torch.from_numpy(g[f"{tag}_x{k}"]).cuda()
            assert np.array_equal(ms.sel(x).cpu().numpy(), g[f"{tag}_sel{k}"])
        for op in ("sum", "prod", "mean", "amax", "amin"):
            mr = _compiled(red_idx=g["red_idx"], n=n, op=op)
            e1, e3, o3 = (torch.from_numpy(g[f"{tag}_{k}"]).cuda() for k in ("e1", "e3", "o3"))
            assert np.array_equal(mr.red(e1).cpu().numpy(), g[f"{tag}_{op}_1"]), (tag, op)
            assert np.array_equal(mr.red(e3).cpu().numpy(), g[f"{tag}_{op}_3"]), (tag, op)
            o = o3.clone()
            res = mr.red(e3, out=o)
            assert res.data_ptr() == o.data_ptr()
            assert np.array_equal(o.cpu().numpy(), g[f"{tag}_{op}_3out"]), (tag, op)


def test_reference_known_answers():
    # tests/core/test_module.py:28-87 of the reference, restated
    idx = torch.tensor([1, 1, 2, 2, 2])
    edge = torch.randn(5, 3, 4)
    m = _compiled(red_idx=idx, n=3)
    res0 = m.red(edge.cuda()).cpu()
    res1 = torch.zeros(3, 3, 4)
    res1[1] = edge[0] + edge[1]
    res1[2] = edge[2] + edge[3] + edge[4]
    assert torch.equal(res0, res1)
    out = torch.rand(3, 3, 4)
    o = out.cuda()
    m.red(edge.cuda(), out=o)
    res1[0] = out[0]
    assert torch.equal(o.cpu(), res1)
    sidx = torch.randint(0, 10, (20,))
    s = _compiled(sel_idx=sidx)
    t = torch.randn(10, 1, 2)
    assert torch.equal(s.sel(t.cuda()).cpu(), t[sidx])


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.int64, torch.int32])
def test_large_random_bitwise_vs_oracle(dtype):
    g = torch.Generator().manual_seed(3)
    m, n_in, n = 300_000, 50_000, 40_000
    sidx = torch.randint(0, n_in, (m,), generator=g)
    ridx = torch.randint(0, n, (m,), generator=g)
    if dtype.is_floating_point:
        x = torch.randn(n_in, 3, generator=g).to(dtype)
        e = torch.randn(m, generator=g).to(dtype)
    else:
        x = torch.randint(-1000, 1000, (n_in, 3), generator=g).to(dtype)
        e = torch.randint(-1000, 1000, (m,), generator=g).to(dtype)
    ms = _compiled(sel_idx=sidx)
    assert torch.equal(ms.sel(x.cuda()).cpu(), osp.select(x, sidx))
    for op in ("sum", "amax", "amin") + (("mean", "prod") if dtype.is_floating_point else ()):
        mr = _compiled(red_idx=ridx, n=n, op=op)
        got = mr.red(e.cuda()).cpu()
        assert torch.equal(got, osp.reduce(e, ridx, n, op)), op
        assert torch.equal(mr.red(e.cuda()).cpu(), got)  # deterministic


def test_empty_and_edge_cases():
    m = _compiled(sel_idx=torch.zeros(0, dtype=torch.long))
    assert m.sel(torch.randn(4).cuda()).shape == (0,)
    r = _compiled(red_idx=torch.zeros(0, dtype=torch.long), n=5)
    out = r.red(torch.zeros(0).cuda())
    assert torch.equal(out.cpu(), torch.zeros(5))
    s = _compiled(sel_idx=torch.tensor([0, 3]))
    with pytest.raises(IndexError):
        s.sel(torch.randn(3).cuda())
    with pytest.raises(ValueError):
        r.red(torch.zeros(0).cuda(), out=torch.zeros(4).cuda())


def test_selector_before_compile_raises():
    s = esr.Selector(torch.tensor([0, 1]))
    with pytest.raises(RuntimeError, match="run compile"):
        s(torch.randn(3).cuda())
    r = esr.Reducer(torch.tensor([0, 1]), 2)
    with pytest.raises(RuntimeError, match="run compile"):
        r(torch.randn(2).cuda())


def test_device_bounds_check_flags_instead_of_faulting():
    from easier_gb300 import _lib
    ops.device_status(clear=True)
    x = torch.arange(4, dtype=torch.float64, device="cuda")
    idx = torch.tensor([0, 7, 1], dtype=torch.int32, device="cuda")  # 7 is out of range
    y = torch.full((3,), -1.0, dtype=torch.float64, device="cuda")
    _lib.call("esr_gather", _lib.ptr(x), 4, 8, _lib.ptr(idx), 3, _lib.ptr(y), _lib.stream_handle())
    assert ops.device_status(clear=True) & _lib.DEV_IDX_RANGE
    assert y.cpu().tolist() == [0.0, -1.0, 1.0]
    assert ops.device_status(clear=True) == 0


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_aggregators(dtype):
    g = torch.Generator().manual_seed(5)
    t = torch.randn(123_457, 2, generator=g).to(dtype)
    tc = t.cuda()
    tol = 1e-12 if dtype == torch.float64 else 1e-5
    exact = t.double()
    assert torch.allclose(esr.sum(tc).cpu().double(), exact.sum(0, keepdim=True), rtol=tol, atol=tol * 100)
    assert torch.allclose(esr.norm(tc).cpu().double(), exact.norm(dim=0, keepdim=True), rtol=tol)
    assert torch.equal(esr.max(tc).cpu(), t.amax(0, keepdim=True))
    assert torch.equal(esr.min(tc).cpu(), t.amin(0, keepdim=True))
    small = (1 + 1e-3 * torch.randn(50, generator=g)).to(dtype)
    assert torch.allclose(esr.prod(small.cuda()).cpu().double(), small.double().prod(0, keepdim=True), rtol=tol)
    a, b = esr.sum(tc), esr.sum(tc)
    assert torch.equal(a, b)
    ti = torch.randint(-5, 5, (1000,), generator=g)
    assert torch.equal(esr.sum(ti.cuda()).cpu(), ti.sum(0, keepdim=True))


def test_full_size_edge_exchange_properties():
    """The bench mesh's edge exchange at full size (N=2000: 47,992,000
    directed edges onto 16,000,000 cells): the Selector gathers the source
    ids exactly, the Reducer's sum of ones is each cell's in-degree, its sum
    of source ids is the oracle's per-cell id sum (integers: exact), and the
    FP64 sum of all cell sums is the sum over all edges."""
    from easier_gb300 import mesh
    m = mesh.triangular_mesh(2000)
    src, dst = torch.from_numpy(m.src), torch.from_numpy(m.dst)
    mod = _compiled(sel_idx=src, red_idx=dst, n=m.nc)
    ids = torch.arange(m.nc, dtype=torch.int64, device="cuda")
    got_src = mod.sel(ids)
    assert torch.equal(got_src.cpu(), src)
    deg = mod.red(torch.ones(len(src), dtype=torch.float64, device="cuda"))
    assert torch.equal(deg.cpu(), torch.bincount(dst, minlength=m.nc).double())
    idsum = mod.red(got_src)
    ref = torch.zeros(m.nc, dtype=torch.int64).index_add_(0, dst, src)
    assert torch.equal(idsum.cpu(), ref)
    w = torch.rand(len(src), dtype=torch.float64, generator=torch.Generator().manual_seed(0))
    cell = mod.red(w.cuda())
    assert abs(float(cell.sum()) - float(w.sum())) <= 1e-9 * float(w.sum())


def test_reducer_csr_built_on_the_device_equals_the_host_csr():
    """compile for CUDA builds each Reducer's stable CSR with a device sort:
    the same rowptr/perm as esr_csr_from_index on the host."""
    from easier_gb300 import mesh

    class M(esr.Module):
        def __init__(self):
            super().__init__()
            g = torch.Generator().manual_seed(3)
            self.idx = torch.randint(0, 5000, (200_003,), generator=g)
            self.red = esr.Reducer(self.idx, 5000)
            self.x = esr.Tensor(torch.randn(200_003, generator=g, dtype=torch.float64), mode="partition")

        def forward(self):
            return self.red(self.x)

    m = M()
    [m] = esr.compile([m], "cuda")
    rowptr, perm = mesh.csr_from_index(m.idx.numpy(), 5000)
    assert np.array_equal(m.red._rowptr32.cpu().numpy(), rowptr.astype(np.int32))
    assert np.array_equal(m.red._perm32.cpu().numpy(), perm.astype(np.int32))


def test_reducer_index_out_of_range_fails_at_compile():
    from easier_gb300.utils import EasierJitException

    class M(esr.Module):
        def __init__(self):
            super().__init__()
            self.red = esr.Reducer(torch.tensor([0, 3, 9]), 4)

    with pytest.raises(EasierJitException, match="out of range"):
        esr.compile([M()], "cuda")
