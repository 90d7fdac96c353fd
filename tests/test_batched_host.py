"""Host packing of the batched PCG: the block-diagonal SELL-32 system applies
each instance's Linsys exactly (checked against the oracle's
index-multiply-scatter-add), padding rows are identity rows, no column
crosses an instance, and the df64 split is exact to ~48 bits."""
import numpy as np
import torch

from easier_gb300 import mesh
from easier_gb300.numeric.batched import (ROWS_PER_BLOCK, LinsysInstance, PackedBatch, join_df64, p1_instances,
                                          split_df64)
from oracle import sparse as osp


def _sell_apply(pk: PackedBatch, x: np.ndarray) -> np.ndarray:
    y = pk.diag * x
    nsl = pk.n // 32
    for s in range(nsl):
        b, e = int(pk.slice_ptr[s]), int(pk.slice_ptr[s + 1])
        w = (e - b) // 32
        for k in range(w):
            sl = slice(b + 32 * k, b + 32 * k + 32)
            c = pk.col[sl]
            ok = c >= 0
            rows = 32 * s + np.arange(32)
            y[rows[ok]] += pk.val[sl][ok] * x[c[ok]]
    return y


def test_pack_applies_each_instance():
    rng = np.random.default_rng(0)
    insts = []
    for n in (5, 9, 20):  # 16, 64 and 361 unknowns: one partial block, one, two
        kappa = mesh.kappa_from_field(mesh.gaussian_random_field(n, n))
        s = mesh.p1_system(n, kappa)
        insts.append(LinsysInstance(s.nunk, s.row, s.col, s.Ae, s.Av, rng.standard_normal(s.nunk)))
    pk = PackedBatch(insts)
    assert pk.n == ROWS_PER_BLOCK * pk.nblocks
    assert list(pk.inst_block0) == [0, 1, 2, 4]
    assert list(pk.block_inst) == [0, 1, 2, 2]
    x = rng.standard_normal(pk.n)
    y = _sell_apply(pk, x)
    for i, s in enumerate(insts):
        rows = pk.rows(i)
        ref = osp.linsys_apply(torch.from_numpy(x[rows].copy()), s.row, s.col, torch.from_numpy(s.Ae),
                               torch.from_numpy(s.Av)).numpy()
        assert np.allclose(y[rows], ref, rtol=1e-13, atol=1e-13)
        assert np.array_equal(pk.b[rows], s.b)
        # columns of instance i stay inside its padded block range
        lo, hi = int(pk.row0[i]), int(pk.inst_block0[i + 1]) * ROWS_PER_BLOCK
        s0 = lo // 32
        s1 = hi // 32
        c = pk.col[pk.slice_ptr[s0]:pk.slice_ptr[s1]]
        c = c[c >= 0]
        assert c.size and c.min() >= lo and c.max() < lo + s.n
    pad = np.ones(pk.n, bool)
    for i in range(len(insts)):
        pad[pk.rows(i)] = False
    assert np.all(pk.diag[pad] == 1.0) and np.all(pk.b[pad] == 0.0)
    assert np.array_equal(y[pad], x[pad])


def test_pack_empty_and_exact_block_instances():
    s = mesh.p1_system(17)  # 256 unknowns: exactly one block, no padding
    pk = PackedBatch([LinsysInstance(s.nunk, s.row, s.col, s.Ae, s.Av, np.ones(s.nunk)),
                      LinsysInstance(0, np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0), np.zeros(0),
                                     np.zeros(0))])
    assert s.nunk == 256 and pk.nblocks == 2 and list(pk.inst_block0) == [0, 1, 2]


def test_df64_split_roundtrip():
    rng = np.random.default_rng(3)
    v = torch.from_numpy(rng.standard_normal(1000) * 10.0 ** rng.integers(-8, 8, 1000))
    d = split_df64(v)
    assert d.dtype == torch.float32 and d.shape == (1000, 2)
    err = (join_df64(d) - v).abs() / v.abs()
    assert float(err.max()) < 2.0 ** -47
    # hi is the FP32 rounding of v, and |lo| <= ulp(hi) / 2
    assert torch.equal(d[:, 0], v.to(torch.float32))


def test_p1_instances_seeded():
    a = p1_instances(3, 8, 16, seed=5)
    b = p1_instances(3, 8, 16, seed=5)
    assert [s.n for s in a] == [s.n for s in b]
    for s, t in zip(a, b):
        assert np.array_equal(s.Ae, t.Ae) and np.array_equal(s.b, t.b)
        m = int(round(np.sqrt(s.n))) + 1
        assert 8 <= m <= 16 and (m - 1) ** 2 == s.n


def test_chunk_layout():
    from easier_gb300.numeric.batched import chunk_layout
    ib0 = np.array([0, 1, 2, 4, 14], np.int32)
    ct0, ci, ic0 = chunk_layout(ib0, 4)
    assert list(ct0) == [0, 1, 2, 4, 8, 12, 14]
    assert list(ci) == [0, 1, 2, 3, 3, 3]
    assert list(ic0) == [0, 1, 2, 3, 6]
    for m in (1, 3, 16):
        ct0, ci, ic0 = chunk_layout(ib0, m)
        assert ct0[0] == 0 and ct0[-1] == 14 and np.all(np.diff(ct0) >= 1) and np.all(np.diff(ct0) <= m)
        # every chunk lies inside its instance's tiles
        assert np.all(ct0[:-1] >= ib0[ci]) and np.all(ct0[1:] <= ib0[ci + 1])
        assert np.array_equal(np.searchsorted(ic0, np.arange(len(ci)), side="right") - 1, ci)


def test_pack_leaves_out_zero_couplings_but_the_gnn_graph_keeps_them():
    """Exact-zero couplings (P1: the hypotenuse pairs) are not stored for the
    SpMV, which still applies the same operator; the GNN's pack keeps them."""
    rng = np.random.default_rng(1)
    s = mesh.p1_system(12)
    assert (s.Ae == 0).sum() > 0
    inst = LinsysInstance(s.nunk, s.row, s.col, s.Ae, s.Av, rng.standard_normal(s.nunk),
                          edge_len=np.ones(len(s.Ae)))
    lean, full = PackedBatch([inst]), PackedBatch([inst], edge_features=True)
    stored = lambda pk: int((pk.col >= 0).sum())  # noqa: E731
    assert stored(lean) == int((s.Ae != 0).sum()) and stored(full) == len(s.Ae)
    x = rng.standard_normal(lean.n)
    assert np.array_equal(_sell_apply(lean, x), _sell_apply(full, x))


def test_poly_jacobi_oracle_is_the_neumann_polynomial():
    """The oracle's polynomial-Jacobi preconditioner (d+1 damped Jacobi
    sweeps from z = 0) equals sum_{j<=d} (I - W A)^j W r formed densely."""
    from oracle import cg as ocg
    n = 7
    kappa = mesh.kappa_from_field(mesh.gaussian_random_field(n, 3))
    s = mesh.p1_system(n, kappa)
    Ae, Av = torch.from_numpy(s.Ae), torch.from_numpy(s.Av)
    A = lambda v: osp.linsys_apply(v, s.row, s.col, Ae, Av)  # noqa: E731
    dense = torch.stack([A(e) for e in torch.eye(s.nunk, dtype=torch.float64)], 1)
    r = torch.from_numpy(np.random.default_rng(1).standard_normal(s.nunk))
    for d, om in ((2, 0.8), (3, 2 / 3), (4, 0.8)):
        W = torch.diag(om / Av)
        T = torch.eye(s.nunk, dtype=torch.float64) - W @ dense
        ref = sum(torch.linalg.matrix_power(T, j) for j in range(d + 1)) @ W @ r
        z = ocg.poly_jacobi(A, Av, r, d, om)
        assert torch.allclose(z, ref, rtol=1e-12, atol=1e-12)
        # M = p(WA) W is symmetric positive definite on this SPD system
        M = sum(torch.linalg.matrix_power(T, j) for j in range(d + 1)) @ W
        assert torch.allclose(M, M.T, rtol=1e-10, atol=1e-12)
        assert float(torch.linalg.eigvalsh(0.5 * (M + M.T)).min()) > 0.0


def test_poly_jacobi_arguments_are_checked_before_any_device_work():
    import pytest
    from easier_gb300.numeric.batched import BatchedPCG
    insts = p1_instances(2, 6, 8, seed=0)
    for kw, msg in (({"poly_degree": 1}, "poly_degree"), ({"poly_degree": 17}, "poly_degree"),
                    ({"poly_degree": 4, "jacobi": False}, "jacobi"),
                    ({"poly_degree": 4, "poly_omega": 0.0}, "poly_omega")):
        with pytest.raises(ValueError, match=msg):
            BatchedPCG(insts, device="cuda", **kw)


def test_poly_jacobi_batch_rejected_by_the_c_abi():
    """esr_bcg_init refuses a polynomial batch with a bad degree, a GNN or
    no scratch before it touches memory (the pointers here are dummies, so
    the test runs only where no GPU could be reached)."""
    import ctypes
    import pytest
    from easier_gb300 import _lib
    if torch.cuda.is_available():
        pytest.skip("dummy device pointers: host-only check")
    lib = _lib.lib()
    d = 0x1000
    g = _lib.Gnn(*([d] * 10), 0.0, 1, 16, 0)

    def batch(degree, tmp=d, gnn=None):
        return _lib.Batch(256, 1, 1, 256, 1, 1, 1, *([d] * 12), gnn, tmp, degree, 0)

    for b, msg in ((batch(1), b"poly_degree"), (batch(17), b"poly_degree"), (batch(4, tmp=None), b"poly_tmp"),
                   (batch(4, gnn=ctypes.pointer(g)), b"exclude")):
        rc = lib.esr_bcg_init(ctypes.byref(b), d, d, d, d, d, d, 1e-8, 0.0, -1, d, None)
        assert rc == 1, rc  # ESR_ERR_ARG
        assert msg in lib.esr_last_error()
