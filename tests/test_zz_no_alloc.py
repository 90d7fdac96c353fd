"""The allocation-free aggregate, ``esr_aggregate_noalloc``, called through
the C ABI: it must give exactly what ``esr_aggregate`` gives with a
caller-provided workspace.

It is for callers that cannot call cudaMalloc where they aggregate (the
call synchronises the whole device, can run out of memory mid-run, or the
host application owns all device memory), so its scratch is a static device
array instead.  Two calls in a row, on different data and sizes, check that
the contents the previous call left in that shared array never leak into a
result.  This file sorts last so a stop-at-first-failure run has already run
every other test when it gets here.
"""
import ctypes

import pytest
import torch

from easier_gb300 import _lib

pytestmark = pytest.mark.gpu


def _aggregate_with_workspace(t: torch.Tensor, agg: int) -> torch.Tensor:
    n, cols = t.shape[0], int(t[0].numel()) if t.dim() > 1 else 1
    out = torch.empty((1,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
    ws = torch.empty(max(int(_lib.lib().esr_aggregate_workspace_bytes(n, cols)), 16), dtype=torch.uint8,
                     device=t.device)
    _lib.call("esr_aggregate", _lib.dtype_code(t.dtype), agg, _lib.ptr(t), n, cols, _lib.ptr(out), _lib.ptr(ws),
              _lib.stream_handle(t.device))
    return out


def _aggregate_noalloc(t: torch.Tensor, agg: int) -> torch.Tensor:
    n, cols = t.shape[0], int(t[0].numel()) if t.dim() > 1 else 1
    out = torch.empty((1,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
    _lib.call("esr_aggregate_noalloc", _lib.dtype_code(t.dtype), agg, _lib.ptr(t), n, cols, _lib.ptr(out),
              _lib.stream_handle(t.device))
    return out


def test_noalloc_aggregate_matches_workspace_version_twice_in_a_row():
    g = torch.Generator().manual_seed(21)
    first = torch.randn(3_000_001, 5, generator=g, dtype=torch.float64).cuda()
    second = torch.randn(70_000, 64, generator=g).cuda()
    cases = [(first, _lib.AGG_SUM), (second, _lib.AGG_NORM)]
    got = [_aggregate_noalloc(t, agg) for t, agg in cases]          # two calls in a row
    want = [_aggregate_with_workspace(t, agg) for t, agg in cases]
    torch.cuda.synchronize()
    for a, b in zip(got, want):
        assert torch.equal(a, b)
    # and once more on the first input, after the second call left its
    # partials behind in the shared array
    again = _aggregate_noalloc(first, _lib.AGG_SUM)
    assert torch.equal(again, want[0])


def test_noalloc_aggregate_rejects_sizes_beyond_its_scratch():
    # one row of 100,000 columns needs 1.2 MB of partials: more than the 1 MiB array
    t = torch.zeros(1, 100_000, dtype=torch.float32, device="cuda")
    out = torch.empty(1, 100_000, dtype=torch.float32, device="cuda")
    status = _lib.lib().esr_aggregate_noalloc(_lib.F32, _lib.AGG_SUM, _lib.ptr(t), 1, 100_000, _lib.ptr(out),
                                              ctypes.c_void_p(_lib.stream_handle()))
    assert status == 1
    assert b"static array" in _lib.lib().esr_last_error()
