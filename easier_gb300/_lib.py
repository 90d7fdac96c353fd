"""ctypes binding of ``libesr_gb300.so`` (declared in ``include/esr_gb300.h``).

The library is loaded once per process.  If it is missing or was built from
different sources, the import of any device op raises: there is no CPU
fallback for the device path.
"""
from __future__ import annotations

import ctypes
import os
import threading
from ctypes import POINTER, Structure, c_double, c_int, c_int32, c_int64, c_void_p, c_char_p
from pathlib import Path

from .utils import EasierJitException

F32, F64, I32, I64 = 0, 1, 2, 3
REDUCE_OPS = {"sum": 0, "prod": 1, "mean": 2, "amax": 3, "amin": 4}
AGG_SUM, AGG_PROD, AGG_NORM, AGG_MAX, AGG_MIN = 0, 1, 2, 3, 4
DEV_IDX_RANGE, DEV_NONFINITE, DEV_WAIT_TIMEOUT = 1, 2, 4

_LOCK = threading.Lock()
_LIB = None


class SweMesh(Structure):
    _fields_ = [("nc", c_int64), ("width", c_int32), ("dtype", c_int32),
                ("nbr", c_void_p), ("sx", c_void_p), ("sy", c_void_p),
                ("alpha", c_void_p), ("area", c_void_p), ("inv_area", c_void_p),
                ("exact", c_int32), ("pad_", c_int32)]


class SweTiles(Structure):
    _fields_ = [("nc", c_int64), ("ntiles", c_int32), ("dtype", c_int32), ("max_local", c_int32),
                ("max_l3", c_int32), ("max_own", c_int32), ("max_halo3", c_int32),
                ("meta", c_void_p), ("off3", c_void_p), ("offh", c_void_p), ("halo", c_void_p),
                ("slots", c_void_p), ("area", c_void_p), ("inv_area", c_void_p), ("exact", c_int32),
                ("slot_info", c_int32)]


SWE_TILE_AUTO, SWE_TILE_BLOCKED, SWE_TILE_PIPELINED = 0, 1, 2


class Sell(Structure):
    _fields_ = [("n", c_int64), ("nslots", c_int64), ("dtype", c_int32), ("pad_", c_int32),
                ("slice_ptr", c_void_p), ("col", c_void_p), ("val", c_void_p), ("diag", c_void_p)]


class CgScalars(Structure):
    _fields_ = [("rz", c_double), ("pq", c_double), ("alpha", c_double), ("beta", c_double),
                ("rr", c_double), ("bnorm", c_double), ("tol", c_double), ("rz_new", c_double),
                ("rz_prev", c_double), ("true_rr", c_double),
                ("iters", c_int32), ("done", c_int32), ("maxiter", c_int32), ("replacements", c_int32)]


class GmresScalars(Structure):
    _fields_ = [("rnorm", c_double), ("bnorm", c_double), ("tol", c_double), ("jend", c_int32),
                ("broken", c_int32), ("cycles", c_int32), ("pad_", c_int32)]


class Gnn(Structure):
    _fields_ = [("node_lk", c_void_p), ("edge_feat", c_void_p), ("inst_rows", c_void_p), ("h0", c_void_p),
                ("h1", c_void_p), ("enc_w", c_void_p), ("enc_b", c_void_p), ("layer_w", c_void_p),
                ("layer_b", c_void_p), ("dec_w", c_void_p), ("dec_b", ctypes.c_float), ("grid", c_int32),
                ("stall_window", c_int32), ("pad_", c_int32)]


class Batch(Structure):
    _fields_ = [("n", c_int64), ("ninst", c_int32), ("nblocks", c_int32), ("rows_per_block", c_int32),
                ("df64", c_int32), ("nchunks", c_int32), ("grid", c_int32), ("slice_ptr", c_void_p),
                ("col", c_void_p), ("val", c_void_p), ("diag", c_void_p), ("invdiag", c_void_p),
                ("val64", c_void_p), ("diag64", c_void_p), ("block_inst", c_void_p), ("inst_block0", c_void_p),
                ("chunk_tile0", c_void_p), ("chunk_inst", c_void_p), ("inst_chunk0", c_void_p),
                ("gnn", POINTER(Gnn)), ("poly_tmp", c_void_p), ("poly_degree", c_int32), ("pad_poly_", c_int32)]


class BcgInst(Structure):
    _fields_ = [("rz", c_double), ("pq", c_double), ("alpha", c_double), ("beta", c_double),
                ("rr", c_double), ("bnorm", c_double), ("tol", c_double), ("true_rr", c_double),
                ("sigma", c_double), ("rr_mark", c_double), ("rz_jac", c_double), ("theta", c_double),
                ("iters", c_int32), ("done", c_int32), ("verified", c_int32), ("restarts", c_int32),
                ("maxiter", c_int32), ("mode", c_int32), ("refresh", c_int32), ("fallbacks", c_int32),
                ("nrows", c_int32), ("gnn_iters", c_int32), ("clips", c_int32), ("clips_mark", c_int32),
                ("alpha_df", ctypes.c_float * 2), ("beta_df", ctypes.c_float * 2)]


_P = c_void_p
_SIGS = {
    "esr_last_error": (c_char_p, []),
    "esr_abi_version": (c_int, []),
    "esr_device_status": (c_int, [POINTER(c_int), c_int, _P]),
    "esr_mesh_sizes": (c_int, [c_int64, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]),
    "esr_mesh_triangular": (c_int, [c_int64, _P, _P, _P, _P, _P, _P]),
    "esr_swe_geometry": (c_int, [c_int64, c_int64, c_int64] + [_P] * 14),
    "esr_poisson_fv_assemble": (c_int, [c_int64, c_int64, c_int64] + [_P] * 11),
    "esr_mesh_triangular_device": (c_int, [c_int64] + [_P] * 7),
    "esr_swe_geometry_device": (c_int, [c_int64, c_int64, c_int64, c_int64] + [_P] * 15),
    "esr_poisson_fv_assemble_device": (c_int, [c_int64, c_int64, c_int64, c_int64] + [_P] * 16),
    "esr_p1_sizes": (c_int, [c_int64, POINTER(c_int64), POINTER(c_int64)]),
    "esr_p1_assemble": (c_int, [c_int64, _P, _P, _P, _P, _P]),
    "esr_csr_from_index": (c_int, [_P, c_int64, c_int64, _P, _P]),
    "esr_rcm_order": (c_int, [c_int64, c_int64, _P, _P, _P]),
    "esr_sell_build": (c_int, [c_int64, _P, _P, _P, c_int64, _P, _P, _P]),
    "esr_gather": (c_int, [_P, c_int64, c_int64, _P, c_int64, _P, _P]),
    "esr_segreduce": (c_int, [c_int, c_int, _P, c_int64, _P, _P, c_int64, _P, _P]),
    "esr_aggregate_workspace_bytes": (c_int64, [c_int64, c_int64]),
    "esr_aggregate": (c_int, [c_int, c_int, _P, c_int64, c_int64, _P, _P, _P]),
    "esr_aggregate_noalloc": (c_int, [c_int, c_int, _P, c_int64, c_int64, _P, _P]),
    "esr_dot_workspace_bytes": (c_int64, [c_int64]),
    "esr_dot": (c_int, [c_int, _P, _P, c_int64, _P, _P, _P]),
    "esr_swe_workspace_bytes": (c_int64, [POINTER(SweMesh)]),
    "esr_swe_step": (c_int, [POINTER(SweMesh), c_double, _P, c_int64, _P, _P]),
    "esr_swe_delta": (c_int, [POINTER(SweMesh), _P, _P, _P]),
    "esr_swe_tile_smem_bytes": (c_int64, [POINTER(SweTiles)]),
    "esr_swe_tile_threads": (c_int, [POINTER(SweTiles)]),
    "esr_swe_tile_step": (c_int, [POINTER(SweTiles), c_double, _P, _P, c_int64, _P]),
    "esr_swe_tile_kernel": (c_int, [POINTER(SweTiles)]),
    "esr_swe_tile_step_with": (c_int, [POINTER(SweTiles), c_int, c_double, _P, _P, c_int64, _P]),
    "esr_bisect_partition": (c_int, [c_int64, c_int64, _P, _P, c_int64, _P, _P]),
    "esr_swe_host_plan_create": (c_int, [POINTER(SweTiles), _P, _P, _P, _P, c_int32, POINTER(c_void_p)]),
    "esr_swe_host_step": (c_int, [_P, c_double, _P, c_int64, _P]),
    "esr_swe_host_plan_destroy": (c_int, [_P]),
    "esr_bisect_device_workspace_bytes": (c_int64, [c_int64, c_int64, c_int64]),
    "esr_bisect_partition_device": (c_int, [c_int64, c_int64, _P, _P, c_int64, _P, _P, _P, c_int64, _P]),
    "esr_swe_tile_layout": (c_int, [c_int64, _P, _P, c_int64, _P, POINTER(c_int64), POINTER(c_int64), _P, _P, _P,
                                    _P, _P, _P]),
    "esr_spmv": (c_int, [POINTER(Sell), _P, _P, _P]),
    "esr_cg_workspace_bytes": (c_int64, [c_int64]),
    "esr_cg_init": (c_int, [POINTER(Sell), _P, _P, _P, _P, _P, _P, c_double, c_double, c_int32, _P, _P]),
    "esr_cg_iterate": (c_int, [POINTER(Sell), _P, _P, _P, _P, _P, _P, c_int32, _P, _P]),
    "esr_cg_read_scalars": (c_int, [_P, POINTER(CgScalars), _P]),
    "esr_cg_mixed_init": (c_int, [POINTER(Sell), POINTER(Sell), _P, _P, _P, _P, _P, _P, _P, c_double, c_double,
                                  c_int32, _P, _P]),
    "esr_cg_mixed_iterate": (c_int, [POINTER(Sell), POINTER(Sell), _P, _P, _P, _P, _P, _P, _P, _P, c_int32, _P,
                                     _P]),
    "esr_true_residual": (c_int, [POINTER(Sell), _P, _P, _P, _P, _P, _P]),
    "esr_convert": (c_int, [c_int, _P, c_int, _P, c_int64, c_double, _P]),
    "esr_axpy_f64": (c_int, [_P, c_int, _P, c_double, c_int64, _P]),
    "esr_bcg_workspace_bytes": (c_int64, [c_int32, c_int32, c_int32]),
    "esr_bcg_init": (c_int, [POINTER(Batch), _P, _P, _P, _P, _P, _P, c_double, c_double, c_int32, _P, _P]),
    "esr_bcg_iterate": (c_int, [POINTER(Batch), _P, _P, _P, _P, _P, c_int32, _P, _P]),
    "esr_bcg_verify": (c_int, [POINTER(Batch), _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "esr_bcg_status": (c_int, [_P, c_int32, c_int32, POINTER(c_int32), POINTER(BcgInst), _P]),
    "esr_gnn_apply": (c_int, [POINTER(Batch), _P, _P, _P, _P]),
    "esr_bcg_graph_create": (c_int, [POINTER(Batch), _P, _P, _P, _P, _P, _P, _P, _P, _P, c_double, c_double, c_int32,
                                     c_int32, _P, POINTER(c_void_p)]),
    "esr_bcg_graph_launch": (c_int, [_P, _P]),
    "esr_bcg_graph_destroy": (c_int, [_P]),
    "esr_wait_selftest": (c_int, [c_int32, _P, _P]),
    "esr_gmres_workspace_bytes": (c_int64, [c_int64, c_int32]),
    "esr_gmres_init": (c_int, [POINTER(Sell), _P, c_double, c_double, _P, _P]),
    "esr_gmres_residual": (c_int, [POINTER(Sell), _P, _P, _P, _P, _P]),
    "esr_gmres_cycle": (c_int, [POINTER(Sell), _P, _P, _P, _P, _P, _P, c_int32, _P, _P]),
    "esr_gmres_read": (c_int, [_P, POINTER(GmresScalars), _P]),
}

ABI_VERSION = 11


def library_path() -> Path:
    return Path(__file__).resolve().parent / "libesr_gb300.so"


def lib():
    """The loaded library; builds it first when it is absent or stale."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = library_path()
        if os.environ.get("EASIER_GB300_NO_BUILD") != "1":
            from . import _build
            path = _build.build()
        if not path.exists():
            raise EasierJitException(
                f"native library {path} is missing; run `python -c 'import __graft_entry__ as g; g.build()'`")
        handle = ctypes.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        if handle.esr_abi_version() != ABI_VERSION:
            raise EasierJitException("libesr_gb300.so ABI version mismatch; rebuild it")
        _LIB = handle
        return _LIB


def exported_symbols():
    return list(_SIGS.keys())


def check(status: int, what: str = "") -> None:
    """Raise on a non-zero status from the library."""
    if status != 0:
        msg = lib().esr_last_error()
        msg = msg.decode() if msg else ""
        kinds = {1: ValueError, 2: RuntimeError, 3: RuntimeError, 4: NotImplementedError}
        raise kinds.get(status, RuntimeError)(f"{what}: {msg}" if what else msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args), name)


def ptr(t) -> int:
    """Device or host address of a torch tensor / numpy array (None -> NULL)."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def stream_handle(device=None) -> int:
    import torch
    return torch.cuda.current_stream(device).cuda_stream


def dtype_code(dtype) -> int:
    import torch
    m = {torch.float32: F32, torch.float64: F64, torch.int32: I32, torch.int64: I64}
    if dtype not in m:
        raise NotImplementedError(f"dtype {dtype} is not supported by the GB300 path")
    return m[dtype]
