"""easier_gb300: the sparse-mesh hot path of EASIER on one GB300 (sm_103a).

Drop-in for the ``easier`` API on this path (``import easier_gb300 as esr``):
``Tensor``, ``Module``, ``Selector``, ``Reducer``, aggregators, data
factories, ``init``, ``compile(backend='cuda')`` and ``numeric`` (Linsys,
CG, GMRES, preconditioners).  Device work runs in hand-written sm_103a
kernels of ``libesr_gb300.so`` through its C ABI (``include/esr_gb300.h``).
"""
from .module import (Tensor, Module, Selector, Reducer, sum, prod, norm, max, min, hdf5, full, zeros, ones,
                     full_like, zeros_like, ones_like, arange)
from .jit import init, compile
from .utils import logger, EasierJitException
from . import numeric

__all__ = ["Tensor", "Module", "Selector", "Reducer", "sum", "prod", "norm", "max", "min", "hdf5", "full",
           "zeros", "ones", "full_like", "zeros_like", "ones_like", "arange", "init", "compile", "logger",
           "EasierJitException", "numeric"]
