"""Ragged batches: many 1-D complex transforms of different 13-smooth sizes, one launch.

`plan_ragged(sizes)` plans the whole batch once (see include/lfg.h, lfg_plan_ragged); its
`execute` replays a CUDA graph of one persistent kernel.  `per_size=True` builds the
comparison point instead: one batched launch per distinct size.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Optional, Sequence

import numpy as np

from ._lib import LFG_F64, LFG_MEASURE, check, lib

LFG_PER_SIZE = 2
LFG_PER_SIZE_CONCURRENT = 64
LFG_NO_GRAPH = 4


class RaggedInfo(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int64), ("classes", ctypes.c_int64), ("items", ctypes.c_int64),
                ("grid", ctypes.c_int64), ("smem_bytes", ctypes.c_int64),
                ("launches", ctypes.c_int64), ("in_bytes", ctypes.c_int64),
                ("out_bytes", ctypes.c_int64), ("points", ctypes.c_int64),
                ("flops", ctypes.c_double), ("tile_target", ctypes.c_int64),
                ("single_max", ctypes.c_int64), ("block_shape", ctypes.c_int64)]


class RaggedTuning(ctypes.Structure):
    _fields_ = [("tile_target", ctypes.c_int64), ("single_max", ctypes.c_int64),
                ("n_over", ctypes.c_int), ("over_n", ctypes.POINTER(ctypes.c_int64)),
                ("over_npass", ctypes.POINTER(ctypes.c_int)),
                ("over_radices", ctypes.POINTER(ctypes.c_int)), ("block_shape", ctypes.c_int)]


_VP = ctypes.c_void_p
_I64P = ctypes.POINTER(ctypes.c_int64)


def _bind():
    L = lib()
    if getattr(L, "_ragged_bound", False):
        return L
    L.lfg_plan_ragged.restype = ctypes.c_int
    L.lfg_plan_ragged.argtypes = [_I64P, ctypes.c_size_t, _I64P, _I64P, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_uint, ctypes.POINTER(RaggedTuning), ctypes.POINTER(_VP)]
    L.lfg_execute_ragged.restype = ctypes.c_int
    L.lfg_execute_ragged.argtypes = [_VP, _VP, _VP, _VP]
    L.lfg_execute_ragged_host.restype = ctypes.c_int
    L.lfg_execute_ragged_host.argtypes = [_VP, _VP, _VP]
    L.lfg_destroy_ragged.restype = None
    L.lfg_destroy_ragged.argtypes = [_VP]
    L.lfg_get_ragged_info.restype = ctypes.c_int
    L.lfg_get_ragged_info.argtypes = [_VP, ctypes.POINTER(RaggedInfo)]
    L.lfg_get_ragged_radices.restype = ctypes.c_int
    L.lfg_get_ragged_radices.argtypes = [_VP, ctypes.c_int64, ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int)]
    L._ragged_bound = True
    return L


class RaggedPlan:
    def __init__(self, handle, sizes, in_offsets, out_offsets):
        self._h = handle
        self.sizes = sizes
        self.in_offsets = in_offsets
        self.out_offsets = out_offsets

    def info(self) -> RaggedInfo:
        i = RaggedInfo()
        check(_bind().lfg_get_ragged_info(self._h, ctypes.byref(i)))
        return i

    def radices(self, n: int):
        arr = (ctypes.c_int * 24)()
        np_ = ctypes.c_int()
        check(_bind().lfg_get_ragged_radices(self._h, n, arr, ctypes.byref(np_)))
        return list(arr[: np_.value])

    def execute(self, inp, out, stream=None):
        import torch
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        elif hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        check(_bind().lfg_execute_ragged(self._h, _VP(inp.data_ptr()), _VP(out.data_ptr()),
                                         _VP(stream)))
        return out

    def execute_host(self, inp: np.ndarray, out: np.ndarray) -> np.ndarray:
        check(_bind().lfg_execute_ragged_host(self._h, _VP(inp.ctypes.data), _VP(out.ctypes.data)))
        return out

    def destroy(self):
        if self._h:
            _bind().lfg_destroy_ragged(self._h)
            self._h = _VP(0)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def plan_ragged(sizes: Sequence[int], sign: int = -1, in_offsets=None, out_offsets=None,
                per_size: bool = False, graph: bool = True, measure: bool = False,
                concurrent: bool = False,
                tile_target: int = 0, single_max: int = 0, block_shape: int = 0,
                radices: Optional[Dict[int, Sequence[int]]] = None) -> RaggedPlan:
    L = _bind()
    s = np.ascontiguousarray(sizes, dtype=np.int64)
    io = None if in_offsets is None else np.ascontiguousarray(in_offsets, dtype=np.int64)
    oo = None if out_offsets is None else np.ascontiguousarray(out_offsets, dtype=np.int64)
    flags = (LFG_PER_SIZE if per_size else 0) | (0 if graph else LFG_NO_GRAPH) | \
            (LFG_MEASURE if measure else 0) | (LFG_PER_SIZE_CONCURRENT if concurrent else 0)
    tun = RaggedTuning(tile_target, single_max, 0, None, None, None, block_shape)
    keep = []
    if radices:
        ns = np.array(list(radices.keys()), dtype=np.int64)
        npass = np.array([len(radices[n]) for n in ns], dtype=np.int32)
        rad = np.zeros(24 * len(ns), dtype=np.int32)
        for j, n in enumerate(ns):
            rad[24 * j: 24 * j + len(radices[n])] = radices[n]
        keep = [ns, npass, rad]
        tun.n_over = len(ns)
        tun.over_n = ns.ctypes.data_as(_I64P)
        tun.over_npass = npass.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        tun.over_radices = rad.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    h = _VP()
    check(L.lfg_plan_ragged(s.ctypes.data_as(_I64P), s.size,
                            None if io is None else io.ctypes.data_as(_I64P),
                            None if oo is None else oo.ctypes.data_as(_I64P),
                            sign, LFG_F64, flags, ctypes.byref(tun), ctypes.byref(h)))
    del keep
    if io is None:
        io = np.concatenate([[0], np.cumsum(s)[:-1]]).astype(np.int64) if s.size else s
    if oo is None:
        oo = np.concatenate([[0], np.cumsum(s)[:-1]]).astype(np.int64) if s.size else s
    return RaggedPlan(h, s, io, oo)


def smooth13_sizes(lo: int = 2, hi: int = 16384) -> np.ndarray:
    out = []
    for n in range(lo, hi + 1):
        m = n
        for p in (2, 3, 5, 7, 11, 13):
            while m % p == 0:
                m //= p
        if m == 1:
            out.append(n)
    return np.array(out, dtype=np.int64)


def ragged_sizes(count: int = 8192, seed: int = 20261016, lo: int = 2, hi: int = 16384) -> np.ndarray:
    """Sizes drawn log-uniformly from [lo, hi] and snapped to the nearest 13-smooth integer
    in log distance (ties to the smaller): u ~ U[ln lo, ln hi) from numpy default_rng(seed)."""
    S = smooth13_sizes(lo, hi)
    L = np.log(S.astype(np.float64))
    u = np.random.default_rng(seed).uniform(np.log(lo), np.log(hi), count)
    i = np.clip(np.searchsorted(L, u), 1, len(S) - 1)
    left = u - L[i - 1] <= L[i] - u
    return np.where(left, S[i - 1], S[i]).astype(np.int64)


def shard_ragged(sizes: Sequence[int], nshards: int):
    """Split a ragged batch over `nshards` devices (lfg_shard_ragged): returns (shard, cost),
    shard[i] the device of transform i, cost[s] the codelet operations of device s.  The
    split balances those operations, largest transforms first, and is deterministic, so every
    rank of a job computes the same one; rank r then plans `sizes[shard == r]`."""
    s = np.ascontiguousarray(sizes, dtype=np.int64)
    shard = np.empty(s.size, dtype=np.int32)
    cost = np.empty(int(nshards), dtype=np.float64)
    check(lib().lfg_shard_ragged(s.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), s.size,
                                 int(nshards), shard.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                 cost.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return shard, cost
