"""ctypes binding of the native library (lfg/liblfg.so, C ABI in include/lfg.h).

The library is the product: every transform runs in its CUDA kernels.  If it is missing,
loading fails with an error that says how to build it; nothing falls back to a CPU or
library FFT.
"""
from __future__ import annotations

import ctypes
import os
from functools import lru_cache

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblfg.so")

LFG_OK = 0
LFG_ERR_UNSUPPORTED = 1
LFG_ERR_INVALID = 2
LFG_ERR_CUDA = 3
LFG_ERR_NOMEM = 4
LFG_ERR_TIMEOUT = 5

LFG_F64 = 0
LFG_F32 = 1

LFG_ESTIMATE = 0
LFG_MEASURE = 1
LFG_ADJOINT = 8
LFG_NO_COMPENSATION = 16
LFG_TEST_WAIT_GIVE_UP = 32
LFG_PER_SIZE_CONCURRENT = 64
LFG_GENERIC_KERNELS = 128


class PlanInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("howmany", ctypes.c_int64), ("sign", ctypes.c_int),
                ("precision", ctypes.c_int), ("npass", ctypes.c_int), ("ngroups", ctypes.c_int),
                ("radices", ctypes.c_int * 24), ("in_bytes", ctypes.c_int64),
                ("out_bytes", ctypes.c_int64), ("flops", ctypes.c_double),
                ("cluster_ctas", ctypes.c_int), ("direct_groups", ctypes.c_int),
                ("small_kernel", ctypes.c_int)]


class LfgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"lfg status {status}: {msg}")
        self.status = status


class Unsupported(LfgError):
    pass


# (name, restype, argtypes) of every entry point declared in include/lfg.h
_VP = ctypes.c_void_p
_SIG = {
    "lfg_plan_spec": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.c_size_t, ctypes.c_int,
                                      ctypes.c_uint, ctypes.POINTER(_VP)]),
    "lfg_plan_1d": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, ctypes.c_int,
                                    ctypes.c_uint, ctypes.POINTER(_VP)]),
    "lfg_plan_1d_radices": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t,
                                            ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                            ctypes.POINTER(_VP)]),
    "lfg_plan_r2r": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, ctypes.c_int,
                                    ctypes.c_uint, ctypes.POINTER(ctypes.c_void_p)]),
    "lfg_plan_r2c": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint,
                                     ctypes.POINTER(_VP)]),
    "lfg_plan_c2r": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint,
                                     ctypes.POINTER(_VP)]),
    "lfg_plan_r2c_2d": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t,
                                        ctypes.c_int, ctypes.c_uint, ctypes.POINTER(_VP)]),
    "lfg_plan_c2r_2d": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t,
                                        ctypes.c_int, ctypes.c_uint, ctypes.POINTER(_VP)]),
    "lfg_set_scale": (ctypes.c_int, [_VP, ctypes.c_double]),
    "lfg_execute": (ctypes.c_int, [_VP, _VP, _VP, _VP]),
    "lfg_execute_host": (ctypes.c_int, [_VP, _VP, _VP]),
    "lfg_destroy": (None, [_VP]),
    "lfg_device_status": (ctypes.c_int, [_VP]),
    "lfg_get_plan_info": (ctypes.c_int, [_VP, ctypes.POINTER(PlanInfo)]),
    "lfg_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "lfg_last_error": (ctypes.c_char_p, []),
    "lfg_cos_sin_table": (ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)]),
    "lfg_shard_ragged": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64), ctypes.c_size_t,
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_double)]),
    "lfg_plan_layout": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "lfg_wisdom_import": (ctypes.c_int, [ctypes.c_char_p]),
    "lfg_wisdom_export": (ctypes.c_int, [ctypes.c_char_p]),
    "lfg_wisdom_forget": (None, []),
    "lfg_wisdom_count": (ctypes.c_size_t, []),
}


@lru_cache(maxsize=1)
def lib() -> ctypes.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"native library {LIB_PATH} is missing: build it with "
                          f"`python -c 'import __graft_entry__ as g; g.build()'` "
                          f"or `python -m lfg.build` in lean-fftw_gb300/")
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIG.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def check(status: int) -> None:
    if status == LFG_OK:
        return
    msg = lib().lfg_last_error().decode(errors="replace")
    if status == LFG_ERR_UNSUPPORTED:
        raise Unsupported(status, msg)
    raise LfgError(status, msg)
