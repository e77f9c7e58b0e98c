"""Python mirror of lean-fftw's plan/execute interface over the native library.

lean-fftw exposes two entry-point families (LeanFFTW/FFI.lean:50-58,
LeanFFTW/Asm/Planner.lean:293-306, bench/backends/bench-leanfftw.c:225-291):

    lfftw_generic_plan(spec) -> plan | none      lfftw_generic_exec(plan, in, out)
    lfa_plan_measure(N, fwd, in, out) -> plan    lfa_call(plan, in, out)

Here `plan_spec(spec)` and `plan_measure(n, fwd)` return a `Plan`, and `Plan.execute`
runs it on device tensors (torch, on the current stream) or `Plan.execute_host` on host
arrays (numpy).  Unsupported problems raise `Unsupported` and never compute a different
transform (lean-fftw docs/CONTRACT.md:44-45).
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import LFG_ESTIMATE, LFG_F32, LFG_F64, LFG_MEASURE, PlanInfo, check, lib


class Plan:
    """An executable plan (owns device twiddle tables; release with `destroy` or GC)."""

    def __init__(self, handle: ctypes.c_void_p):
        self._h = handle

    @property
    def handle(self) -> int:
        return self._h.value

    def set_scale(self, scale: float) -> "Plan":
        """Multiply the outputs by `scale` inside the kernel (complex plans)."""
        check(lib().lfg_set_scale(self._h, float(scale)))
        return self

    def info(self) -> PlanInfo:
        pi = PlanInfo()
        check(lib().lfg_get_plan_info(self._h, ctypes.byref(pi)))
        return pi

    @property
    def radices(self):
        i = self.info()
        return [i.radices[k] for k in range(i.npass)]

    def execute(self, inp, out=None, stream=None):
        """Run on device buffers.  `inp`/`out` are torch CUDA tensors (or raw device
        addresses); the work is enqueued on `stream` (default: torch's current stream)."""
        import torch
        if out is None:
            out = torch.empty_like(inp)   # complex transforms; real ones must pass `out`
        ip = inp.data_ptr() if hasattr(inp, "data_ptr") else int(inp)
        op = out.data_ptr() if hasattr(out, "data_ptr") else int(out)
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        elif hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        check(lib().lfg_execute(self._h, ctypes.c_void_p(ip), ctypes.c_void_p(op),
                                ctypes.c_void_p(stream)))
        return out

    def execute_host(self, inp: np.ndarray, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Run on host arrays (copies in and out around the kernels, synchronous)."""
        if out is None:
            out = np.empty_like(inp)
        assert inp.flags.c_contiguous and out.flags.c_contiguous
        check(lib().lfg_execute_host(self._h, ctypes.c_void_p(inp.ctypes.data),
                                     ctypes.c_void_p(out.ctypes.data)))
        return out

    def destroy(self) -> None:
        if self._h:
            lib().lfg_destroy(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def _prec(precision) -> int:
    if precision in (LFG_F64, "f64", "float64", np.float64, np.complex128):
        return LFG_F64
    if precision in (LFG_F32, "f32", "float32", np.float32, np.complex64):
        return LFG_F32
    raise ValueError(f"unknown precision {precision!r}")


def plan_1d(n: int, sign: int = -1, howmany: int = 1, precision="f64",
            radices: Optional[Sequence[int]] = None, measure: bool = False,
            compensated: bool = True, generic_kernels: bool = False) -> Plan:
    """1-D complex transform of size n on `howmany` contiguous lines.  Binary32 plans of
    size >= 2^16 use compensated twiddle products in their last passes unless
    compensated=False."""
    h = ctypes.c_void_p()
    if radices is not None:
        arr = (ctypes.c_int * len(radices))(*[int(r) for r in radices])
        check(lib().lfg_plan_1d_radices(n, sign, howmany, _prec(precision), arr, len(radices),
                                        ctypes.byref(h)))
    else:
        flags = (LFG_MEASURE if measure else LFG_ESTIMATE) | (0 if compensated else 16) | \
            (128 if generic_kernels else 0)
        check(lib().lfg_plan_1d(n, sign, howmany, _prec(precision), flags, ctypes.byref(h)))
    return Plan(h)


def plan_r2c(n: int, howmany: int = 1, precision="f64", adjoint: bool = False,
             generic_kernels: bool = False) -> Plan:
    """Real forward transform of even size n on `howmany` contiguous lines: n doubles in,
    n/2+1 complex out per line (the generic engine's r2c, Core/Problem.lean:145-147).
    adjoint=True doubles output bins 1..n/2-1: the gradient of c2r.  generic_kernels: run
    the kernels with runtime pass descriptors (the same bits)."""
    h = ctypes.c_void_p()
    flags = (_lib.LFG_ADJOINT if adjoint else 0) | (_lib.LFG_GENERIC_KERNELS if generic_kernels else 0)
    check(lib().lfg_plan_r2c(n, howmany, _prec(precision), flags, ctypes.byref(h)))
    return Plan(h)


def plan_c2r(n: int, howmany: int = 1, precision="f64", adjoint: bool = False) -> Plan:
    """Backward transform of a half spectrum (n/2+1 complex per line) to n reals
    (Core/Problem.lean:148-150): unnormalised, imaginary parts of bins 0 and n/2 ignored.
    adjoint=True halves input bins 1..n/2-1: the gradient of r2c."""
    h = ctypes.c_void_p()
    check(lib().lfg_plan_c2r(n, howmany, _prec(precision), _lib.LFG_ADJOINT if adjoint else 0,
                             ctypes.byref(h)))
    return Plan(h)


R2R_KINDS = {"r2hc": 0, "hc2r": 1, "dht": 2, "redft00": 3, "redft01": 4, "redft10": 5,
             "redft11": 6, "rodft00": 7, "rodft01": 8, "rodft10": 9, "rodft11": 10}


def plan_r2r(n: int, kind, howmany: int = 1, precision="f64") -> Plan:
    """Real-to-real transform of one of the eleven kinds (name or libbench2 number) on
    `howmany` contiguous lines of n reals (Core/Problem.lean:64-112, 151-163)."""
    k = R2R_KINDS[kind.lower()] if isinstance(kind, str) else int(kind)
    h = ctypes.c_void_p()
    check(lib().lfg_plan_r2r(n, k, howmany, _prec(precision), 0, ctypes.byref(h)))
    return Plan(h)


def plan_r2c_2d(n0: int, n1: int, howmany: int = 1, precision="f64",
                generic_kernels: bool = False) -> Plan:
    """Rank-2 r2c of n0 x n1 real images to n0 x (n1/2+1) complex (Core/Problem.lean:228-233).
    generic_kernels: run the kernels with runtime pass descriptors (the same bits)."""
    h = ctypes.c_void_p()
    check(lib().lfg_plan_r2c_2d(n0, n1, howmany, _prec(precision),
                                _lib.LFG_GENERIC_KERNELS if generic_kernels else 0, ctypes.byref(h)))
    return Plan(h)


def plan_c2r_2d(n0: int, n1: int, howmany: int = 1, precision="f64",
                generic_kernels: bool = False) -> Plan:
    """Rank-2 c2r: complex backward along the first axis, then c2r along the last."""
    h = ctypes.c_void_p()
    check(lib().lfg_plan_c2r_2d(n0, n1, howmany, _prec(precision),
                                _lib.LFG_GENERIC_KERNELS if generic_kernels else 0, ctypes.byref(h)))
    return Plan(h)


def plan_measure(n: int, fwd: bool, howmany: int = 1) -> Plan:
    """lfa_plan_measure analogue (LeanFFTW/Asm/Planner.lean:293-302)."""
    return plan_1d(n, -1 if fwd else 1, howmany, measure=True)


def plan_spec(spec: Sequence[float], precision="f64", measure: bool = False) -> Plan:
    """lfftw_generic_plan analogue (LeanFFTW/FFI.lean:50-52): spec in the FFI encoding
    [kind, sign, rank, vrank, inRe, inIm, outRe, outIm, (n,is,os) x rank, (n,is,os) x vrank,
    r2rkind x rank]."""
    a = np.ascontiguousarray(spec, dtype=np.float64)
    h = ctypes.c_void_p()
    check(lib().lfg_plan_spec(a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), a.size,
                              _prec(precision), LFG_MEASURE if measure else LFG_ESTIMATE,
                              ctypes.byref(h)))
    return Plan(h)


def cos_sin_table(n: int) -> np.ndarray:
    """Trig.cosSin2PiTable n (LeanFFTW/Core/Trig.lean:131-134) as an (n, 2) array."""
    out = np.empty(2 * n, dtype=np.float64)
    check(lib().lfg_cos_sin_table(n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return out.reshape(n, 2)


def wisdom_import(path: str) -> None:
    """Merge the tuning-cache entries of a file (lfg_wisdom_import)."""
    check(lib().lfg_wisdom_import(str(path).encode()))


def wisdom_export(path: str) -> None:
    """Write every tuning-cache entry to a file (lfg_wisdom_export)."""
    check(lib().lfg_wisdom_export(str(path).encode()))


def wisdom_forget() -> None:
    """Empty the process's tuning cache (lfg_wisdom_forget)."""
    lib().lfg_wisdom_forget()


def wisdom_count() -> int:
    """Entries held in the process's tuning cache (lfg_wisdom_count)."""
    return int(lib().lfg_wisdom_count())


def plan_layout(n: int, precision="f64"):
    """(radices, passes in the first pass group) of a default 1-D plan of size n, computed on
    the host (lfg_plan_layout); the first group holds every pass when the plan has one group."""
    rs = (ctypes.c_int * 24)()
    npass, first = ctypes.c_int(), ctypes.c_int()
    check(lib().lfg_plan_layout(int(n), _prec(precision), rs, ctypes.byref(npass),
                                ctypes.byref(first)))
    return [rs[i] for i in range(npass.value)], first.value
