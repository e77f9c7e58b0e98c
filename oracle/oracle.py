"""ORACLE (test infrastructure only): Python front end of the CPU restatements.

What is here, and the reference code each piece follows (paths inside lean-fftw):

* `ref_transform`      refTransform / stockhamWith / passWith (Gen/Stockham.lean:263-301):
                       the binary64 Stockham passes the reference's fast engine reproduces
                       bit for bit; twiddle tables from `trig_ref` (Core/Trig.lean:131-134,
                       Core/FastPlan.lean:163-183).
* `generic_dft`        the generic engine, exec floatOps (mkPlan floatOps fwd
                       (primeFactors n)) (Core/Alg.lean:236-254, Core/Problem.lean:126-127).
* `generic_r2c/c2r`    LineOp.apply for r2c and c2r (Core/Problem.lean:142-150, hermExt :137).
* `generic_rank2_r2c`  planProblemCore for rdft2 forward, rank 2 (Core/Problem.lean:228-233):
                       r2c along the last axis, then a complex forward DFT along the first.
* `r2r_embed/extract`  R2RKind.embedSize / embed / extract and the hc2r branch of
                       LineOp.apply (Core/Problem.lean:64-112, 151-163): exact index maps;
                       `generic_r2r` (the generic engine's r2r), `fast_r2r` (the same
                       embedding around refTransform: what the GPU computes, bit for bit),
                       `dd_r2r` (extended precision).
* `dd_dft`             extended-precision (double-double) DFT: the accuracy oracle.
* `lcg_rand`           randArr of scripts/AsmTest.lean:7-13, the reference tests' inputs.
* `bfly`               one butterfly of the oracle: radices 2, 4, 8 and 16 are lean-fftw's own
                       generated kernels (LeanFFTW/Native/Kernels.lean, via native_dag.py).

The reference engine itself cannot run here: it needs a Lean 4.35 toolchain (absent, no
network) and AVX-512 (absent on aarch64 hosts).  Parity is pinned instead through the
reference's published known answers and generated kernels (tests/test_oracle.py,
tests/test_codegen_pins.py, tests/test_native_kernels.py).

Only tests, the smoke check and the CPU-baseline leg of the benchmark may import this module.
"""
from __future__ import annotations

import ctypes
import os
import sys
from functools import lru_cache
from typing import List, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import trig_ref  # noqa: E402

_dp = ctypes.POINTER(ctypes.c_double)


@lru_cache(maxsize=1)
def lib() -> ctypes.CDLL:
    so = os.path.join(HERE, "_build", "liboracle.so")
    if not os.path.exists(so):
        import build_oracle
        build_oracle.build()
    L = ctypes.CDLL(so)
    L.lfo_ref_transform.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.POINTER(ctypes.c_int),
                                    ctypes.c_int, ctypes.POINTER(_dp), _dp, _dp, ctypes.c_long,
                                    ctypes.c_int]
    L.lfo_ref_transform.restype = ctypes.c_int
    L.lfo_generic_dft.argtypes = [ctypes.c_int, ctypes.c_long, _dp, _dp, ctypes.c_long,
                                  ctypes.c_long, _dp, ctypes.c_long, ctypes.c_long,
                                  ctypes.c_long, ctypes.c_int]
    L.lfo_generic_dft.restype = ctypes.c_int
    L.lfo_dd_dft.argtypes = [ctypes.c_int, ctypes.c_long, _dp, _dp, ctypes.c_long, ctypes.c_long,
                             _dp, _dp, ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_int]
    L.lfo_dd_dft.restype = ctypes.c_int
    L.lfo_ref_ragged.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.POINTER(ctypes.c_long),
                                 ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_long, ctypes.POINTER(ctypes.c_long),
                                 ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long),
                                 _dp, _dp, ctypes.c_int]
    L.lfo_ref_ragged.restype = ctypes.c_int
    L.lfo_rel_l2.argtypes = [_dp, _dp, _dp, ctypes.c_long]
    L.lfo_rel_l2.restype = ctypes.c_double
    L.lfo_cos_sin_table.argtypes = [ctypes.c_uint64, _dp]
    L.lfo_cos_sin_table.restype = ctypes.c_int
    L.lfo_bfly.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]
    L.lfo_bfly.restype = ctypes.c_int
    return L


def _p(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def bfly(fwd: bool, R: int, tw: bool, x: np.ndarray, native: bool = True) -> np.ndarray:
    """One radix-R butterfly of the oracle on x (2R data values, then 2(R-1) twiddle values
    when tw): lean-fftw's generated kernel (native, radices 2/4/8/16) or the restated
    generator's (other radices)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    assert x.size == (4 * R - 2 if tw else 2 * R)
    y = np.empty(2 * R, dtype=np.float64)
    if lib().lfo_bfly(int(fwd), R, int(tw), int(native), _p(x), _p(y)) != 0:
        raise ValueError(f"no oracle butterfly for radix {R}")
    return y


def nthreads_default() -> int:
    return max(1, min(os.cpu_count() or 1, 16))


# ------------------------------------------------------------------ twiddles

def pass_ns(rs: Sequence[int], t: int) -> int:
    """Product of the radices before pass t (FastPlan.lean:158)."""
    p = 1
    for r in rs[:t]:
        p *= r
    return p


@lru_cache(maxsize=4096)
def table(n: int) -> np.ndarray:
    """cosSin2PiTable n (Trig.lean:131-134) as an (n, 2) array, from the oracle's C
    restatement (trig_ref.c; checked against trig_ref.py in the tests)."""
    out = np.empty(2 * n, dtype=np.float64)
    assert lib().lfo_cos_sin_table(n, _p(out)) == 0
    return out.reshape(n, 2)


def pass_twiddles(tab: np.ndarray, fwd: bool, N: int, R: int, ns: int) -> np.ndarray:
    """FastPlan.lean:163-173 on a table array: for r = 1..R-1 the ns real parts then the ns
    imaginary parts of tab[r*k*N/(ns*R)], imaginary negated (never to -0.0) when fwd."""
    step = N // (ns * R)
    k = np.arange(ns)
    rows = []
    for r in range(1, R):
        t = tab[r * k * step]
        im = t[:, 1]
        if fwd:
            im = np.where(im == 0.0, 0.0, -im)
        rows += [t[:, 0], im]
    return np.ascontiguousarray(np.concatenate(rows)) if rows else np.zeros(0)


@lru_cache(maxsize=4096)
def _plan_twiddles(fwd: bool, N: int, rs: tuple):
    tab = table(N)
    out = [np.zeros(1)]
    for t in range(1, len(rs)):
        out.append(pass_twiddles(tab, fwd, N, rs[t], pass_ns(rs, t)))
    return out


def plan_twiddles(fwd: bool, N: int, rs: Sequence[int]) -> List[np.ndarray]:
    """Twiddle table of every pass t >= 1 (entry 0 unused)."""
    return _plan_twiddles(bool(fwd), int(N), tuple(int(r) for r in rs))


def _tab_array(n: int) -> np.ndarray:
    return table(n).reshape(-1)


@lru_cache(maxsize=64)
def _dd_tab_array(n: int) -> np.ndarray:
    return np.ascontiguousarray(np.array(trig_ref.dd_table(n), dtype=np.float64).reshape(-1))


# ------------------------------------------------------------------ transforms

def _as_batch(x: np.ndarray, N: int) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.complex128)
    return x.reshape(-1, N)


def ref_transform(fwd: bool, N: int, rs: Sequence[int], x: np.ndarray,
                  nthreads: int = 1) -> np.ndarray:
    """refTransform fwd N rs on each row of x (complex128, last axis N)."""
    rs = [int(r) for r in rs]
    assert int(np.prod(rs)) == N, (N, rs)
    shape = x.shape
    xb = _as_batch(x, N)
    out = np.empty_like(xb)
    tws = plan_twiddles(fwd, N, rs)
    arr = (_dp * len(rs))(*[_p(t) for t in tws])
    rsa = (ctypes.c_int * len(rs))(*rs)
    xin = xb.view(np.float64)
    xo = out.view(np.float64)
    rc = lib().lfo_ref_transform(int(fwd), N, rsa, len(rs), arr, _p(xin), _p(xo), xb.shape[0],
                                 nthreads)
    assert rc == 0, "reference transform failed (radix without a codelet?)"
    return out.reshape(shape)


class RaggedRef:
    """refTransform over a ragged batch in one C call (one transform per thread): sizes[i]
    with radices plans[sizes[i]], data at complex offsets in_off[i] / out_off[i]."""

    def __init__(self, fwd: bool, sizes, plans, in_off, out_off):
        self.fwd = bool(fwd)
        classes = sorted(set(int(n) for n in sizes))
        idx = {n: c for c, n in enumerate(classes)}
        self.cN = (ctypes.c_long * len(classes))(*classes)
        self.cnp = (ctypes.c_int * len(classes))(*[len(plans[n]) for n in classes])
        self._rs = [(ctypes.c_int * len(plans[n]))(*plans[n]) for n in classes]
        self.crs = (ctypes.POINTER(ctypes.c_int) * len(classes))(
            *[ctypes.cast(a, ctypes.POINTER(ctypes.c_int)) for a in self._rs])
        self._tw = [plan_twiddles(fwd, n, plans[n]) for n in classes]
        self._twp = [(_dp * len(t))(*[_p(a) for a in t]) for t in self._tw]
        self.ctw = (ctypes.POINTER(_dp) * len(classes))(
            *[ctypes.cast(a, ctypes.POINTER(_dp)) for a in self._twp])
        self.ncls = len(classes)
        self.count = len(sizes)
        self.cls = (ctypes.c_long * len(sizes))(*[idx[int(n)] for n in sizes])
        self.ioff = (ctypes.c_long * len(sizes))(*[int(v) for v in in_off])
        self.ooff = (ctypes.c_long * len(sizes))(*[int(v) for v in out_off])

    def run(self, x: np.ndarray, out: np.ndarray, nthreads: int = 1) -> np.ndarray:
        rc = lib().lfo_ref_ragged(int(self.fwd), self.ncls, self.cN, self.cnp, self.crs,
                                  self.ctw, self.count, self.cls, self.ioff, self.ooff,
                                  _p(x.view(np.float64)), _p(out.view(np.float64)), nthreads)
        assert rc == 0
        return out


def generic_dft(fwd: bool, x: np.ndarray, nthreads: int = 1) -> np.ndarray:
    """The generic engine's 1-D DFT along the last axis."""
    N = x.shape[-1]
    xb = _as_batch(x, N)
    out = np.empty_like(xb)
    lib().lfo_generic_dft(int(fwd), N, _p(_tab_array(N)), _p(xb.view(np.float64)), 1, N,
                          _p(out.view(np.float64)), 1, N, xb.shape[0], nthreads)
    return out.reshape(x.shape)


def dd_dft(fwd: bool, x: np.ndarray, nthreads: int = 1):
    """Double-double DFT along the last axis: returns (hi, lo) complex128 arrays whose sum
    is the transform to about 106 bits."""
    N = x.shape[-1]
    xb = _as_batch(x, N)
    hi = np.empty_like(xb)
    lo = np.empty_like(xb)
    lib().lfo_dd_dft(int(fwd), N, _p(_dd_tab_array(N)), _p(xb.view(np.float64)), 1, N,
                     _p(hi.view(np.float64)), _p(lo.view(np.float64)), 1, N, xb.shape[0],
                     nthreads)
    return hi.reshape(x.shape), lo.reshape(x.shape)


def rel_l2(y: np.ndarray, ref) -> float:
    """Relative L2 error ||y - ref|| / ||ref||, ref = (hi, lo) double-double or an array."""
    if isinstance(ref, tuple):
        hi, lo = ref
    else:
        hi, lo = ref, np.zeros_like(ref)
    yv = np.ascontiguousarray(y).reshape(-1).view(np.float64) if np.iscomplexobj(y) else \
        np.ascontiguousarray(y, dtype=np.float64).reshape(-1)
    hv = np.ascontiguousarray(hi).reshape(-1)
    lv = np.ascontiguousarray(lo).reshape(-1)
    if np.iscomplexobj(hv):
        hv, lv = hv.view(np.float64), lv.view(np.float64)
    return float(lib().lfo_rel_l2(_p(yv), _p(np.ascontiguousarray(hv)),
                                  _p(np.ascontiguousarray(lv)), yv.size))


# ------------------------------------------------------------------ real transforms

def herm_ext(h: np.ndarray, n: int) -> np.ndarray:
    """Hermitian extension of the half spectrum (Problem.lean:137-138)."""
    full = np.empty(h.shape[:-1] + (n,), dtype=np.complex128)
    full[..., : n // 2 + 1] = h[..., : n // 2 + 1]
    k = np.arange(n // 2 + 1, n)
    full[..., k] = np.conj(h[..., n - k])
    return full


def generic_r2c(x: np.ndarray, nthreads: int = 1) -> np.ndarray:
    """r2c by the generic engine (Problem.lean:145-147)."""
    n = x.shape[-1]
    F = generic_dft(True, x.astype(np.complex128), nthreads)
    return np.ascontiguousarray(F[..., : n // 2 + 1])


def generic_c2r(h: np.ndarray, n: int, nthreads: int = 1) -> np.ndarray:
    """c2r by the generic engine (Problem.lean:148-150): the imaginary parts of the
    self-conjugate entries are ignored through the Hermitian extension."""
    G = generic_dft(False, herm_ext(h, n), nthreads)
    return np.ascontiguousarray(G.real)


def generic_rank2_r2c(x: np.ndarray, nthreads: int = 1) -> np.ndarray:
    """Rank-2 rdft2 forward (Problem.lean:228-233) on x of shape (..., n0, n1)."""
    h = generic_r2c(x, nthreads)                       # (..., n0, n1/2+1)
    ht = np.ascontiguousarray(np.swapaxes(h, -1, -2))  # (..., n1/2+1, n0)
    return np.ascontiguousarray(np.swapaxes(generic_dft(True, ht, nthreads), -1, -2))


def dd_r2c(x: np.ndarray, nthreads: int = 1):
    n = x.shape[-1]
    hi, lo = dd_dft(True, x.astype(np.complex128), nthreads)
    return (np.ascontiguousarray(hi[..., : n // 2 + 1]), np.ascontiguousarray(lo[..., : n // 2 + 1]))


def dd_c2r(h: np.ndarray, n: int, nthreads: int = 1):
    hi, lo = dd_dft(False, herm_ext(h, n), nthreads)
    return np.ascontiguousarray(hi.real), np.ascontiguousarray(lo.real)


def dd_rank2_r2c(x: np.ndarray, nthreads: int = 1):
    """Rank-2 r2c in double-double: dd rows, then dd columns (the column pass takes the
    rounded row result, whose rounding error is ~1e-32 relative, far below binary64)."""
    n1 = x.shape[-1]
    hi, lo = dd_dft(True, x.astype(np.complex128), nthreads)
    hi, lo = hi[..., : n1 // 2 + 1], lo[..., : n1 // 2 + 1]
    ht = np.ascontiguousarray(np.swapaxes(hi, -1, -2))
    lt = np.ascontiguousarray(np.swapaxes(lo, -1, -2))
    h2, l2 = dd_dft(True, ht, nthreads)
    h3, _ = dd_dft(True, lt, nthreads)
    # DFT is linear: DFT(hi) + DFT(lo); DFT(lo) is ~1e-16 smaller, so its own binary64
    # evaluation error is ~1e-32 relative to the result.
    return (np.ascontiguousarray(np.swapaxes(h2, -1, -2)),
            np.ascontiguousarray(np.swapaxes(l2 + h3, -1, -2)))


# ------------------------------------------------------------------ inputs

def lcg_rand(n: int, seed: int) -> np.ndarray:
    """randArr n seed (scripts/AsmTest.lean:7-13): doubles in [-1, 1) from a 64-bit LCG."""
    out = np.empty(n, dtype=np.float64)
    x = (seed * 2654435761 + 12345) & 0xFFFFFFFFFFFFFFFF
    for i in range(n):
        x = (x * 6364136223846793005 + 1442695040888963407) & 0xFFFFFFFFFFFFFFFF
        out[i] = ((x >> 11) / 9007199254740992.0) * 2.0 - 1.0
    return out


def uniform_complex(shape, seed: int = 20261016) -> np.ndarray:
    """re, im iid uniform[-0.5, 0.5) from numpy's default_rng(seed) (the benchmark
    protocol's seed)."""
    rng = np.random.default_rng(seed)
    a = rng.random(tuple(shape) + (2,)) - 0.5
    return a.view(np.complex128).reshape(shape)


# ---- real-to-real kinds (Core/Problem.lean:64-112, 151-163) -----------------------------------

R2R_KINDS = ["r2hc", "hc2r", "dht", "redft00", "redft01", "redft10", "redft11",
             "rodft00", "rodft01", "rodft10", "rodft11"]   # libbench2 numbering (FFI.lean:29-31)


def r2r_embed_size(kind: str, n: int) -> int:
    """embedSize (Problem.lean:66-72)."""
    if kind in ("r2hc", "hc2r", "dht"):
        return n
    if kind == "redft00":
        return 2 * (n - 1)
    if kind == "rodft00":
        return 2 * (n + 1)
    if kind in ("redft10", "redft01", "rodft10", "rodft01"):
        return 4 * n
    return 8 * n


def r2r_embed(kind: str, x: np.ndarray) -> np.ndarray:
    """The complex sequence whose DFT holds the transform (embed, Problem.lean:76-98; for
    hc2r the Hermitian extension of the halfcomplex input, :153-158); last axis."""
    n = x.shape[-1]
    M = r2r_embed_size(kind, n)
    z = np.zeros(x.shape[:-1] + (M,), dtype=np.complex128)
    i = np.arange(M)
    X = lambda j: x[..., j]
    if kind in ("r2hc", "dht"):
        z.real[...] = x
    elif kind == "hc2r":
        k = np.where(i <= n // 2, i, n - i)
        ik = np.where((0 < k) & (k < n - k), X(np.where((0 < k) & (k < n - k), n - k, 0)), 0.0)
        z.real[...] = X(k)
        z.imag[...] = np.where(i <= n // 2, ik, -ik)
    elif kind == "redft00":
        z.real[...] = X(np.where(i < n, i, M - i))
    elif kind == "rodft00":
        lo = (1 <= i) & (i <= n)
        hi = (n + 2 <= i) & (i < M)
        v = np.where(lo, X(np.clip(i - 1, 0, n - 1)), 0.0)
        z.real[...] = np.where(hi, -X(np.clip(M - i - 1, 0, n - 1)), v)
    elif kind in ("redft10", "rodft10"):
        sgn = 1.0 if kind == "redft10" else -1.0
        odd = (i % 2) == 1
        a = X(np.clip(i // 2, 0, n - 1))
        b = sgn * X(np.clip((M - i) // 2, 0, n - 1))
        z.real[...] = np.where(odd, np.where(i < 2 * n, a, b), 0.0)
    elif kind in ("redft11", "rodft11"):
        sgn = 1.0 if kind == "redft11" else -1.0
        odd = (i % 2) == 1
        a = X(np.clip(i // 2, 0, n - 1))
        b = sgn * X(np.clip((M - i) // 2, 0, n - 1))
        z.real[...] = np.where(odd & (i < 2 * n), a, np.where(odd & (6 * n < i), b, 0.0))
    elif kind == "redft01":
        z.real[...] = np.where(i < n, X(np.clip(i, 0, n - 1)),
                               np.where((3 * n < i) & (i < M), X(np.clip(M - i, 0, n - 1)), 0.0))
    elif kind == "rodft01":
        lo = (1 <= i) & (i <= n)
        hi = (3 * n < i) & (i < M)
        z.real[...] = np.where(lo, X(np.clip(i - 1, 0, n - 1)),
                               np.where(hi, -X(np.clip(M - i - 1, 0, n - 1)), 0.0))
    else:
        raise ValueError(kind)
    return z


def r2r_extract(kind: str, n: int, F: np.ndarray) -> np.ndarray:
    """extract (Problem.lean:101-110) on the last axis of the DFT F of the embedding."""
    j = np.arange(n)
    if kind == "r2hc":
        return np.where(j <= n // 2, F.real[..., np.minimum(j, n - 1)],
                        F.imag[..., (n - j) % max(n, 1)])
    if kind in ("hc2r", "redft00", "redft10"):
        return np.ascontiguousarray(F.real[..., :n])
    if kind == "dht":
        return np.ascontiguousarray(F.real[..., :n] - F.imag[..., :n])
    if kind in ("redft01", "redft11"):
        return np.ascontiguousarray(F.real[..., 2 * j + 1])
    if kind in ("rodft00", "rodft10"):
        return np.ascontiguousarray(-F.imag[..., j + 1])
    return np.ascontiguousarray(-F.imag[..., 2 * j + 1])


def _r2r_dft_fwd(kind: str) -> bool:
    return kind != "hc2r"


def generic_r2r(kind: str, x: np.ndarray, nthreads: int = 1) -> np.ndarray:
    """The generic engine's r2r line (LineOp.apply, Problem.lean:151-163)."""
    z = r2r_embed(kind, x)
    if z.shape[-1] == 1:
        return r2r_extract(kind, x.shape[-1], z)
    return r2r_extract(kind, x.shape[-1], generic_dft(_r2r_dft_fwd(kind), z, nthreads))


def fast_r2r(kind: str, x: np.ndarray, radices, nthreads: int = 1) -> np.ndarray:
    """The same embedding around refTransform of the embedding size with `radices`."""
    z = r2r_embed(kind, x)
    M = z.shape[-1]
    if M == 1:
        return r2r_extract(kind, x.shape[-1], z)
    return r2r_extract(kind, x.shape[-1], ref_transform(_r2r_dft_fwd(kind), M, radices, z, nthreads))


def dd_r2r(kind: str, x: np.ndarray, nthreads: int = 1):
    """Extended precision: (hi, lo) of the extraction from the double-double DFT (the
    extraction is exact except DHT's re - im, taken on both parts)."""
    z = r2r_embed(kind, x)
    n = x.shape[-1]
    if z.shape[-1] == 1:
        return r2r_extract(kind, n, z), np.zeros(x.shape)
    hi, lo = dd_dft(_r2r_dft_fwd(kind), z, nthreads)
    if kind == "dht":
        # re - im with its rounding error kept (TwoSum), so (hi, lo) stays extended
        a, b = hi.real[..., :n], -hi.imag[..., :n]
        s = a + b
        bb = s - a
        err = (a - (s - bb)) + (b - bb)
        return np.ascontiguousarray(s), np.ascontiguousarray(err + (lo.real[..., :n] - lo.imag[..., :n]))
    return r2r_extract(kind, n, hi), r2r_extract(kind, n, lo)

