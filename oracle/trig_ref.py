"""ORACLE (test infrastructure only): exact-integer twiddles and double-double twiddles.

This is the checker's own restatement of lean-fftw `LeanFFTW/Core/Trig.lean:25-134`,
written independently of the product's copies (`lfg/codegen/trig.py`, `csrc/trig.cpp`) so
that the three can be checked against each other and against the reference's pinned
known answers (`results/repro-2026-11-04/kernel-constants.txt`, 237 binary64 bit patterns).

It also provides cos/sin(2*pi*m/n) as double-double pairs (hi + lo, about 106 bits) for the
extended-precision DFT oracle, from the same 160-bit fixed-point series.

Only tests, the smoke check and the CPU-baseline leg of the benchmark may import this.
"""
from __future__ import annotations

import math
import struct
from functools import lru_cache

_P = 160
_PI = 3141592653589793238462643383279502884197169399375105820974944 * (1 << _P) // 10 ** 60


def _series(theta: int):
    """(cos, sin) * 2^160 of theta * 2^-160, theta in [0, pi/4] (Trig.lean:43-62)."""
    t2 = theta * theta >> _P
    one = 1 << _P
    pos_c, neg_c, pos_s, neg_s = one, 0, theta, 0
    tc, ts = one, theta
    for j in range(1, 40):
        tc = (tc * t2 >> _P) // ((2 * j - 1) * 2 * j)
        ts = (ts * t2 >> _P) // (2 * j * (2 * j + 1))
        if j & 1:
            neg_c, neg_s = neg_c + tc, neg_s + ts
        else:
            pos_c, pos_s = pos_c + tc, pos_s + ts
    return pos_c - neg_c, pos_s - neg_s


def _round_fixed(v: int) -> float:
    """v * 2^-160 -> nearest binary64, ties to even (Trig.lean:67-86), via exact integer
    division, which Python rounds correctly to nearest-even."""
    return v / (1 << _P)


def _small_fixed(n: int, num: int):
    return _series(2 * _PI * num // (8 * n))


def _octant(k: int, n: int, small):
    """Exact octant reduction (Trig.lean:104-122) on any value type with negation."""
    k %= n
    octant, rem = divmod(8 * k, n)
    c, s = small(rem) if octant % 2 == 0 else small(n - rem)
    nz = lambda x: -x if x != 0 else x
    return [(c, s), (s, c), (nz(s), c), (nz(c), s), (nz(c), nz(s)), (nz(s), nz(c)),
            (s, nz(c)), (c, nz(s))][octant]


@lru_cache(maxsize=None)
def table(n: int):
    """[(cos, sin)(2*pi*m/n) for m < n] as binary64 (Trig.lean:131-134)."""
    g = math.gcd(8, n)
    memo = [tuple(_round_fixed(v) for v in _small_fixed(n, g * i)) for i in range(n // g + 1)]
    out = []
    for m in range(n):
        c, s = _octant(m, n, lambda num: memo[num // g])
        out.append((c + 0.0, s + 0.0))  # never -0.0
    return out


def cos_sin(k: int, n: int):
    return _octant(k, n, lambda num: tuple(_round_fixed(v) for v in _small_fixed(n, num)))


def tan2pi(num: int, den: int) -> float:
    c, s = _series(2 * _PI * num // den)
    return _round_fixed(s * (1 << _P) // c)


def pass_twiddles(tab, fwd: bool, N: int, R: int, ns: int):
    """Twiddles of one Stockham pass (FastPlan.lean:163-173): for r = 1..R-1 the ns real
    parts then the ns imaginary parts of tab[r*k*N/(ns*R)]; imaginary parts negated
    (never to -0.0) for forward transforms."""
    step = N // (ns * R)
    out = []
    for r in range(1, R):
        row = [tab[r * k * step] for k in range(ns)]
        out += [c for c, _ in row]
        out += [(-s if s != 0.0 else 0.0) if fwd else s for _, s in row]
    return out


def dd_table(n: int):
    """[(cos_hi, cos_lo, sin_hi, sin_lo)(2*pi*m/n)] as double-double pairs."""
    g = math.gcd(8, n)

    def to_dd(v: int):
        hi = _round_fixed(abs(v))
        p, q = hi.as_integer_ratio()          # exact: q is a power of two <= 2^160
        rest = abs(v) - p * (1 << _P) // q
        lo = rest / (1 << _P)
        return (hi, lo) if v >= 0 else (-hi, -lo)

    memo = [_small_fixed(n, g * i) for i in range(n // g + 1)]
    out = []
    for m in range(n):
        c, s = _octant(m, n, lambda num: memo[num // g])
        ch, cl = to_dd(c)
        sh, sl = to_dd(s)
        out.append((ch, cl, sh, sl))
    return out


def bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]
