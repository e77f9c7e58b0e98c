"""Twiddle factors from exact integer arithmetic (build-time copy for codelet constants).

Restates lean-fftw's `LeanFFTW/Core/Trig.lean:25-134`: cos/sin(2*pi*k/n) are summed as
Taylor series in 160-bit fixed point after an exact octant reduction of the rational
angle k/n, then rounded to the nearest binary64 (ties to even).  No libm call is made,
so every constant is a pure function of (k, n).

The run-time twiddle tables of a plan are produced by the C++ restatement in
`csrc/trig.cpp`; this module gives the same values to the code generator, which bakes the
butterfly constants (`Cst`) into the generated CUDA and C sources as hexadecimal literals.
"""
from __future__ import annotations

import functools
import math
import struct

PREC_BITS = 160                                    # Trig.lean:25
PI_DIGITS = 3141592653589793238462643383279502884197169399375105820974944  # Trig.lean:28
PI_SCALE = 10 ** 60                                # Trig.lean:30
PI_FIXED = PI_DIGITS * 2 ** PREC_BITS // PI_SCALE  # Trig.lean:33
ONE = 1 << PREC_BITS


def fmul(a: int, b: int) -> int:
    """floor(a*b / 2^160) (Trig.lean:36)."""
    return (a * b) >> PREC_BITS


def angle_fixed(num: int, den: int) -> int:
    """theta * 2^160 for theta = 2*pi*num/den (Trig.lean:39)."""
    return 2 * PI_FIXED * num // den


def cos_sin_fixed(theta: int) -> tuple[int, int]:
    """Taylor series of cos and sin at fixed point, 0 <= theta <= pi/4 (Trig.lean:43-62).

    Positive and negative terms are accumulated separately and subtracted once, exactly
    as the reference does, so the truncation pattern is identical."""
    th2 = fmul(theta, theta)
    c_pos, c_neg, s_pos, s_neg = ONE, 0, theta, 0
    tc, ts = ONE, theta
    for j in range(1, 40):
        tc = fmul(tc, th2) // ((2 * j - 1) * (2 * j))
        ts = fmul(ts, th2) // ((2 * j) * (2 * j + 1))
        if j % 2 == 1:
            c_neg += tc
            s_neg += ts
        else:
            c_pos += tc
            s_pos += ts
    return c_pos - c_neg, s_pos - s_neg


def fixed_to_bits(v: int) -> int:
    """Round v * 2^-160 (v >= 0) to binary64, ties to even; return the bit pattern
    (Trig.lean:67-86)."""
    if v == 0:
        return 0
    lg = v.bit_length() - 1
    if lg <= 52:
        q = v << (52 - lg)
    else:
        sh = lg - 52
        q = v >> sh
        r = v - (q << sh)
        half = 1 << (sh - 1)
        if r > half or (r == half and q % 2 == 1):
            q += 1
    if q == 1 << 53:
        q, lg = 1 << 52, lg + 1
    e = lg - PREC_BITS + 1023
    return (e << 52) | (q - (1 << 52))


def bits_to_float(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def float_to_bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def fixed_to_float(v: int) -> float:
    return bits_to_float(fixed_to_bits(v))


def tan2pi(num: int, den: int) -> float:
    """tan(2*pi*num/den), num/den in [0, 1/8]: quotient of the fixed-point series, rounded
    once (Trig.lean:90-92)."""
    c, s = cos_sin_fixed(angle_fixed(num, den))
    return fixed_to_float(s * 2 ** PREC_BITS // c)


def neg_z(x: float) -> float:
    """Negation that never produces -0.0 (Trig.lean:95)."""
    return 0.0 if x == 0.0 else -x


@functools.lru_cache(maxsize=None)
def small_at(n: int, num: int) -> tuple[float, float]:
    """(cos, sin) of 2*pi*num/(8n), 0 <= num <= n (Trig.lean:98-100)."""
    c, s = cos_sin_fixed(angle_fixed(num, 8 * n))
    return fixed_to_float(c), fixed_to_float(s)


def cos_sin_2pi_with(small, k: int, n: int) -> tuple[float, float]:
    """Exact octant reduction (Trig.lean:104-122)."""
    if n == 0:
        return 1.0, 0.0
    k %= n
    octant, rem = divmod(8 * k, n)
    c, s = small(rem) if octant % 2 == 0 else small(n - rem)
    if octant == 0:
        return c, s
    if octant == 1:
        return s, c
    if octant == 2:
        return neg_z(s), c
    if octant == 3:
        return neg_z(c), s
    if octant == 4:
        return neg_z(c), neg_z(s)
    if octant == 5:
        return neg_z(s), neg_z(c)
    if octant == 6:
        return s, neg_z(c)
    return c, neg_z(s)


def cos_sin_2pi(k: int, n: int) -> tuple[float, float]:
    """(cos(2*pi*k/n), sin(2*pi*k/n)) as binary64 (Trig.lean:126)."""
    return cos_sin_2pi_with(lambda num: small_at(n, num), k, n)


def cos_sin_2pi_table(n: int) -> list[tuple[float, float]]:
    """m -> cos_sin_2pi(m, n) for m < n, evaluating only n/gcd(8,n)+1 reduced angles
    (Trig.lean:131-134)."""
    g = math.gcd(8, n)
    memo = [small_at(n, g * i) for i in range(n // g + 1)]
    return [cos_sin_2pi_with(lambda num: memo[num // g], m, n) for m in range(n)]
