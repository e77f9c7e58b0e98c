"""Symbolic complex arithmetic and the generic Cooley-Tukey algorithm run on expressions.

Restates lean-fftw's `LeanFFTW/Gen/Sym.lean` (symbolic complex values `SC`, canonicalised
twiddle rotations, Sym.lean:205-286) and the parts of `LeanFFTW/Core/Alg.lean` that the
generator instantiates with symbolic values: `mkPlan`/`exec` (Alg.lean:236-254),
`sumRange` (Alg.lean:231-232) and `primeFactors` (Alg.lean:262-272).

A symbolic complex value is either ("tw", fwd, n, k), the twiddle exp(-+2*pi*i*k/n)
(minus when fwd), or ("val", re, im) with real expressions re, im.
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple

from .sexpr import (E, ZERO, cst, fma, fms, mk_add, mk_fma_c, mk_fms_c, mk_fnma_c, mk_mul_c,
                    mk_neg, mk_sub, mul)

SC = Tuple


def val(re: E, im: E) -> SC:
    return ("val", re, im)


def tw(fwd: bool, n: int, k: int) -> SC:
    return ("tw", fwd, n, k)


VZERO = val(ZERO, ZERO)


def mul_ipow(q: int, re: E, im: E) -> Tuple[E, E]:
    """Multiply by i^q (Sym.lean:220-225)."""
    q %= 4
    if q == 0:
        return re, im
    if q == 1:
        return mk_neg(im), re
    if q == 2:
        return mk_neg(re), mk_neg(im)
    return im, mk_neg(re)


def rot_q(k: int, n: int, a: E, b: E) -> Tuple[E, E]:
    """Multiply a+ib by exp(i*theta), theta = 2*pi*k/n in [0, pi/2) (Sym.lean:228-243).

    Quarter turn: free.  pi/4: two multiplications by sqrt(1/2).  Otherwise the
    tan-factored form c*(a - t*b), c*(b + t*a) with the octant chosen so 0 < t < 1."""
    if k == 0:
        return a, b
    if 8 * k == n:
        return (mk_mul_c(("sqrthalf",), mk_sub(a, b)),
                mk_mul_c(("sqrthalf",), mk_add(a, b)))
    if 8 * k < n:
        return (mk_mul_c(("cos", k, n), mk_fnma_c(("tan", k, n), b, a)),
                mk_mul_c(("cos", k, n), mk_fma_c(("tan", k, n), a, b)))
    k2 = n - 4 * k
    return (mk_mul_c(("cos", k2, 4 * n), mk_fms_c(("tan", k2, 4 * n), a, b)),
            mk_mul_c(("cos", k2, 4 * n), mk_fma_c(("tan", k2, 4 * n), b, a)))


def rot(fwd: bool, n: int, k: int, a: E, b: E) -> Tuple[E, E]:
    """Multiply a+ib by exp(-+2*pi*i*k/n) (Sym.lean:246-254)."""
    k %= n
    if fwd:
        k = (n - k) % n
    q = 4 * k // n
    k1 = 4 * k - q * n
    a2, b2 = rot_q(k1, 4 * n, a, b)
    return mul_ipow(q, a2, b2)


def parts(x: SC) -> Tuple[E, E]:
    """Real and imaginary parts (Sym.lean:257-261)."""
    if x[0] == "val":
        return x[1], x[2]
    _, fwd, n, k = x
    return rot(fwd, n, k, cst(("cos", 0, 1)), ZERO)


def sc_add(x: SC, y: SC) -> SC:
    a, b = parts(x)
    c, d = parts(y)
    return val(mk_add(a, c), mk_add(b, d))


def sc_sub(x: SC, y: SC) -> SC:
    a, b = parts(x)
    c, d = parts(y)
    return val(mk_sub(a, c), mk_sub(b, d))


def mul_gen(x: SC, y: SC) -> SC:
    """General complex product, re = fms(a, c, b*d), im = fma(a, d, b*c) (Sym.lean:274-277)."""
    a, b = parts(x)
    c, d = parts(y)
    return val(fms(a, c, mul(b, d)), fma(a, d, mul(b, c)))


def sc_mul(x: SC, y: SC) -> SC:
    """Sym.lean:279-286."""
    if x[0] == "tw" and y[0] == "val":
        return val(*rot(x[1], x[2], x[3], y[1], y[2]))
    if x[0] == "val" and y[0] == "tw":
        return val(*rot(y[1], y[2], y[3], x[1], x[2]))
    if x[0] == "tw" and y[0] == "tw":
        a, b = parts(y)
        return val(*rot(x[1], x[2], x[3], a, b))
    return mul_gen(x, y)


def get(v: Sequence[SC], i: int) -> SC:
    """symOps.get: out-of-range reads give zero (Sym.lean:298)."""
    return v[i] if 0 <= i < len(v) else VZERO


# ---------------------------------------------------------------- generic algorithm (Alg.lean)

def prime_factors(n: int) -> List[int]:
    """Prime factors in nondecreasing order, [] for n <= 1 (Alg.lean:262-272)."""
    out: List[int] = []
    d = 2
    while n > 1:
        if d * d > n:
            out.append(n)
            break
        if n % d == 0:
            out.append(d)
            n //= d
        else:
            d += 1
    return out


def sum_range(n: int, f: Callable[[int], SC]) -> SC:
    """Left-to-right sum from zero (Alg.lean:231-232)."""
    acc = VZERO
    for j in range(n):
        acc = sc_add(acc, f(j))
    return acc


# A plan is ("direct", n, fwd) or ("ct", r, n, fwd, sub); the twiddle vectors of the
# reference's `Plan` are the symbolic twiddles tw(fwd, n, i), so only (fwd, n) is stored.

def mk_plan(fwd: bool, fs: List[int]):
    """Alg.lean:236-242."""
    if not fs:
        return ("direct", 1, fwd)
    if len(fs) == 1:
        return ("direct", fs[0], fwd)
    sub = mk_plan(fwd, fs[1:])
    n = fs[0]
    for f in fs[1:]:
        n *= f
    return ("ct", fs[0], n, fwd, sub)


def plan_size(p) -> int:
    return p[1] if p[0] == "direct" else p[2]


def exec_plan(p, x: Callable[[int], SC]) -> List[SC]:
    """Alg.lean:245-254 over symbolic values."""
    if p[0] == "direct":
        _, n, fwd = p
        xs = [x(j) for j in range(n)]
        return [sum_range(n, lambda j, k=k: sc_mul(tw(fwd, n, j * k % n), xs[j]))
                for k in range(n)]
    _, r, n, fwd, sub = p
    m = plan_size(sub)
    ys = [exec_plan(sub, lambda j2, j1=j1: x(j1 + r * j2)) for j1 in range(r)]
    return [sum_range(r, lambda j1, k=k: sc_mul(tw(fwd, n, j1 * k % n), get(ys[j1], k % m)))
            for k in range(n)]
